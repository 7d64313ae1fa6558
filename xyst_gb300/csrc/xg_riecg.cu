// RieCG on one GB300: superedge-equivalent node-gather gradient and residual
// kernels, fused low-storage RK update, nodal BCs and CFL reduction.
//
// Reference path (all paths relative to the reference project root):
//   riemann::grad   src/Physics/Riemann.cpp:229-367
//   riemann::rhs    src/Physics/Riemann.cpp:909-946 (advdom :652-766 with
//                   rusanov :369-478 / hllc :480-650 and muscl :34-143,
//                   advbnd :768-878)
//   RieCG::solve    src/Inciter/RieCG.cpp:992-1057 (rkcoef :41)
//   RieCG::BC       src/Inciter/RieCG.cpp:764-785 -> src/Physics/BC.cpp
//   RieCG::dt       src/Inciter/RieCG.cpp:787-852
//   riemann::src    src/Physics/Riemann.cpp:880-907 (manufactured sources)
//
// Data layout in HBM (n nodes):
//   U, Un     double SoA [5][n]  conserved state and stage-0 copy
//   W[0..1]   F [n][8]           (rho, u, v, w, e, x, y, z) records, ping-pong
//   G         F [n][16]          15 volume-divided gradients + pad (FP32: the
//                                component-paired order of gslot, for the
//                                packed FP32x2 pipe)
//   vol       double [n]
//   adjacency SELL-32: slice s of 32 consecutive nodes holds width[s] entries
//             per node at off[s] + k*32 + lane, each one packed record: the
//             neighbour (int32, ~q when the node is the second end of the
//             canonical edge, PAD for padding) and the canonical edge
//             integral D (16 bytes in FP32 mode, 32 in FP64 mode).
//   ivol, cbrtv  1/vol (double) and cbrt(vol) (float) for the FP32 epilogue
// In FP64 mode every edge flux is evaluated with the canonical orientation
// (left = first end), so the sum is the reference's up to summation order;
// FP32 mode evaluates it in the owner's orientation.  Each node owns its
// writes: no atomics except the scalar CFL minimum.

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <string>
#include <vector>

#include "xg_internal.hpp"
#include "xg_source.cuh"

namespace xg {

namespace {

constexpr int kSlice = 32;
constexpr int32_t kPad = INT32_MIN;
constexpr int kBlock = 256;

struct Scalars {
  double dt;                  // current step size
  unsigned long long dtmin;   // running minimum of the per-node CFL dt (bits)
  int32_t blowup;             // set when a dt fell below eps
  int32_t pad;
  long long step;             // steps taken in the current run (dt history index)
  double t;                   // time at the start of the current step
  double tnext;               // time at the start of the next step
};

// A manufactured source (enum xg_source) and its parameters alpha,
// beta[3], kappa, r0, p0, ce.

}  // namespace

struct RieCGDev {
  Arena arena;      // mesh-sized arrays
  Arena bcarena;    // boundary condition program
  Arena scratch;    // drop-in staging buffers
  int64_t n = 0, nslice = 0, nent = 0, nbn = 0, nbt = 0, nbent = 0;
  xg_riecg_params prm{};
  bool fp32 = false;
  // node arrays
  double *U = nullptr, *Un = nullptr, *vol = nullptr;
  int32_t* bidx = nullptr;  // per node: index into boundary lists or -1
  void* W[2] = {nullptr, nullptr};
  void* G = nullptr;
  // adjacency
  int32_t *soff = nullptr, *swidth = nullptr;
  void* ent = nullptr;  // int4 (FP32 mode) or Ent64 (FP64 mode) per entry
  // half-edge lists of the residual: the edges a node owns (list 1, with
  // the position of each edge in its other end's list) and the edges its
  // neighbours own (list 2, whose slots receive those owners' fluxes)
  int64_t nent1 = 0, nent2 = 0;
  int32_t *soff1 = nullptr, *sw1 = nullptr, *soff2 = nullptr, *sw2 = nullptr, *pos1 = nullptr;
  void* ent1 = nullptr;
  void* fbuf = nullptr;  // F: [nent2][4] components 0-3, then [nent2] component 4
  void* Rp = nullptr;    // F [5][n] first-end partial residuals
  double* ivol = nullptr;
  float* cbrtv = nullptr;
  // boundary triangles, per boundary node lists of (tri << 2 | position)
  int32_t *bptr = nullptr, *bnode = nullptr;
  int4* bent4 = nullptr;  // per boundary entry: the triangle's 3 nodes, pos | sym flags << 2
  void* Rb = nullptr;  // F [5][nbn] domain residual of the boundary nodes
  int32_t* bcof = nullptr;  // per boundary node: its BC program entry or -1
  // BC program: one thread per BC node
  int64_t nbc = 0;
  int32_t *bcnode = nullptr, *bcdir = nullptr, *bcsymp = nullptr, *bcfar = nullptr,
          *bcpre = nullptr, *dirmask = nullptr;
  double *symn = nullptr, *dirval = nullptr, *farn = nullptr, *preval = nullptr;
  double* dirxyz = nullptr;       // [ndir][3] Dirichlet node coordinates
  std::vector<double> xyz_host;  // [3][n] node coordinates (for dirxyz)
  double far5[5] = {1, 0, 0, 0, 1};
  // scalars and run bookkeeping
  Scalars* scal = nullptr;
  double* dthist = nullptr;
  int64_t dthist_cap = 0;
  int cur = 0;
  double t = 0.0;
  bool dt_valid = false;
  // two whole time steps captured once and replayed (launch overhead)
  cudaGraphExec_t graph = nullptr;
  // and one step from either primitive-buffer parity (single-step runs)
  cudaGraphExec_t graph1[2] = {nullptr, nullptr};
  // edge-coloured residual (xg_riecg_rhs_coloured), built on first use:
  // colour c holds edges coff[c] .. coff[c+1] - 1 as (owner, other end) and
  // the edge integral in the owner's orientation; cR: F [n][8] records
  Arena colarena;
  std::vector<int64_t> coff;
  int2* cpq = nullptr;
  float4* cd = nullptr;
  float* cR = nullptr;
  // manufactured source: problem, parameters, and s V per node at the time
  // of the current step (F [5][n], its own arena)
  SrcPrm src{};
  Arena srcarena;
  void* Sv = nullptr;
  // staging for the drop-in entry points
  double* stage_buf = nullptr;
  void* stage_W = nullptr;
  void* stage_G = nullptr;
  // profiling
  bool prof = false;
  struct KT {
    const char* name;
    double ms;
    int64_t launches;
  };
  std::vector<KT> ktimes;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
};

// Captured time-loop graphs are dropped whenever what they captured changes
// (BCs, the source, the dt history buffer).
void drop_graphs(RieCGDev* d) {
  if (d->graph) cudaGraphExecDestroy(d->graph);
  d->graph = nullptr;
  for (auto& g : d->graph1) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
}

void destroy_riecg(RieCGDev* d) {
  if (!d) return;
  drop_graphs(d);
  if (d->dthist) cudaFree(d->dthist);
  for (auto& p : d->pending) {
    cudaEventDestroy(p.second.first);
    cudaEventDestroy(p.second.second);
  }
  delete d;
}

size_t bytes_riecg(const RieCGDev* d) {
  return d ? d->arena.bytes() + d->bcarena.bytes() + d->scratch.bytes() + d->colarena.bytes() +
                 d->srcarena.bytes()
           : 0;
}

// The device address of a caller's pinned (page-locked) host buffer, which
// kernels may read and write over the host link, or nullptr for any other
// memory (pageable host memory, 8-byte misaligned pointers).
void* pinned_view(const void* p) {
  if (reinterpret_cast<uintptr_t>(p) % alignof(double) != 0) return nullptr;
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    (void)cudaGetLastError();  // clear the query's error: the buffer is not one of CUDA's
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// ---------------------------------------------------------------------------
// device code

namespace {

// Record loads and stores as single 256-bit accesses (one 32-byte sector per
// lane: half the L1 wavefronts of two 128-bit accesses on scattered rows).
// Loads use the read-only path: every record read this way is either not
// written by the kernel or read before the same thread overwrites it.
__device__ __forceinline__ void load8(const float* p, float o[8]) {
  asm volatile("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=f"(o[0]), "=f"(o[1]), "=f"(o[2]), "=f"(o[3]), "=f"(o[4]), "=f"(o[5]),
                 "=f"(o[6]), "=f"(o[7])
               : "l"(p));
}
__device__ __forceinline__ void load8(const double* p, double o[8]) {
  asm volatile("ld.global.nc.v4.f64 {%0,%1,%2,%3}, [%4];"
               : "=d"(o[0]), "=d"(o[1]), "=d"(o[2]), "=d"(o[3])
               : "l"(p));
  asm volatile("ld.global.nc.v4.f64 {%0,%1,%2,%3}, [%4];"
               : "=d"(o[4]), "=d"(o[5]), "=d"(o[6]), "=d"(o[7])
               : "l"(p + 4));
}
__device__ __forceinline__ void store8(float* p, const float o[8]) {
  asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(p), "f"(o[0]), "f"(o[1]),
               "f"(o[2]), "f"(o[3]), "f"(o[4]), "f"(o[5]), "f"(o[6]), "f"(o[7])
               : "memory");
}
__device__ __forceinline__ void store8(double* p, const double o[8]) {
  asm volatile("st.global.v4.f64 [%0], {%1,%2,%3,%4};" ::"l"(p), "d"(o[0]), "d"(o[1]), "d"(o[2]),
               "d"(o[3])
               : "memory");
  asm volatile("st.global.v4.f64 [%0], {%1,%2,%3,%4};" ::"l"(p + 4), "d"(o[4]), "d"(o[5]),
               "d"(o[6]), "d"(o[7])
               : "memory");
}
template <class F>
__device__ __forceinline__ void load16(const F* p, F o[16]) {
  load8(p, o);
  load8(p + 8, o + 8);
}
template <class F>
__device__ __forceinline__ void store16(F* p, const F o[16]) {
  store8(p, o);
  store8(p + 8, o + 8);
}

// Five primitives of a W record (the coordinates in slots 5-7 are not read).
__device__ __forceinline__ void load5(const float* p, float o[5]) {
  const float4 a = __ldg(reinterpret_cast<const float4*>(p));
  o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
  o[4] = __ldg(p + 4);
}
__device__ __forceinline__ void load5(const double* p, double o[5]) {
  const double2* q = reinterpret_cast<const double2*>(p);
  const double2 a = __ldg(q), b = __ldg(q + 1);
  o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
  o[4] = __ldg(p + 4);
}

// Asynchronous global -> shared copies (cp.async, 16 bytes, L2 only) with
// their commit/wait group fences.  The adjacency entries a thread will need
// are streamed into a per-thread ring in shared memory several iterations
// ahead, so the coalesced entry stream stays in flight while the thread waits
// on its gathers.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Primitive variables from conserved ones (primitive(),
// src/Physics/Riemann.cpp:211-227), evaluated in double.
__device__ __forceinline__ void prim5(const double u[5], double w[5]) {
  w[0] = u[0];
  w[1] = u[1] / w[0];
  w[2] = u[2] / w[0];
  w[3] = u[3] / w[0];
  w[4] = u[4] / w[0] - 0.5 * (w[1] * w[1] + w[2] * w[2] + w[3] * w[3]);
}

// The five primitives of a W record from a node's FP64 state: FP64 mode
// the reference's expressions (primitive(), src/Physics/Riemann.cpp:211-227);
// FP32 mode FP32 arithmetic with one reciprocal (the records are FP32).
template <class F>
__device__ __forceinline__ void prim_record(const double u[5], F o[5]) {
  if constexpr (sizeof(F) == 8) {
    double pw[5];
    prim5(u, pw);
#pragma unroll
    for (int c = 0; c < 5; ++c) o[c] = pw[c];
  } else {
    const float r = float(u[0]);
    const float ir = __frcp_rn(r);
    const float uu = float(u[1]) * ir, vv = float(u[2]) * ir, ww = float(u[3]) * ir;
    o[0] = r;
    o[1] = uu;
    o[2] = vv;
    o[3] = ww;
    o[4] = float(u[4]) * ir - 0.5f * (uu * uu + vv * vv + ww * ww);
  }
}

// Per-node CFL time step (src/Inciter/RieCG.cpp:827-838), before the CFL factor.
__device__ __forceinline__ double node_dt(const double u[5], double vol, double g) {
  double r = u[0];
  double uu = u[1] / r, vv = u[2] / r, ww = u[3] / r;
  double pr = (u[4] - 0.5 * r * (uu * uu + vv * vv + ww * ww)) * (g - 1.0);
  double c = sqrt(g * fmax(pr, 0.0) / r);
  double L = cbrt(vol);
  double vel = sqrt(uu * uu + vv * vv + ww * ww);
  return L / fmax(vel + c, 1.0e-8);
}

// Block-wide minimum of positive doubles folded into *dst with one atomic per
// block.  Positive IEEE doubles order like their bit patterns.
__device__ __forceinline__ void block_min_atomic(double v, unsigned long long* dst) {
  __shared__ double red[32];
  unsigned long long bits = __double_as_longlong(v);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long other = __shfl_xor_sync(0xffffffffu, bits, o);
    bits = other < bits ? other : bits;
  }
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = __longlong_as_double(bits);
  __syncthreads();
  if (wid == 0) {
    int nw = (blockDim.x + 31) >> 5;
    double x = lane < nw ? red[lane] : DBL_MAX;
    unsigned long long b = __double_as_longlong(x);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long other = __shfl_xor_sync(0xffffffffu, b, o);
      b = other < b ? other : b;
    }
    if (lane == 0) atomicMin(dst, b);
  }
}

// MUSCL reconstruction of the five flow variables on edge L->R
// (muscl(), src/Physics/Riemann.cpp:34-143) from the edge-end primitives and
// the projections g1 = G_L.(x_R - x_L), g2 = G_R.(x_R - x_L).  The van Leer
// limiter of a pair, phi(r) = (|r| + r)/(|r| + 1) at r = a/b and at 1/r, is
// the same pair of numbers as 2|a|/(|a|+|b|), 2|b|/(|a|+|b|) for a b > 0 and
// 0, 0 otherwise.  Both precisions reduce the limited reconstruction
// algebraically (below): FP64 exactly, with one division for all ten
// quotients instead of the reference's four per side (the difference is
// rounding, a few 1e-16 of the increment); FP32 to the harmonic slope.
template <class F>
__device__ __forceinline__ void muscl(const F wl[5], const F wr[5], const F g1[5],
                                      const F g2[5], F l[5], F r[5]) {
  const F eps = F(1.0e-9);
  const F k = F(1.0) / F(3.0);
  F d1[5], d3[5];
  if constexpr (sizeof(F) == 8) {
    // FP64: with a = d2 + eps, b = d1 + eps of one sign s (a b > 0), the
    // reconstruction wl + ((1-k) d1 phiL + (1+k) d2 phiLi) / 4 is, exactly,
    // wl + (a b - s (eps/2) ((1-k)|a| + (1+k)|b|)) / (a + b), and the right
    // state likewise with e = d3 + eps (the reference's form up to rounding,
    // a few 1e-16 of the increment).  The ten quotients come from one
    // division (batch inversion: prefix products, one reciprocal,
    // back-substitution); an unused denominator (a b <= 0) counts as 1, and
    // a product outside [1e-290, 1e290] falls back to ten divisions.
    const F h = F(0.5) * eps;
    F d2[5], num[10], den[10], pre[10];
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      d2[c] = wr[c] - wl[c];
      d1[c] = F(2.0) * g1[c] - d2[c];
      d3[c] = F(2.0) * g2[c] - d2[c];
      const F a = d2[c] + eps, b = d1[c] + eps, e3 = d3[c] + eps;
      const F pl = a * b, pr = a * e3;
      const F sh = copysign(h, a);
      const F ka = (F(1.0) - k) * fabs(a);
      num[2 * c] = pl > F(0) ? pl - sh * (ka + (F(1.0) + k) * fabs(b)) : F(0);
      num[2 * c + 1] = pr > F(0) ? pr - sh * (ka + (F(1.0) + k) * fabs(e3)) : F(0);
      den[2 * c] = pl > F(0) ? a + b : F(1);
      den[2 * c + 1] = pr > F(0) ? a + e3 : F(1);
    }
    pre[0] = den[0];
#pragma unroll
    for (int m = 1; m < 10; ++m) pre[m] = pre[m - 1] * den[m];
    F q[10];
    const F ap = fabs(pre[9]);
    if (ap > F(1e-290) && ap < F(1e290)) {
      F inv = F(1.0) / pre[9];
#pragma unroll
      for (int m = 9; m > 0; --m) {
        q[m] = inv * pre[m - 1];
        inv *= den[m];
      }
      q[0] = inv;
    } else {
#pragma unroll
      for (int m = 0; m < 10; ++m) q[m] = F(1.0) / den[m];
    }
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      l[c] = wl[c] + num[2 * c] * q[2 * c];
      r[c] = wr[c] - num[2 * c + 1] * q[2 * c + 1];
    }
  } else {
    // FP32: with a = d2 + eps, b = d1 + eps of one sign s, the limited
    // slope (1-k) d1 phiL + (1+k) d2 phiLi = ((1-k) d1 |a| + (1+k) d2 |b|)
    // 2/(|a|+|b|) is 4 s|a||b|/(|a|+|b|) - 4 eps w, w in [1-k, 1+k]/2, so
    // the reconstruction (a quarter of it) is the harmonic slope
    // a b/(a + b) shifted by eps w (at most 7e-10, far below FP32
    // rounding): one product, one sum and one quotient per side.
    // Components 0-1 and 2-3 go through the packed FP32x2 pipe (two
    // components per instruction, each rounded as its scalar FMA), 4 alone.
    (void)k;
#pragma unroll
    for (int c = 0; c < 4; c += 2) {
      const float2 m1 = make_float2(-1.f, -1.f), two = make_float2(2.f, 2.f),
                   e2 = make_float2(eps, eps);
      const float2 wl2 = make_float2(wl[c], wl[c + 1]), wr2 = make_float2(wr[c], wr[c + 1]);
      const float2 nd2 = __ffma2_rn(wr2, m1, wl2);  // -(wr - wl)
      const float2 dd1 = __ffma2_rn(make_float2(g1[c], g1[c + 1]), two, nd2);
      const float2 dd3 = __ffma2_rn(make_float2(g2[c], g2[c + 1]), two, nd2);
      const float2 a = __ffma2_rn(nd2, m1, e2);
      const float2 b = __fadd2_rn(dd1, e2), e3 = __fadd2_rn(dd3, e2);
      const float2 pl = __fmul2_rn(a, b), pr = __fmul2_rn(a, e3);
      const float2 sl = __fadd2_rn(a, b), sr = __fadd2_rn(a, e3);
      const float2 isl = make_float2(__fdividef(1.f, sl.x), __fdividef(1.f, sl.y));
      const float2 isr = make_float2(__fdividef(1.f, sr.x), __fdividef(1.f, sr.y));
      const float2 ql = __fmul2_rn(pl, isl), qr = __fmul2_rn(pr, isr);
      const float2 lz = make_float2(pl.x > 0.f ? ql.x : 0.f, pl.y > 0.f ? ql.y : 0.f);
      const float2 rz = make_float2(pr.x > 0.f ? qr.x : 0.f, pr.y > 0.f ? qr.y : 0.f);
      const float2 l2 = __fadd2_rn(wl2, lz), r2 = __ffma2_rn(rz, m1, wr2);
      d1[c] = dd1.x;
      d1[c + 1] = dd1.y;
      d3[c] = dd3.x;
      d3[c + 1] = dd3.y;
      l[c] = l2.x;
      l[c + 1] = l2.y;
      r[c] = r2.x;
      r[c + 1] = r2.y;
    }
    {
      const float d2 = wr[4] - wl[4];
      d1[4] = 2.f * g1[4] - d2;
      d3[4] = 2.f * g2[4] - d2;
      const float a = d2 + eps, b = d1[4] + eps, e3 = d3[4] + eps;
      const float pl = a * b, pr = a * e3;
      l[4] = wl[4] + (pl > 0.f ? __fdividef(pl, a + b) : 0.f);
      r[4] = wr[4] - (pr > 0.f ? __fdividef(pr, a + e3) : 0.f);
    }
  }
  if (wl[0] < d1[0] || wl[4] < d1[4]) {
#pragma unroll
    for (int c = 0; c < 5; ++c) l[c] = wl[c];
  }
  if (wr[0] < -d3[0] || wr[4] < -d3[4]) {
#pragma unroll
    for (int c = 0; c < 5; ++c) r[c] = wr[c];
  }
}

// sqrt: IEEE in double; x * rsqrt(x) in float (x >= 0).
__device__ __forceinline__ double xsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float xsqrt(float x) { return x > 0.f ? x * rsqrtf(x) : 0.f; }

// Rusanov edge flux (rusanov(), src/Physics/Riemann.cpp:369-478).
template <class F>
__device__ __forceinline__ void rusanov(const F wl[5], const F wr[5], const F g1[5],
                                        const F g2[5], F nx, F ny, F nz, F gamma, bool stab2,
                                        F stab2coef, F f[5]) {
  F l[5], r[5];
  muscl(wl, wr, g1, g2, l, r);
  F pL = l[0] * l[4] * (gamma - F(1.0));
  F pR = r[0] * r[4] * (gamma - F(1.0));
  const F cLe = l[4], cRe = r[4];
  F vnL = l[1] * nx + l[2] * ny + l[3] * nz;
  F vnR = r[1] * nx + r[2] * ny + r[3] * nz;
  l[4] = (l[4] + F(0.5) * (l[1] * l[1] + l[2] * l[2] + l[3] * l[3])) * l[0];
  l[1] *= l[0];
  l[2] *= l[0];
  l[3] *= l[0];
  r[4] = (r[4] + F(0.5) * (r[1] * r[1] + r[2] * r[2] + r[3] * r[3])) * r[0];
  r[1] *= r[0];
  r[2] *= r[0];
  r[3] *= r[0];
  // sound speed^2 = gamma p / rho with p = rho e (gamma - 1): gamma (gamma - 1) e
  // (the reference divides p by rho; the same value up to rounding); e is
  // the reconstructed internal energy, kept in cLe / cRe before the
  // conversion to total energy below.  c |D| is taken as one root,
  // sqrt(gamma (gamma - 1) e |D|^2), where the reference multiplies the
  // roots of the two (the same value up to rounding; one square root fewer)
  const F gl = gamma * (gamma - F(1.0)) * (nx * nx + ny * ny + nz * nz);
  F sl = fabs(vnL) + xsqrt(gl * cLe);
  F sr = fabs(vnR) + xsqrt(gl * cRe);
  F fw = sl > sr ? sl : sr;
  f[0] = l[0] * vnL + r[0] * vnR + fw * (r[0] - l[0]);
  f[1] = l[1] * vnL + r[1] * vnR + (pL + pR) * nx + fw * (r[1] - l[1]);
  f[2] = l[2] * vnL + r[2] * vnR + (pL + pR) * ny + fw * (r[2] - l[2]);
  f[3] = l[3] * vnL + r[3] * vnR + (pL + pR) * nz + fw * (r[3] - l[3]);
  f[4] = (l[4] + pL) * vnL + (r[4] + pR) * vnR + fw * (r[4] - l[4]);
  if (stab2) {
    F fws = stab2coef * fw;
#pragma unroll
    for (int c = 0; c < 5; ++c) f[c] -= fws * (l[c] - r[c]);
  }
}

// HLLC edge flux (hllc(), src/Physics/Riemann.cpp:480-650).
template <class F>
__device__ __forceinline__ void hllc(const F wl[5], const F wr[5], const F g1[5], const F g2[5],
                                     F dx, F dy, F dz, F gamma, bool stab2, F stab2coef,
                                     F f[5]) {
  F l[5], r[5];
  muscl(wl, wr, g1, g2, l, r);
  F nx = -dx, ny = -dy, nz = -dz;
  F len = sqrt(nx * nx + ny * ny + nz * nz);
  nx /= len;
  ny /= len;
  nz /= len;
  F qL = l[1] * nx + l[2] * ny + l[3] * nz;
  F qR = r[1] * nx + r[2] * ny + r[3] * nz;
  F pL = l[0] * l[4] * (gamma - F(1.0));
  F pR = r[0] * r[4] * (gamma - F(1.0));
  l[4] = (l[4] + F(0.5) * (l[1] * l[1] + l[2] * l[2] + l[3] * l[3])) * l[0];
  l[1] *= l[0];
  l[2] *= l[0];
  l[3] *= l[0];
  r[4] = (r[4] + F(0.5) * (r[1] * r[1] + r[2] * r[2] + r[3] * r[3])) * r[0];
  r[1] *= r[0];
  r[2] *= r[0];
  r[3] *= r[0];
  F cL = sqrt(gamma * pL / l[0]);
  F cR = sqrt(gamma * pR / r[0]);
  F sL = fmin(qL - cL, qR - cR);
  F sR = fmax(qL + cL, qR + cR);
  F tL = sL - qL;
  F tR = sR - qR;
  F sM = (r[0] * qR * tR - l[0] * qL * tL + pL - pR) / (r[0] * tR - l[0] * tL);
  F pS = pL - l[0] * tL * (qL - sM);
  F L2 = F(-2.0) * len;
  if (sL > F(0.0)) {
    F qL2 = qL * L2;
    f[0] = l[0] * qL2;
    f[1] = l[1] * qL2 + pL * (nx * L2);
    f[2] = l[2] * qL2 + pL * (ny * L2);
    f[3] = l[3] * qL2 + pL * (nz * L2);
    f[4] = (l[4] + pL) * qL2;
  } else if (sL <= F(0.0) && sM > F(0.0)) {
    F s = sL - sM;
    F uL0 = tL * l[0] / s;
    F uL1 = (tL * l[1] + (pS - pL) * nx) / s;
    F uL2 = (tL * l[2] + (pS - pL) * ny) / s;
    F uL3 = (tL * l[3] + (pS - pL) * nz) / s;
    F uL4 = (tL * l[4] - pL * qL + pS * sM) / s;
    F qL2 = qL * L2, sL2 = sL * L2;
    f[0] = l[0] * qL2 + sL2 * (uL0 - l[0]);
    f[1] = l[1] * qL2 + pL * (nx * L2) + sL2 * (uL1 - l[1]);
    f[2] = l[2] * qL2 + pL * (ny * L2) + sL2 * (uL2 - l[2]);
    f[3] = l[3] * qL2 + pL * (nz * L2) + sL2 * (uL3 - l[3]);
    f[4] = (l[4] + pL) * qL2 + sL2 * (uL4 - l[4]);
  } else if (sM <= F(0.0) && sR >= F(0.0)) {
    F s = sR - sM;
    F uR0 = tR * r[0] / s;
    F uR1 = (tR * r[1] + (pS - pR) * nx) / s;
    F uR2 = (tR * r[2] + (pS - pR) * ny) / s;
    F uR3 = (tR * r[3] + (pS - pR) * nz) / s;
    F uR4 = (tR * r[4] - pR * qR + pS * sM) / s;
    F qR2 = qR * L2, sR2 = sR * L2;
    f[0] = r[0] * qR2 + sR2 * (uR0 - r[0]);
    f[1] = r[1] * qR2 + pR * (nx * L2) + sR2 * (uR1 - r[1]);
    f[2] = r[2] * qR2 + pR * (ny * L2) + sR2 * (uR2 - r[2]);
    f[3] = r[3] * qR2 + pR * (nz * L2) + sR2 * (uR3 - r[3]);
    f[4] = (r[4] + pR) * qR2 + sR2 * (uR4 - r[4]);
  } else {
    F qR2 = qR * L2;
    f[0] = r[0] * qR2;
    f[1] = r[1] * qR2 + pR * (nx * L2);
    f[2] = r[2] * qR2 + pR * (ny * L2);
    f[3] = r[3] * qR2 + pR * (nz * L2);
    f[4] = (r[4] + pR) * qR2;
  }
  if (stab2) {
    F sl = fabs(qL) + cL;
    F sr = fabs(qR) + cR;
    F fws = stab2coef * (sl > sr ? sl : sr) * len;
#pragma unroll
    for (int c = 0; c < 5; ++c) f[c] -= fws * (l[c] - r[c]);
  }
}

// Adjacency entry: neighbour id (~q when this node is the second end) and
// the canonical edge integral, 16 bytes in FP32 mode, 32 in FP64 mode.
struct alignas(32) Ent64 {
  double dx, dy, dz;
  int32_t q, pad;
};
template <class F>
struct EntOf;
template <>
struct EntOf<float> {
  using type = int4;
};
template <>
struct EntOf<double> {
  using type = Ent64;
};


// Ring entries: copy one entry into its shared-memory slot, decode a landed one.
template <class E>
__device__ __forceinline__ void fetch_ent(E* slot, const E* g) {
#pragma unroll
  for (int i = 0; i < int(sizeof(E) / 16); ++i)
    cp_async16(reinterpret_cast<char*>(slot) + 16 * i, reinterpret_cast<const char*>(g) + 16 * i);
}
__device__ __forceinline__ void dec_ent(const int4* slot, int32_t& q, float& d0, float& d1,
                                        float& d2) {
  const int4 v = *slot;
  q = v.x;
  d0 = __int_as_float(v.y);
  d1 = __int_as_float(v.z);
  d2 = __int_as_float(v.w);
}
__device__ __forceinline__ void dec_ent(const Ent64* slot, int32_t& q, double& d0, double& d1,
                                        double& d2) {
  const double2* p = reinterpret_cast<const double2*>(slot);
  const double2 a = p[0], b = p[1];
  d0 = a.x;
  d1 = a.y;
  d2 = b.x;
  q = __double2loint(b.y);
}
// Ring depth in entries per thread: 8 x 16 bytes (FP32 entries) or
// 4 x 32 bytes (FP64 entries), 32 KiB per 256-thread block either way.
template <class E>
constexpr int ring_len() {
  return sizeof(E) == 16 ? 8 : 4;
}

// Flux slots: components 0-3 as one 16-byte (float) / 32-byte (double)
// record, component 4 in a separate array, so a gather costs two sectors.
__device__ __forceinline__ void store_f4(float* a, int64_t i, const float f[5]) {
  reinterpret_cast<float4*>(a)[i] = make_float4(f[0], f[1], f[2], f[3]);
}
__device__ __forceinline__ void store_f4(double* a, int64_t i, const double f[5]) {
  double2* q = reinterpret_cast<double2*>(a) + 2 * i;
  q[0] = make_double2(f[0], f[1]);
  q[1] = make_double2(f[2], f[3]);
}
__device__ __forceinline__ void load_f4(const float* a, int64_t i, float f[4]) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(a) + i);
  f[0] = v.x;
  f[1] = v.y;
  f[2] = v.z;
  f[3] = v.w;
}
__device__ __forceinline__ void load_f4(const double* a, int64_t i, double f[4]) {
  const double2* q = reinterpret_cast<const double2*>(a) + 2 * i;
  const double2 u = __ldg(q), v = __ldg(q + 1);
  f[0] = u.x;
  f[1] = u.y;
  f[2] = v.x;
  f[3] = v.y;
}

// G . v for one component, the same expression at both ends of an edge so
// that the projections negate exactly when v does.
template <class F>
__device__ __forceinline__ F proj(const F* g, F v0, F v1, F v2) {
  return g[0] * v0 + g[1] * v1 + g[2] * v2;
}

// Slot of gradient component c, direction j in a G record.  FP64: 3c + j.
// FP32 pairs components for the packed FP32x2 pipe:
//   [c0x c1x | c0y c1y | c0z c1z | c2x c3x | c2y c3y | c2z c3z | c4x c4y | c4z pad]
template <class F>
__host__ __device__ constexpr int gslot(int c, int j) {
  return sizeof(F) == 8 ? 3 * c + j : c < 2 ? 2 * j + c : c < 4 ? 6 + 2 * j + (c - 2) : 12 + j;
}
// Canonical gradients g[3c + j] to a record and back (register renaming).
template <class F>
__device__ __forceinline__ void to_rec(const F g[16], F o[16]) {
#pragma unroll
  for (int c = 0; c < 5; ++c)
#pragma unroll
    for (int j = 0; j < 3; ++j) o[gslot<F>(c, j)] = g[3 * c + j];
  o[15] = F(0);
}
template <class F>
__device__ __forceinline__ void from_rec(const F o[16], F g[16]) {
#pragma unroll
  for (int c = 0; c < 5; ++c)
#pragma unroll
    for (int j = 0; j < 3; ++j) g[3 * c + j] = o[gslot<F>(c, j)];
  g[15] = F(0);
}

// The five projections G.v at one end from an FP32 record (paired layout):
// components 0-1 and 2-3 two per packed FP32x2 instruction, 4 alone; the
// same expression at both ends, as proj.
__device__ __forceinline__ void proj5(const float g[16], float v0, float v1, float v2,
                                      float o[5]) {
  const float2 V0 = make_float2(v0, v0), V1 = make_float2(v1, v1), V2 = make_float2(v2, v2);
  float2 t = __fmul2_rn(make_float2(g[0], g[1]), V0);
  t = __ffma2_rn(make_float2(g[2], g[3]), V1, t);
  t = __ffma2_rn(make_float2(g[4], g[5]), V2, t);
  float2 u = __fmul2_rn(make_float2(g[6], g[7]), V0);
  u = __ffma2_rn(make_float2(g[8], g[9]), V1, u);
  u = __ffma2_rn(make_float2(g[10], g[11]), V2, u);
  o[0] = t.x;
  o[1] = t.y;
  o[2] = u.x;
  o[3] = u.y;
  o[4] = fmaf(g[14], v2, fmaf(g[13], v1, g[12] * v0));
}

// SoA -> node-major (host layout).
__global__ void k_soa_to_aos(int64_t n, int nc, const double* __restrict__ s,
                             double* __restrict__ a) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n * nc) return;
  int64_t p = i / nc;
  int c = static_cast<int>(i - p * nc);
  a[i] = s[c * n + p];
}

// W records from node-major host-layout U (drop-in entry points).
template <class F>
__global__ void k_prim_aos(int64_t n, const double* __restrict__ Ua, const F* __restrict__ Wsrc,
                           F* __restrict__ W) {
  int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (p >= n) return;
  double u[5];
#pragma unroll
  for (int c = 0; c < 5; ++c) u[c] = Ua[p * 5 + c];
  F o[8];
  load8(Wsrc + p * 8, o);
  prim_record<F>(u, o);
  store8(W + p * 8, o);
}

// G records <-> node-major 15-wide doubles.
template <class F>
__global__ void k_grec_to_aos(int64_t n, const F* __restrict__ G, double* __restrict__ a) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n * 15) return;
  int64_t p = i / 15;
  int c = static_cast<int>(i - p * 15);
  a[i] = double(G[p * 16 + gslot<F>(c / 3, c % 3)]);
}
template <class F>
__global__ void k_aos_to_grec(int64_t n, const double* __restrict__ a, F* __restrict__ G) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n * 16) return;
  int64_t p = i / 16;
  int c = static_cast<int>(i - p * 16);
  if (c == 15) {
    G[i] = F(0);
    return;
  }
  // the canonical index held by slot c
  int k = c;
  for (int cc = 0; cc < 5; ++cc)
    for (int j = 0; j < 3; ++j)
      if (gslot<F>(cc, j) == c) k = 3 * cc + j;
  G[i] = F(a[p * 15 + k]);
}

template <class F>
struct Adj {
  const int32_t* soff;
  const int32_t* swidth;
  const typename EntOf<F>::type* ent;
};
struct Bnd {
  const int32_t* bnode;  // node of each boundary index
  const int32_t* bidx;   // boundary index of each node, or -1
  const int32_t* bptr;   // per boundary node: its range of entries
  const int4* bent4;     // per entry: triangle nodes N0, N1, N2 and
                         // pos | symN0 << 2 | symN1 << 3 | symN2 << 4
};
// Per-node factors of the FP32-mode epilogue: 1/vol and cbrt(vol).
struct NodeAux {
  const double* ivol;
  const float* cbrtv;
};

// Nodal gradients of primitive variables (riemann::grad,
// src/Physics/Riemann.cpp:229-367): sum over the node's edges of
// -/+ D (u_p + u_q) plus the boundary-triangle term, optionally divided by the
// nodal volume (RieCG::rhs, src/Inciter/RieCG.cpp:936-939).
//
// The adjacency entries stream into a per-thread ring in shared memory
// (cp.async, RG - 1 groups of GU entries ahead); each group's GU neighbour
// records are gathered together, so GU gathers are in flight per thread while
// the entry stream runs ahead.  The ring is kept small: shared memory comes
// out of the L1 capacity that serves the neighbour gathers.
// Weak gradient to nodal gradient: divide by the nodal volume
// (RieCG::rhs, src/Inciter/RieCG.cpp:936-939), as 1/vol in FP32 mode.
template <class F>
__device__ __forceinline__ void finish_grad(const F g[15], int divide,
                                            const double* __restrict__ vol, NodeAux aux,
                                            int64_t p, F o[16]) {
  if (divide) {
    if constexpr (sizeof(F) == 8) {
      const double v = vol[p];
#pragma unroll
      for (int i = 0; i < 15; ++i) o[i] = g[i] / v;
    } else {
      const float iv = float(aux.ivol[p]);
#pragma unroll
      for (int i = 0; i < 15; ++i) o[i] = g[i] * iv;
    }
  } else {
#pragma unroll
    for (int i = 0; i < 15; ++i) o[i] = g[i];
  }
}

template <class F>
struct GradShape {
  static constexpr int GU = 2;                        // entries per group
  static constexpr int RG = 2;                        // ring groups per thread
  static constexpr int BLOCK = 256;
};

template <class F>
__global__ void __launch_bounds__(GradShape<F>::BLOCK)
    k_grad(int64_t n, Adj<F> adj, const F* __restrict__ W, Bnd bnd,
           const double* __restrict__ vol, NodeAux aux, int divide, F* __restrict__ G) {
  using EntT = typename EntOf<F>::type;
  constexpr int GU = GradShape<F>::GU, RG = GradShape<F>::RG, NB = GradShape<F>::BLOCK;
  static_assert((RG & (RG - 1)) == 0 && RG >= 2, "ring of a power-of-two number of groups");
  __shared__ EntT ring[GU * RG][NB];
  int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (p >= n) return;
  const int tid = threadIdx.x;
  const int lane = static_cast<int>(p & (kSlice - 1));
  const int64_t s = p >> 5;
  const int32_t off = __ldg(adj.soff + s), w = __ldg(adj.swidth + s);
  const EntT* src = adj.ent + off + lane;
  // group j holds entries GU*j..GU*j+GU-1; groups 0..RG-2 are requested up
  // front, group k+RG-1 while group k is processed, into the slots group k-1
  // freed
#pragma unroll
  for (int j = 0; j < RG - 1; ++j) {
#pragma unroll
    for (int u = 0; u < GU; ++u)
      if (GU * j + u < w) fetch_ent(&ring[GU * j + u][tid], src + (GU * j + u) * kSlice);
    cp_async_commit();
  }
  F wp[5];
  load5(W + p * 8, wp);
  F g[15];
#pragma unroll
  for (int i = 0; i < 15; ++i) g[i] = F(0);
  const int ng = (w + GU - 1) / GU;
  for (int kg = 0; kg < ng; ++kg) {
    cp_async_wait<RG - 2>();
    const int sl = (kg & (RG - 1)) * GU;
    int32_t q[GU];
    F d[GU][3];
#pragma unroll
    for (int u = 0; u < GU; ++u) {
      q[u] = kPad;
      if (GU * kg + u < w) dec_ent(&ring[sl + u][tid], q[u], d[u][0], d[u][1], d[u][2]);
    }
    const int jn = kg + RG - 1;
    const int sn = (jn & (RG - 1)) * GU;
#pragma unroll
    for (int u = 0; u < GU; ++u)
      if (GU * jn + u < w) fetch_ent(&ring[sn + u][tid], src + (GU * jn + u) * kSlice);
    cp_async_commit();
    F wq[GU][5];
#pragma unroll
    for (int u = 0; u < GU; ++u) {
      if (q[u] == kPad) continue;
      if (q[u] >= 0) {  // this node is the first end: G -= f
        d[u][0] = -d[u][0];
        d[u][1] = -d[u][1];
        d[u][2] = -d[u][2];
      } else {
        q[u] = ~q[u];
      }
      load5(W + int64_t(q[u]) * 8, wq[u]);
    }
#pragma unroll
    for (int u = 0; u < GU; ++u) {
      if (q[u] == kPad) continue;
#pragma unroll
      for (int c = 0; c < 5; ++c) {
        F sum = wq[u][c] + wp[c];
        g[c * 3 + 0] += d[u][0] * sum;
        g[c * 3 + 1] += d[u][1] * sum;
        g[c * 3 + 2] += d[u][2] * sum;
      }
    }
  }
  cp_async_wait<0>();
  F o[16];
  if (__ldg(bnd.bidx + p) >= 0) {
    // boundary node: the domain sum as it stands; k_grad_bnd adds the
    // boundary integral and divides (the reference's order of summation)
#pragma unroll
    for (int i = 0; i < 15; ++i) o[i] = g[i];
  } else {
    finish_grad(g, divide, vol, aux, p, o);
  }
  o[15] = F(0);
  F rec[16];
  to_rec(o, rec);
  store16(G + p * 16, rec);
}

// Boundary-triangle term of riemann::grad (src/Physics/Riemann.cpp:329-364)
// at boundary node p, added to g in the node's triangle order.
template <class F>
__device__ __forceinline__ void grad_bnd_term(const Bnd& bnd, int32_t bi, const F* __restrict__ W,
                                              F g[15]) {
  for (int32_t j = __ldg(bnd.bptr + bi); j < __ldg(bnd.bptr + bi + 1); ++j) {
    const int4 te = __ldg(bnd.bent4 + j);
    F a[8], b[8], c[8];
    load8(W + int64_t(te.x) * 8, a);
    load8(W + int64_t(te.y) * 8, b);
    load8(W + int64_t(te.z) * 8, c);
    F bax = b[5] - a[5], bay = b[6] - a[6], baz = b[7] - a[7];
    F cax = c[5] - a[5], cay = c[6] - a[6], caz = c[7] - a[7];
    F nn[3] = {(bay * caz - cay * baz) / F(12.0), (baz * cax - caz * bax) / F(12.0),
               (bax * cay - cax * bay) / F(12.0)};
#pragma unroll
    for (int cc = 0; cc < 5; ++cc) {
      F uab = (a[cc] + b[cc]) / F(4.0);
      F ubc = (b[cc] + c[cc]) / F(4.0);
      F uca = (c[cc] + a[cc]) / F(4.0);
      F gg[3] = {uab + uca + a[cc], uab + ubc + b[cc], ubc + uca + c[cc]};
#pragma unroll
      for (int j2 = 0; j2 < 3; ++j2) g[cc * 3 + j2] += gg[j2] * nn[j2];
    }
  }
}

// Boundary nodes of the gradient pass, one thread per boundary node.
template <class F>
__global__ void __launch_bounds__(kBlock) k_grad_bnd(int64_t nbn, Bnd bnd,
                                                      const F* __restrict__ W,
                                                      const double* __restrict__ vol,
                                                      NodeAux aux, int divide, F* G) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= nbn) return;
  const int64_t p = __ldg(bnd.bnode + i);
  F rec[16], g[16];
  load16(G + p * 16, rec);
  from_rec(rec, g);
  grad_bnd_term(bnd, static_cast<int32_t>(i), W, g);
  F o[16];
  finish_grad(g, divide, vol, aux, p, o);
  o[15] = F(0);
  to_rec(o, rec);
  store16(G + p * 16, rec);
}

// FP32-mode per-node CFL time step from the FP64 state (the formula of
// RieCG::dt, src/Inciter/RieCG.cpp:827-838, in float with cbrt(vol) given).
__device__ __forceinline__ float node_dt_f(const double ud[5], float L, float g) {
  const float r = float(ud[0]);
  const float ir = __frcp_rn(r);
  const float uu = float(ud[1]) * ir, vv = float(ud[2]) * ir, ww = float(ud[3]) * ir;
  const float k2 = uu * uu + vv * vv + ww * ww;
  const float pr = (float(ud[4]) - 0.5f * r * k2) * (g - 1.f);
  const float c = xsqrt(g * fmaxf(pr, 0.f) * ir);
  const float vel = xsqrt(k2);
  return __fdividef(L, fmaxf(vel + c, 1.0e-8f));
}

// Half-edge residual, pass 1: every edge flux once, at the edge's owner end
// (riemann::rhs advdom, src/Physics/Riemann.cpp:695-759), in the edge's
// canonical orientation in FP64 mode (-f summed into the owner's partial
// residual when the owner is the first end, +f otherwise) and in the owner's
// orientation in FP32 mode; the other end's contribution is stored into
// that end's list-2 slot (pos1), so the second pass reads its fluxes as a
// coalesced stream.
template <class F>
struct Half {
  const int32_t* soff1;
  const int32_t* sw1;
  const typename EntOf<F>::type* ent1;
  const int32_t* pos1;
  const int32_t* soff2;
  const int32_t* sw2;
  int64_t nent2;
};

template <class F, int FLUX>
__global__ void __launch_bounds__(kBlock, sizeof(F) == 4 ? 3 : 1)
    k_flux1(int64_t n, Half<F> h, const F* __restrict__ W, const F* __restrict__ G,
            double gamma_d, int stab2, double stab2coef_d, F* __restrict__ fbuf,
            F* __restrict__ Rp) {
  using EntT = typename EntOf<F>::type;
  constexpr int RL = ring_len<EntT>();
  __shared__ EntT ring[RL][kBlock];
  int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (p >= n) return;
  const int tid = threadIdx.x;
  const F gamma = F(gamma_d), stab2coef = F(stab2coef_d);
  const int lane = static_cast<int>(p & (kSlice - 1));
  const int64_t s = p >> 5;
  const int32_t off = __ldg(h.soff1 + s), w = __ldg(h.sw1 + s);
  const EntT* src = h.ent1 + off + lane;
  // entries 0..RL-2 requested up front, entry k+RL-1 while entry k is
  // processed, into the slot entry k-1 has freed
#pragma unroll
  for (int j = 0; j < RL - 1; ++j) {
    if (j < w) fetch_ent(&ring[j][tid], src + j * kSlice);
    cp_async_commit();
  }
  F wp[8], gp[16];
  load8(W + p * 8, wp);
  load16(G + p * 16, gp);
  F R[5] = {F(0), F(0), F(0), F(0), F(0)};
  for (int k = 0; k < w; ++k) {
    const int32_t e = off + k * kSlice + lane;
    cp_async_wait<RL - 2>();
    int32_t q;
    F d0, d1, d2;
    dec_ent(&ring[k & (RL - 1)][tid], q, d0, d1, d2);
    if (k + RL - 1 < w) fetch_ent(&ring[(k + RL - 1) & (RL - 1)][tid], src + (k + RL - 1) * kSlice);
    cp_async_commit();
    if (q == kPad) continue;
    const int32_t dst = __ldg(h.pos1 + e);
    const bool first = q >= 0;
    if (!first) q = ~q;
    F wq[8], gq[16];
    load8(W + int64_t(q) * 8, wq);
    load16(G + int64_t(q) * 16, gq);
    const F v0 = wq[5] - wp[5], v1 = wq[6] - wp[6], v2 = wq[7] - wp[7];
    F f[5], fo[5];
    if constexpr (sizeof(F) == 4) {
      // FP32: the flux in the owner's orientation (p -> q, the edge integral
      // signed accordingly), with no per-component orientation selects; it
      // differs from the canonical-orientation flux only through the
      // limiter's 1e-9 regularisation, far below FP32 rounding of the sums
      F g1[5], g2[5];
      proj5(gp, v0, v1, v2, g1);
      proj5(gq, v0, v1, v2, g2);
      if (!first) {
        d0 = -d0;
        d1 = -d1;
        d2 = -d2;
      }
      if (FLUX == XG_HLLC)
        hllc(wp, wq, g1, g2, d0, d1, d2, gamma, stab2 != 0, stab2coef, f);
      else
        rusanov(wp, wq, g1, g2, d0, d1, d2, gamma, stab2 != 0, stab2coef, f);
#pragma unroll
      for (int c = 0; c < 5; ++c) {
        R[c] -= f[c];
        fo[c] = f[c];
      }
    } else {
      // FP64: the canonical orientation (left = first end), as the reference
      F wl[5], wr[5], g1[5], g2[5];
#pragma unroll
      for (int c = 0; c < 5; ++c) {
        const F A = proj(gp + 3 * c, v0, v1, v2);
        const F B = proj(gq + 3 * c, v0, v1, v2);
        g1[c] = first ? A : -B;
        g2[c] = first ? B : -A;
        wl[c] = first ? wp[c] : wq[c];
        wr[c] = first ? wq[c] : wp[c];
      }
      if (FLUX == XG_HLLC)
        hllc(wl, wr, g1, g2, d0, d1, d2, gamma, stab2 != 0, stab2coef, f);
      else
        rusanov(wl, wr, g1, g2, d0, d1, d2, gamma, stab2 != 0, stab2coef, f);
      const F sg = first ? F(-1) : F(1);
#pragma unroll
      for (int c = 0; c < 5; ++c) {
        R[c] += sg * f[c];
        fo[c] = -sg * f[c];
      }
    }
    store_f4(fbuf, dst, fo);
    fbuf[4 * h.nent2 + dst] = fo[4];
  }
  cp_async_wait<0>();
#pragma unroll
  for (int c = 0; c < 5; ++c) Rp[c * n + p] = R[c];
}

// Boundary integral of riemann::rhs (advbnd, src/Physics/Riemann.cpp:768-878)
// at the boundary node with index bi, added to R in the node's triangle order.
template <class F>
__device__ __forceinline__ void rhs_bnd_term(const Bnd& bnd, int32_t bi, const F* __restrict__ W,
                                             F gamma, F R[5]) {
  for (int32_t j = __ldg(bnd.bptr + bi); j < __ldg(bnd.bptr + bi + 1); ++j) {
    const int4 te = __ldg(bnd.bent4 + j);
    const int32_t pos = te.w & 3;
    F x[3][8];
    load8(W + int64_t(te.x) * 8, x[0]);
    load8(W + int64_t(te.y) * 8, x[1]);
    load8(W + int64_t(te.z) * 8, x[2]);
    const bool sy[3] = {((te.w >> 2) & 1) != 0, ((te.w >> 3) & 1) != 0, ((te.w >> 4) & 1) != 0};
    F bax = x[1][5] - x[0][5], bay = x[1][6] - x[0][6], baz = x[1][7] - x[0][7];
    F cax = x[2][5] - x[0][5], cay = x[2][6] - x[0][6], caz = x[2][7] - x[0][7];
    F nx = (bay * caz - cay * baz) / F(12.0);
    F ny = (baz * cax - caz * bax) / F(12.0);
    F nz = (bax * cay - cax * bay) / F(12.0);
    F fl[3][5];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const F r = x[a][0], u = x[a][1], v = x[a][2], ww = x[a][3], ie = x[a][4];
      const F pr = r * ie * (gamma - F(1.0));
      const F vn = sy[a] ? F(0) : (nx * u + ny * v + nz * ww);
      const F re = r * (ie + F(0.5) * (u * u + v * v + ww * ww));
      fl[a][0] = r * vn;
      fl[a][1] = r * u * vn + pr * nx;
      fl[a][2] = r * v * vn + pr * ny;
      fl[a][3] = r * ww * vn + pr * nz;
      fl[a][4] = (re + pr) * vn;
    }
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      // own value, plus the two averages of the pairs containing this node
      F fa = fl[0][c], fb = fl[1][c], fcc = fl[2][c];
      F fab = (fa + fb) / F(4.0), fbc = (fb + fcc) / F(4.0), fca = (fcc + fa) / F(4.0);
      R[c] += pos == 0 ? (fab + fca + fa) : (pos == 1 ? (fab + fbc + fb) : (fbc + fca + fcc));
    }
  }
}

// Nodal BC program, one entry per BC node, applied in the reference order:
// Dirichlet, symmetry (one projection per symmetry set containing the node),
// farfield, pressure (physics::dirbc/symbc/farbc/prebc,
// src/Physics/BC.cpp:29-241).
struct BCProg {
  int64_t nbc;
  const int32_t* node;
  const int32_t* dir;
  const int32_t* symp;
  const int32_t* far;
  const int32_t* pre;
  const int32_t* dirmask;
  const double* dirval;
  const double* symn;
  const double* farn;
  const double* preval;
  double far5[5];
  SrcPrm prob;           // the problem whose analytic state mask-1 Dirichlet values take
  const double* dirxyz;  // [ndir][3] coordinates of the Dirichlet nodes
};

// BC program entry i applied to the conserved state u of its node at time t.
__device__ __forceinline__ void apply_bc(const BCProg& bc, int64_t i, double gamma, double t,
                                         double u[5]) {
  const int32_t d = bc.dir[i];
  if (d >= 0) {
    const double* x = bc.dirxyz + d * 3;
    dirichlet(bc.prob, x[0], x[1], x[2], t, bc.dirmask + d * 5, bc.dirval + d * 5, u);
  }
  for (int32_t k = bc.symp[i]; k < bc.symp[i + 1]; ++k) {
    const double* nn = bc.symn + 3 * k;
    double vn = u[1] * nn[0] + u[2] * nn[1] + u[3] * nn[2];
    u[1] -= vn * nn[0];
    u[2] -= vn * nn[1];
    u[3] -= vn * nn[2];
  }
  const int32_t f = bc.far[i];
  if (f >= 0) {
    const double* nn = bc.farn + 3 * f;
    const double fr = bc.far5[0], fu = bc.far5[1], fv = bc.far5[2], fw = bc.far5[3],
                 fp = bc.far5[4];
    double vn = fu * nn[0] + fv * nn[1] + fw * nn[2];
    double a = sqrt(gamma * fp / fr);
    double M = vn / a;
    if (M <= -1.0) {
      u[0] = fr;
      u[1] = fr * fu;
      u[2] = fr * fv;
      u[3] = fr * fw;
      u[4] = fp / (gamma - 1.0) + 0.5 * fr * (fu * fu + fv * fv + fw * fw);
    } else if (M > -1.0 && M < 0.0) {
      double pr = (u[4] - 0.5 * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) / u[0]) *
                  (gamma - 1.0);
      u[0] = fr;
      u[1] = fr * fu;
      u[2] = fr * fv;
      u[3] = fr * fw;
      u[4] = pr / (gamma - 1.0) + 0.5 * fr * (fu * fu + fv * fv + fw * fw);
    } else if (M >= 0.0 && M < 1.0) {
      double r = u[0], uu = u[1] / r, vv = u[2] / r, ww = u[3] / r;
      u[4] = fp / (gamma - 1.0) + 0.5 * r * (uu * uu + vv * vv + ww * ww);
    }
  }
  const int32_t pr = bc.pre[i];
  if (pr >= 0) {
    u[0] = bc.preval[pr * 2 + 0];
    double r = u[0], uu = u[1] / r, vv = u[2] / r, ww = u[3] / r;
    u[4] = bc.preval[pr * 2 + 1] / (gamma - 1.0) + 0.5 * r * (uu * uu + vv * vv + ww * ww);
  }
}

// One node's stage state (RieCG::solve, src/Inciter/RieCG.cpp:1010-1021):
// un = Un - rkcoef*dt*R/vol from uo (U at stage 0, copied to Un, and Un
// after; in the time loop's lean form uo is U, the state at the start of the
// step, at every stage and nothing is copied).  The FP64 mode keeps the
// reference's expression; FP32 mode uses 1/vol (no FP64 division per node).
template <class F, int STAGE, bool LEAN = false>
__device__ __forceinline__ void stage_state(int64_t n, int64_t p, const F R[5],
                                            const double uo[5],
                                            const double* __restrict__ vol, NodeAux aux,
                                            double dt, double* Un, double un[5]) {
  constexpr double rk = STAGE == 0 ? 1.0 / 3.0 : (STAGE == 1 ? 0.5 : 1.0);
  if constexpr (sizeof(F) == 8) {
    const double v = vol[p];
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      if (STAGE == 0 && !LEAN) Un[c * n + p] = uo[c];
      un[c] = uo[c] - rk * dt * double(R[c]) / v;
    }
  } else {
    const double cf = rk * dt * aux.ivol[p];
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      if (STAGE == 0 && !LEAN) Un[c * n + p] = uo[c];
      un[c] = uo[c] - cf * double(R[c]);
    }
  }
}

// Store a node's new state u: U, its primitive record (coordinates from wp)
// and, when want_dt, its CFL time step (src/Inciter/RieCG.cpp:827-839, the
// FP32 estimate in FP32 mode); DBL_MAX otherwise.
template <class F>
__device__ __forceinline__ double store_node(int64_t n, int64_t p, const double u[5],
                                             const F wp[8], bool want_dt,
                                             const double* __restrict__ vol, NodeAux aux,
                                             double gamma_d, double* U, F* __restrict__ Wout) {
  double dtp = DBL_MAX;
#pragma unroll
  for (int c = 0; c < 5; ++c) U[c * n + p] = u[c];
  F o[8] = {F(0), F(0), F(0), F(0), F(0), wp[5], wp[6], wp[7]};
  prim_record<F>(u, o);
  store8(Wout + p * 8, o);
  if (want_dt)
    dtp = sizeof(F) == 8 ? node_dt(u, vol[p], gamma_d)
                         : double(node_dt_f(u, aux.cbrtv[p], float(gamma_d)));
  return dtp;
}

// A host-layout (node-major) state as the context's state in one pass: the
// FP64 SoA state, the primitive records (coordinates kept) and the CFL
// minimum of the new state (RieCG::dt's formula, the FP32 estimate in FP32
// mode) -- what xg_riecg_set_state needs, reading the upload once.
// The block's nodes are read as one contiguous run of node-major doubles
// (coalesced: Ua may be the caller's pinned host buffer, read over the host
// link) and staged in shared memory.
template <class F>
__global__ void __launch_bounds__(kBlock)
    k_state_in(int64_t n, const double* __restrict__ Ua, const double* __restrict__ vol,
               NodeAux aux, double gamma_d, double* __restrict__ U, F* __restrict__ W,
               unsigned long long* dtmin) {
  __shared__ double su[kBlock * 5];
  const int64_t p0 = blockIdx.x * int64_t(kBlock);
  const int64_t p = p0 + threadIdx.x;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int64_t e = p0 * 5 + threadIdx.x + k * kBlock;
    if (e < n * 5) su[threadIdx.x + k * kBlock] = Ua[e];
  }
  __syncthreads();
  double dtp = DBL_MAX;
  if (p < n) {
    double u[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) u[c] = su[threadIdx.x * 5 + c];
    F o[8];
    load8(W + p * 8, o);  // coordinates
    dtp = store_node<F>(n, p, u, o, true, vol, aux, gamma_d, U, W);
  }
  block_min_atomic(dtp, dtmin);
}

// Store a node's stage state: in the time loop's lean form the inner stages
// write only the primitive record (the FP64 state of an inner stage is not
// read again: every stage updates from the state at the start of the step);
// otherwise as store_node.
template <class F, int STAGE, bool LEAN>
__device__ __forceinline__ double store_stage(int64_t n, int64_t p, const double u[5],
                                              const F wp[8], const double* __restrict__ vol,
                                              NodeAux aux, double gamma_d, double* U,
                                              F* __restrict__ Wout) {
  if (LEAN && STAGE != 2) {
    if constexpr (sizeof(F) == 8) {
      double pw[5];
      prim5(u, pw);
      F o[8] = {F(pw[0]), F(pw[1]), F(pw[2]), F(pw[3]), F(pw[4]), wp[5], wp[6], wp[7]};
      store8(Wout + p * 8, o);
    } else {
      const float r = float(u[0]);
      const float ir = __frcp_rn(r);
      const float uu = float(u[1]) * ir, vv = float(u[2]) * ir, ww = float(u[3]) * ir;
      const float ie = float(u[4]) * ir - 0.5f * (uu * uu + vv * vv + ww * ww);
      F o[8] = {r, uu, vv, ww, ie, wp[5], wp[6], wp[7]};
      store8(Wout + p * 8, o);
    }
    return DBL_MAX;
  }
  return store_node<F>(n, p, u, wp, STAGE == 2, vol, aux, gamma_d, U, Wout);
}


// s V per node at the time of the current step (coordinates from the
// primitive records), once per step: every stage subtracts it.
template <class F>
__global__ void __launch_bounds__(kBlock)
    k_src(int64_t n, SrcPrm q, const Scalars* __restrict__ sc, const F* __restrict__ W,
          const double* __restrict__ vol, F* __restrict__ Sv) {
  const int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (p >= n) return;
  const F* w = W + p * 8;
  double o[5];
  problem_source(q, double(w[5]), double(w[6]), double(w[7]), sc->t, o);
  const double v = vol[p];
#pragma unroll
  for (int c = 0; c < 5; ++c) Sv[c * n + p] = F(o[c] * v);
}

// Half-edge residual, pass 2: the fluxes of the edges the other end owns and
// (optionally) the RK update of one stage with the new primitive records and,
// on the last stage, the CFL minimum.  Boundary nodes only park their domain
// residual in Rb: k_rhs_bnd adds their boundary integral and updates them,
// so no warp here waits on the triangle gathers.
template <class F, int STAGE, bool UPDATE, bool LEAN>
__global__ void __launch_bounds__(kBlock, sizeof(F) == 4 ? 4 : 1)
    k_rhs2(int64_t n, Half<F> h, const F* __restrict__ fbuf, const F* __restrict__ Rp,
           const F* __restrict__ W, Bnd bnd, int64_t nbn, F* __restrict__ Rb,
           const double* __restrict__ vol, NodeAux aux, double gamma_d,
           const Scalars* __restrict__ scal, double* U, double* Un, F* __restrict__ Wout,
           double* __restrict__ Rout, unsigned long long* dtmin, const F* __restrict__ Sv) {
  int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  const bool active = p < n;
  double dtp = DBL_MAX;
  if (active) {
    const int lane = static_cast<int>(p & (kSlice - 1));
    const int64_t s = p >> 5;
    const int32_t off = __ldg(h.soff2 + s), w = __ldg(h.sw2 + s);
    const int32_t bi = __ldg(bnd.bidx + p);
    // every per-node load is issued before the flux stream is summed
    F R[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) R[c] = Rp[c * n + p];
    double uo[5];
    if (UPDATE && bi < 0) {
#pragma unroll
      for (int c = 0; c < 5; ++c) uo[c] = (STAGE == 0 || LEAN) ? U[c * n + p] : Un[c * n + p];
    }
    F wp[8];
    if (UPDATE && bi < 0) load8(W + p * 8, wp);
    // the other ends' contributions, a coalesced stream (padding slots hold
    // 0), four slots per batch with all of a batch's loads in flight
    for (int k0 = 0; k0 < w; k0 += 4) {
      F f[4][4], f4[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (k0 + u < w) {
          const int64_t e = off + (k0 + u) * kSlice + lane;
          load_f4(fbuf, e, f[u]);
          f4[u] = __ldg(fbuf + 4 * h.nent2 + e);
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (k0 + u < w) {
#pragma unroll
          for (int c = 0; c < 4; ++c) R[c] += f[u][c];
          R[4] += f4[u];
        }
      }
    }
    // the manufactured source after the domain (and, in k_rhs_bnd, the
    // boundary) sums, as riemann::rhs adds it last
    if (Sv && bi < 0) {
#pragma unroll
      for (int c = 0; c < 5; ++c) R[c] -= Sv[c * n + p];
    }
    if (bi >= 0) {
#pragma unroll
      for (int c = 0; c < 5; ++c) Rb[c * nbn + bi] = R[c];
    } else if (!UPDATE) {
#pragma unroll
      for (int c = 0; c < 5; ++c) Rout[p * 5 + c] = double(R[c]);
    } else {
      double un[5];
      stage_state<F, STAGE, LEAN>(n, p, R, uo, vol, aux, scal->dt, Un, un);
      dtp = store_stage<F, STAGE, LEAN>(n, p, un, wp, vol, aux, gamma_d, U, Wout);
    }
  }
  if (UPDATE && STAGE == 2) block_min_atomic(dtp, dtmin);
}

// Boundary nodes of pass 2, one thread per boundary node: the boundary
// integral after the domain residual (the reference's order), the stage
// update, then the node's nodal BCs (RieCG::BC after RieCG::solve's update,
// src/Inciter/RieCG.cpp:1010-1030; every BC node lies on a boundary
// triangle) and, on the last stage, the CFL time step of the final state.
template <class F, int STAGE, bool UPDATE, bool LEAN>
__global__ void __launch_bounds__(kBlock)
    k_rhs_bnd(int64_t n, int64_t nbn, Bnd bnd, const F* __restrict__ Rb,
              const F* __restrict__ W, const int32_t* __restrict__ bcof, BCProg bc,
              const double* __restrict__ vol, NodeAux aux, double gamma_d,
              const Scalars* __restrict__ scal, double* U, double* Un, F* __restrict__ Wout,
              double* __restrict__ Rout, unsigned long long* dtmin, const F* __restrict__ Sv) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  double dtp = DBL_MAX;
  if (i < nbn) {
    const int64_t p = __ldg(bnd.bnode + i);
    F R[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) R[c] = Rb[c * nbn + i];
    double uo[5];
    if (UPDATE) {
#pragma unroll
      for (int c = 0; c < 5; ++c) uo[c] = (STAGE == 0 || LEAN) ? U[c * n + p] : Un[c * n + p];
    }
    F wp[8];
    load8(W + p * 8, wp);
    const int32_t b = UPDATE ? __ldg(bcof + i) : -1;
    rhs_bnd_term(bnd, static_cast<int32_t>(i), W, F(gamma_d), R);
    if (Sv) {
#pragma unroll
      for (int c = 0; c < 5; ++c) R[c] -= Sv[c * n + p];
    }
    if (!UPDATE) {
#pragma unroll
      for (int c = 0; c < 5; ++c) Rout[p * 5 + c] = double(R[c]);
    } else {
      double un[5];
      stage_state<F, STAGE, LEAN>(n, p, R, uo, vol, aux, scal->dt, Un, un);
      // at the stage's time, t + c dt with c = 1/3, 1/2, 1 (RieCG.cpp:1028)
      constexpr double rkc = STAGE == 0 ? 1.0 / 3.0 : (STAGE == 1 ? 1.0 / 2.0 : 1.0);
      if (b >= 0) apply_bc(bc, b, gamma_d, scal->t + rkc * scal->dt, un);
      dtp = store_stage<F, STAGE, LEAN>(n, p, un, wp, vol, aux, gamma_d, U, Wout);
    }
  }
  if (UPDATE && STAGE == 2) block_min_atomic(dtp, dtmin);
}

// Edge-coloured residual, the comparison design for the scatter of the
// edge fluxes (xg_riecg_rhs_coloured, FP32 mode): the owned edges split into
// colour classes in which no two edges share a node; one launch per class,
// one thread per edge, evaluates the flux once (in the owner's orientation,
// as k_flux1 does in FP32) and updates both ends' residual records in
// place, R_p -= f and R_q += f, with plain loads and stores: no atomics and
// no deposit slots, at the cost of one launch per colour and of scattered
// read-modify-writes of both ends' records (riemann::rhs advdom,
// src/Physics/Riemann.cpp:695-759, adds -f and +f the same way).
template <int FLUX>
__global__ void __launch_bounds__(kBlock)
    k_flux_colour(int64_t m, const int2* __restrict__ pq, const float4* __restrict__ dd,
                  const float* __restrict__ W, const float* __restrict__ G, double gamma_d,
                  int stab2, double stab2coef_d, float* R) {
  const int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (e >= m) return;
  const float gamma = float(gamma_d), stab2coef = float(stab2coef_d);
  const int2 ends = __ldg(pq + e);
  const float4 d = __ldg(dd + e);
  float wp[8], wq[8], gp[16], gq[16];
  load8(W + int64_t(ends.x) * 8, wp);
  load8(W + int64_t(ends.y) * 8, wq);
  load16(G + int64_t(ends.x) * 16, gp);
  load16(G + int64_t(ends.y) * 16, gq);
  const float v0 = wq[5] - wp[5], v1 = wq[6] - wp[6], v2 = wq[7] - wp[7];
  float g1[5], g2[5], f[5];
  proj5(gp, v0, v1, v2, g1);
  proj5(gq, v0, v1, v2, g2);
  if (FLUX == XG_HLLC)
    hllc(wp, wq, g1, g2, d.x, d.y, d.z, gamma, stab2 != 0, stab2coef, f);
  else
    rusanov(wp, wq, g1, g2, d.x, d.y, d.z, gamma, stab2 != 0, stab2coef, f);
  // each record is read and written by this thread alone in this launch
  float rp[8], rq[8];
  load8(R + int64_t(ends.x) * 8, rp);
  load8(R + int64_t(ends.y) * 8, rq);
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    rp[c] -= f[c];
    rq[c] += f[c];
  }
  store8(R + int64_t(ends.x) * 8, rp);
  store8(R + int64_t(ends.y) * 8, rq);
}

// The coloured residual's node epilogue: the domain sums plus, at boundary
// nodes, the boundary integral (in the reference's order), as FP64
// node-major output.
__global__ void __launch_bounds__(kBlock)
    k_colour_out(int64_t n, const float* __restrict__ R, Bnd bnd, const float* __restrict__ W,
                 double gamma, const float* __restrict__ Sv, double* __restrict__ Rout) {
  const int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (p >= n) return;
  float r[8];
  load8(R + p * 8, r);
  const int32_t bi = __ldg(bnd.bidx + p);
  if (bi >= 0) rhs_bnd_term(bnd, bi, W, float(gamma), r);
  if (Sv) {
#pragma unroll
    for (int c = 0; c < 5; ++c) r[c] -= Sv[c * n + p];
  }
#pragma unroll
  for (int c = 0; c < 5; ++c) Rout[p * 5 + c] = double(r[c]);
}

// Nodal BCs on the device state (RieCG::BC), one thread per BC node; refreshes
// the node's primitive record and, when asked, its CFL dt.
template <class F>
__global__ void __launch_bounds__(kBlock) k_bc(int64_t n, BCProg bc, double gamma, double* U,
                                                F* __restrict__ W, const double* __restrict__ vol,
                                                NodeAux aux, double t, int want_dt,
                                                unsigned long long* dtmin) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  double dtp = DBL_MAX;
  if (i < bc.nbc) {
    const int64_t p = bc.node[i];
    double u[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) u[c] = U[c * n + p];
    apply_bc(bc, i, gamma, t, u);
    F o[8];
    load8(W + p * 8, o);
    dtp = store_node<F>(n, p, u, o, want_dt != 0, vol, aux, gamma, U, W);
  }
  if (want_dt) block_min_atomic(dtp, dtmin);
}

// CFL minimum over all nodes of the current state.
__global__ void __launch_bounds__(kBlock) k_dt(int64_t n, const double* __restrict__ U,
                                                const double* __restrict__ vol, double gamma,
                                                unsigned long long* dtmin) {
  int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  double dtp = DBL_MAX;
  if (p < n) {
    double u[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) u[c] = U[c * n + p];
    dtp = node_dt(u, vol[p], gamma);
  }
  block_min_atomic(dtp, dtmin);
}

// The same minimum with the FP32-mode formula of the step epilogue
// (node_dt_f: FP32 arithmetic on the FP64 state, cbrt(vol) given), so that
// a state set from the host gets the dt the time loop itself would form.
__global__ void __launch_bounds__(kBlock) k_dt_f(int64_t n, const double* __restrict__ U,
                                                  const float* __restrict__ cbrtv, double gamma,
                                                  unsigned long long* dtmin) {
  int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  double dtp = DBL_MAX;
  if (p < n) {
    double u[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) u[c] = U[c * n + p];
    dtp = double(node_dt_f(u, cbrtv[p], float(gamma)));
  }
  block_min_atomic(dtp, dtmin);
}

// Step prologue (RieCG::dt reduction target + RieCG::advance,
// src/Inciter/RieCG.cpp:839-869): dt = cfl * min, blowup when dt < eps; then
// reset the running minimum for the next step.
__global__ void k_step_begin(Scalars* s, double cfl, double const_dt, double* hist) {
  const long long k = s->step;
  s->step = k + 1;
  s->t = s->tnext;
  double dt;
  if (fabs(const_dt) > DBL_EPSILON)
    dt = const_dt;
  else
    dt = __longlong_as_double(s->dtmin) * cfl;
  if (dt < DBL_EPSILON) s->blowup = 1;
  s->dt = dt;
  s->tnext = s->t + dt;
  s->dtmin = __double_as_longlong(DBL_MAX);
  if (hist) hist[k] = dt;
}

__global__ void k_set_dt(Scalars* s, double dt) { s->dt = dt; }
// The time of the next step to start (and of drop-in residuals): t.
__global__ void k_set_time(Scalars* s, double t) {
  s->t = t;
  s->tnext = t;
}
__global__ void k_reset_min(Scalars* s) { s->dtmin = __double_as_longlong(DBL_MAX); }

}  // namespace

// ---------------------------------------------------------------------------
// host side

namespace {

struct Edge {
  int64_t a, b;
  double d[3];
};

struct HalfLists {
  std::vector<int32_t> soff1, sw1, soff2, sw2, q1, pos1;
  std::vector<double> d1;
  int64_t nent1 = 0, nent2 = 0;
};

int launch_done(xg_ctx* c, RieCGDev* d, int slot, cudaEvent_t e0) {
  if (!d->prof) return XG_OK;
  cudaEvent_t e1;
  XG_CUDA(c, cudaEventCreate(&e1));
  XG_CUDA(c, cudaEventRecord(e1, c->stream));
  d->pending.push_back({slot, {e0, e1}});
  return XG_OK;
}

int launch_begin(xg_ctx* c, RieCGDev* d, const char* name, int* slot, cudaEvent_t* e0) {
  if (!d->prof) return XG_OK;
  int k = -1;
  for (size_t i = 0; i < d->ktimes.size(); ++i)
    if (std::strcmp(d->ktimes[i].name, name) == 0) k = static_cast<int>(i);
  if (k < 0) {
    d->ktimes.push_back({name, 0.0, 0});
    k = static_cast<int>(d->ktimes.size() - 1);
  }
  *slot = k;
  XG_CUDA(c, cudaEventCreate(e0));
  XG_CUDA(c, cudaEventRecord(*e0, c->stream));
  return XG_OK;
}

int flush_profile(xg_ctx* c, RieCGDev* d) {
  if (d->pending.empty()) return XG_OK;
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  for (auto& p : d->pending) {
    float ms = 0.f;
    XG_CUDA(c, cudaEventElapsedTime(&ms, p.second.first, p.second.second));
    d->ktimes[p.first].ms += ms;
    d->ktimes[p.first].launches += 1;
    cudaEventDestroy(p.second.first);
    cudaEventDestroy(p.second.second);
  }
  d->pending.clear();
  return XG_OK;
}

#define XG_PROF_LAUNCH(ctx, dev, name, launch)                   \
  do {                                                           \
    int slot_ = 0;                                               \
    cudaEvent_t e0_ = nullptr;                                   \
    int rc_ = launch_begin(ctx, dev, name, &slot_, &e0_);        \
    if (rc_) return rc_;                                         \
    launch;                                                      \
    XG_CHECK_LAUNCH(ctx);                                        \
    rc_ = launch_done(ctx, dev, slot_, e0_);                     \
    if (rc_) return rc_;                                         \
  } while (0)

template <class F>
Adj<F> adj_of(RieCGDev* d) {
  return Adj<F>{d->soff, d->swidth, static_cast<const typename EntOf<F>::type*>(d->ent)};
}
NodeAux aux_of(RieCGDev* d) { return NodeAux{d->ivol, d->cbrtv}; }
// s V per node when a manufactured source is on, else null
template <class F>
const F* src_of(RieCGDev* d) {
  return d->src.problem != XG_SRC_NONE ? static_cast<const F*>(d->Sv) : nullptr;
}
// Evaluate s V at the device's current step time (scal->t) from records W.
template <class F>
int launch_src(xg_ctx* c, RieCGDev* d, const F* W) {
  if (d->src.problem == XG_SRC_NONE) return XG_OK;
  XG_PROF_LAUNCH(c, d, "riecg_src",
                 (k_src<F><<<blocks_for(d->n, kBlock), kBlock, 0, c->stream>>>(
                     d->n, d->src, d->scal, W, d->vol, static_cast<F*>(d->Sv))));
  return XG_OK;
}
Bnd bnd_of(RieCGDev* d) { return Bnd{d->bnode, d->bidx, d->bptr, d->bent4}; }

BCProg bcprog_of(RieCGDev* d) {
  BCProg b;
  b.nbc = d->nbc;
  b.node = d->bcnode;
  b.dir = d->bcdir;
  b.symp = d->bcsymp;
  b.far = d->bcfar;
  b.pre = d->bcpre;
  b.dirmask = d->dirmask;
  b.dirval = d->dirval;
  b.symn = d->symn;
  b.farn = d->farn;
  b.preval = d->preval;
  for (int i = 0; i < 5; ++i) b.far5[i] = d->far5[i];
  b.prob = d->src;
  b.dirxyz = d->dirxyz;
  return b;
}

template <class F>
int launch_grad(xg_ctx* c, RieCGDev* d, const F* W, F* G, int divide) {
  XG_PROF_LAUNCH(c, d, "riecg_grad",
                 (k_grad<F><<<blocks_for(d->n, GradShape<F>::BLOCK), GradShape<F>::BLOCK, 0,
                                c->stream>>>(
                     d->n, adj_of<F>(d), W, bnd_of(d), d->vol, aux_of(d), divide, G)));
  if (d->nbn > 0)
    XG_PROF_LAUNCH(c, d, "riecg_grad_bnd",
                   (k_grad_bnd<F><<<blocks_for(d->nbn, kBlock), kBlock, 0, c->stream>>>(
                       d->nbn, bnd_of(d), W, d->vol, aux_of(d), divide, G)));
  return XG_OK;
}

template <class F>
Half<F> half_of(RieCGDev* d) {
  return Half<F>{d->soff1, d->sw1, static_cast<const typename EntOf<F>::type*>(d->ent1),
                 d->pos1, d->soff2, d->sw2, d->nent2};
}

template <class F, int FLUX, int STAGE, bool UPDATE, bool LEAN>
int launch_rhs_t(xg_ctx* c, RieCGDev* d, const F* W, const F* G, F* Wout, double* Rout) {
  F* fbuf = static_cast<F*>(d->fbuf);
  F* Rp = static_cast<F*>(d->Rp);
  XG_PROF_LAUNCH(c, d, "riecg_flux",
                 (k_flux1<F, FLUX><<<blocks_for(d->n, kBlock), kBlock, 0, c->stream>>>(
                     d->n, half_of<F>(d), W, G, d->prm.gamma, d->prm.stab2, d->prm.stab2coef,
                     fbuf, Rp)));
  XG_PROF_LAUNCH(c, d, "riecg_rhs_update",
                 (k_rhs2<F, STAGE, UPDATE, LEAN><<<blocks_for(d->n, kBlock), kBlock, 0, c->stream>>>(
                     d->n, half_of<F>(d), fbuf, Rp, W, bnd_of(d), d->nbn,
                     static_cast<F*>(d->Rb), d->vol, aux_of(d), d->prm.gamma, d->scal, d->U,
                     d->Un, Wout, Rout, &d->scal->dtmin, src_of<F>(d))));
  if (d->nbn > 0)
    XG_PROF_LAUNCH(c, d, "riecg_rhs_bnd",
                   (k_rhs_bnd<F, STAGE, UPDATE, LEAN><<<blocks_for(d->nbn, kBlock), kBlock, 0,
                                                        c->stream>>>(
                       d->n, d->nbn, bnd_of(d), static_cast<const F*>(d->Rb), W, d->bcof,
                       bcprog_of(d), d->vol, aux_of(d), d->prm.gamma, d->scal, d->U, d->Un,
                       Wout, Rout, &d->scal->dtmin, src_of<F>(d))));
  return XG_OK;
}

template <class F, int FLUX>
int launch_rhs_f(xg_ctx* c, RieCGDev* d, int stage, bool update, bool lean, const F* W,
                 const F* G, F* Wout, double* Rout) {
  if (!update) return launch_rhs_t<F, FLUX, 0, false, false>(c, d, W, G, Wout, Rout);
  if (lean) {
    if (stage == 0) return launch_rhs_t<F, FLUX, 0, true, true>(c, d, W, G, Wout, Rout);
    if (stage == 1) return launch_rhs_t<F, FLUX, 1, true, true>(c, d, W, G, Wout, Rout);
    return launch_rhs_t<F, FLUX, 2, true, true>(c, d, W, G, Wout, Rout);
  }
  if (stage == 0) return launch_rhs_t<F, FLUX, 0, true, false>(c, d, W, G, Wout, Rout);
  if (stage == 1) return launch_rhs_t<F, FLUX, 1, true, false>(c, d, W, G, Wout, Rout);
  return launch_rhs_t<F, FLUX, 2, true, false>(c, d, W, G, Wout, Rout);
}

// The residual pass; with update, also the stage update (lean: the time
// loop's form, see store_stage).
template <class F>
int launch_rhs(xg_ctx* c, RieCGDev* d, int stage, bool update, bool lean, const F* W, const F* G,
               F* Wout, double* Rout) {
  if (d->prm.flux == XG_HLLC)
    return launch_rhs_f<F, XG_HLLC>(c, d, stage, update, lean, W, G, Wout, Rout);
  return launch_rhs_f<F, XG_RUSANOV>(c, d, stage, update, lean, W, G, Wout, Rout);
}

template <class F>
int launch_bc(xg_ctx* c, RieCGDev* d, F* W, int want_dt) {
  if (d->nbc == 0) return XG_OK;
  XG_PROF_LAUNCH(c, d, "riecg_bc",
                 (k_bc<F><<<blocks_for(d->nbc, kBlock), kBlock, 0, c->stream>>>(
                     d->n, bcprog_of(d), d->prm.gamma, d->U, W, d->vol, aux_of(d), d->t, want_dt,
                     &d->scal->dtmin)));
  return XG_OK;
}

// One stage on the device state.  lean: the time loop's form (U holds the
// state at the start of the step and only the last stage writes it);
// otherwise every stage's state lands in U (stage 0 copying U to Un first).
template <class F>
int do_stage(xg_ctx* c, RieCGDev* d, int stage, bool lean) {
  F* Win = static_cast<F*>(d->W[d->cur]);
  F* Wout = static_cast<F*>(d->W[d->cur ^ 1]);
  F* G = static_cast<F*>(d->G);
  int rc = launch_grad<F>(c, d, Win, G, 1);
  if (rc) return rc;
  // the residual pass updates every node and applies the nodal BCs of the
  // boundary nodes (all BC nodes) after their update
  rc = launch_rhs<F>(c, d, stage, true, lean, Win, G, Wout, nullptr);
  if (rc) return rc;
  d->cur ^= 1;
  return XG_OK;
}

int refresh_dt(xg_ctx* c, RieCGDev* d) {
  k_reset_min<<<1, 1, 0, c->stream>>>(d->scal);
  XG_CHECK_LAUNCH(c);
  if (d->fp32)
    k_dt_f<<<blocks_for(d->n, kBlock), kBlock, 0, c->stream>>>(d->n, d->U, d->cbrtv,
                                                                d->prm.gamma, &d->scal->dtmin);
  else
    k_dt<<<blocks_for(d->n, kBlock), kBlock, 0, c->stream>>>(d->n, d->U, d->vol, d->prm.gamma,
                                                              &d->scal->dtmin);
  XG_CHECK_LAUNCH(c);
  d->dt_valid = true;
  return XG_OK;
}

template <class F>
int alloc_and_upload(xg_ctx* c, RieCGDev* d, const double* coord, const double* vol,
                     const std::vector<int32_t>& soff, const std::vector<int32_t>& swidth,
                     const std::vector<int32_t>& nbr, const std::vector<double>& ddx,
                     const std::vector<double>& ddy, const std::vector<double>& ddz,
                     const std::vector<int32_t>& bidx, const std::vector<int32_t>& bptr,
                     const std::vector<int4>& bent4, const HalfLists& hl) {
  const int64_t n = d->n;
  using EntT = typename EntOf<F>::type;
  F *W0, *W1, *G, *fbuf, *Rp, *Rb;
  EntT *ent, *ent1;
  for (int pass = 0; pass < 2; ++pass) {
    Arena& A = d->arena;
    A.plan(d->U, n * 5);
    A.plan(d->Un, n * 5);
    A.plan(d->vol, n);
    A.plan(d->bidx, n);
    A.plan(W0, n * 8);
    A.plan(W1, n * 8);
    A.plan(G, n * 16);
    A.plan(d->soff, soff.size());
    A.plan(d->swidth, swidth.size());
    A.plan(ent, nbr.size());
    A.plan(d->soff1, hl.soff1.size());
    A.plan(d->sw1, hl.sw1.size());
    A.plan(d->soff2, hl.soff2.size());
    A.plan(d->sw2, hl.sw2.size());
    A.plan(d->pos1, std::max<int64_t>(1, hl.nent1));
    A.plan(ent1, std::max<int64_t>(1, hl.nent1));
    A.plan(fbuf, std::max<int64_t>(1, hl.nent2) * 5);
    A.plan(Rp, n * 5);
    A.plan(d->ivol, n);
    A.plan(d->cbrtv, n);
    A.plan(d->bptr, bptr.size());
    A.plan(d->bent4, std::max<size_t>(1, bent4.size()));
    A.plan(d->bcof, std::max<int64_t>(1, d->nbn));
    A.plan(d->bnode, std::max<int64_t>(1, d->nbn));
    A.plan(Rb, std::max<int64_t>(1, d->nbn) * 5);
    A.plan(d->scal, 1);
    if (pass == 0) XG_CUDA(c, A.reserve());
  }
  d->Rb = Rb;
  for (int pass = 0; pass < 2; ++pass) {
    Arena& S = d->scratch;
    S.plan(d->stage_buf, n * 15);
    F* sw;
    F* sg;
    S.plan(sw, n * 8);
    S.plan(sg, n * 16);
    d->stage_W = sw;
    d->stage_G = sg;
    if (pass == 0) XG_CUDA(c, S.reserve());
  }
  d->W[0] = W0;
  d->W[1] = W1;
  d->G = G;
  d->ent = ent;
  d->ent1 = ent1;
  d->fbuf = fbuf;
  d->Rp = Rp;
  d->nent1 = hl.nent1;
  d->nent2 = hl.nent2;
  cudaStream_t s = c->stream;
  auto up = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
    return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s) : cudaSuccess;
  };
  XG_CUDA(c, up(d->vol, vol, n * sizeof(double)));
  XG_CUDA(c, up(d->bidx, bidx.data(), n * sizeof(int32_t)));
  XG_CUDA(c, up(d->soff, soff.data(), soff.size() * 4));
  XG_CUDA(c, up(d->swidth, swidth.data(), swidth.size() * 4));
  {
    std::vector<EntT> h(nbr.size());
    for (size_t i = 0; i < h.size(); ++i) {
      if constexpr (sizeof(F) == 4) {
        float fx = float(ddx[i]), fy = float(ddy[i]), fz = float(ddz[i]);
        int4 v;
        v.x = nbr[i];
        std::memcpy(&v.y, &fx, 4);
        std::memcpy(&v.z, &fy, 4);
        std::memcpy(&v.w, &fz, 4);
        h[i] = v;
      } else {
        h[i].dx = ddx[i];
        h[i].dy = ddy[i];
        h[i].dz = ddz[i];
        h[i].q = nbr[i];
        h[i].pad = 0;
      }
    }
    XG_CUDA(c, cudaMemcpy(ent, h.data(), h.size() * sizeof(EntT), cudaMemcpyHostToDevice));
    std::vector<EntT> h1(hl.nent1);
    for (int64_t i = 0; i < hl.nent1; ++i) {
      if constexpr (sizeof(F) == 4) {
        float fx = float(hl.d1[i * 3]), fy = float(hl.d1[i * 3 + 1]), fz = float(hl.d1[i * 3 + 2]);
        int4 v;
        v.x = hl.q1[i];
        std::memcpy(&v.y, &fx, 4);
        std::memcpy(&v.z, &fy, 4);
        std::memcpy(&v.w, &fz, 4);
        h1[i] = v;
      } else {
        h1[i].dx = hl.d1[i * 3];
        h1[i].dy = hl.d1[i * 3 + 1];
        h1[i].dz = hl.d1[i * 3 + 2];
        h1[i].q = hl.q1[i];
        h1[i].pad = 0;
      }
    }
    XG_CUDA(c, up(ent1, h1.data(), h1.size() * sizeof(EntT)));
    XG_CUDA(c, up(d->soff1, hl.soff1.data(), hl.soff1.size() * 4));
    XG_CUDA(c, up(d->sw1, hl.sw1.data(), hl.sw1.size() * 4));
    XG_CUDA(c, up(d->soff2, hl.soff2.data(), hl.soff2.size() * 4));
    XG_CUDA(c, up(d->sw2, hl.sw2.data(), hl.sw2.size() * 4));
    XG_CUDA(c, up(d->pos1, hl.pos1.data(), hl.pos1.size() * 4));
    // list-2 padding slots are never written and must read as zero
    XG_CUDA(c, cudaMemsetAsync(fbuf, 0, std::max<int64_t>(1, hl.nent2) * 5 * sizeof(F), s));
    XG_CUDA(c, cudaStreamSynchronize(s));
    std::vector<double> iv(n);
    std::vector<float> cv(n);
    for (int64_t i = 0; i < n; ++i) {
      iv[i] = 1.0 / vol[i];
      cv[i] = static_cast<float>(std::cbrt(vol[i]));
    }
    XG_CUDA(c, cudaMemcpy(d->ivol, iv.data(), n * sizeof(double), cudaMemcpyHostToDevice));
    XG_CUDA(c, cudaMemcpy(d->cbrtv, cv.data(), n * sizeof(float), cudaMemcpyHostToDevice));
  }
  std::vector<int32_t> bnode(std::max<int64_t>(1, d->nbn), 0);
  for (int64_t p = 0; p < n; ++p)
    if (bidx[p] >= 0) bnode[bidx[p]] = static_cast<int32_t>(p);
  XG_CUDA(c, cudaMemcpy(d->bnode, bnode.data(), bnode.size() * 4, cudaMemcpyHostToDevice));
  XG_CUDA(c, up(d->bptr, bptr.data(), bptr.size() * 4));
  XG_CUDA(c, up(d->bent4, bent4.data(), bent4.size() * sizeof(int4)));
  XG_CUDA(c, cudaMemsetAsync(d->bcof, 0xff, std::max<int64_t>(1, d->nbn) * 4, s));  // -1
  XG_CUDA(c, cudaMemsetAsync(d->U, 0, n * 5 * sizeof(double), s));
  XG_CUDA(c, cudaMemsetAsync(d->Un, 0, n * 5 * sizeof(double), s));
  XG_CUDA(c, cudaMemsetAsync(G, 0, n * 16 * sizeof(F), s));
  {
    // W records: zero primitives, coordinates in slots 5..7
    std::vector<F> w(n * 8, F(0));
    for (int64_t p = 0; p < n; ++p) {
      w[p * 8 + 5] = F(coord[p]);
      w[p * 8 + 6] = F(coord[n + p]);
      w[p * 8 + 7] = F(coord[2 * n + p]);
    }
    XG_CUDA(c, cudaMemcpy(W0, w.data(), w.size() * sizeof(F), cudaMemcpyHostToDevice));
    XG_CUDA(c, cudaMemcpy(W1, w.data(), w.size() * sizeof(F), cudaMemcpyHostToDevice));
    XG_CUDA(c, cudaMemcpy(d->stage_W, w.data(), w.size() * sizeof(F), cudaMemcpyHostToDevice));
  }
  Scalars s0{};  // every member zero
  double big = DBL_MAX;
  std::memcpy(&s0.dtmin, &big, sizeof(double));
  XG_CUDA(c, cudaMemcpy(d->scal, &s0, sizeof(s0), cudaMemcpyHostToDevice));
  XG_CUDA(c, cudaStreamSynchronize(s));
  return XG_OK;
}

}  // namespace

}  // namespace xg

using namespace xg;

extern "C" {

int xg_riecg_setup(xg_ctx* c, const xg_riecg_params* prm, int64_t npoin, const double* coord,
                   const double* vol, int64_t ntet, const uint64_t* dsupedge0,
                   const double* dsupint0, int64_t ntri, const uint64_t* dsupedge1,
                   const double* dsupint1, int64_t nedge, const uint64_t* dsupedge2,
                   const double* dsupint2, int64_t nbtri, const uint64_t* triinpoel,
                   const uint8_t* besym) {
  XG_HOST_TRY
  int rc = use(c);
  if (rc) return rc;
  if (!prm || npoin <= 0 || !coord || !vol) return fail(c, XG_ERR_ARG, "riecg_setup: bad mesh");
  if (npoin >= (int64_t(1) << 31) - 64) return fail(c, XG_ERR_ARG, "riecg_setup: too many nodes");
  if (prm->flux != XG_RUSANOV && prm->flux != XG_HLLC)
    return fail(c, XG_ERR_ARG, "Flux not configured");
  if (prm->precision != XG_FP64 && prm->precision != XG_FP32_FLUX)
    return fail(c, XG_ERR_ARG, "riecg_setup: unknown precision");
  if ((ntet && (!dsupedge0 || !dsupint0)) || (ntri && (!dsupedge1 || !dsupint1)) ||
      (nedge && (!dsupedge2 || !dsupint2)) || (nbtri && (!triinpoel || !besym)))
    return fail(c, XG_ERR_ARG, "riecg_setup: null superedge or boundary array");
  // Expand superedges into edges in the orientation RieCG evaluates them
  // (tet group: lpoed order (0,1),(1,2),(2,0),(0,3),(1,3),(2,3); triangle
  // group: (0,1),(1,2),(2,0); src/Physics/Riemann.cpp:706-753).
  std::vector<Edge> E;
  E.reserve(static_cast<size_t>(ntet * 6 + ntri * 3 + nedge));
  static const int tp[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
  static const int rp[3][2] = {{0, 1}, {1, 2}, {2, 0}};
  auto bad = [&](uint64_t id) { return id >= static_cast<uint64_t>(npoin); };
  for (int64_t e = 0; e < ntet; ++e) {
    const uint64_t* N = dsupedge0 + e * 4;
    for (int k = 0; k < 6; ++k) {
      if (bad(N[tp[k][0]]) || bad(N[tp[k][1]])) return fail(c, XG_ERR_ARG, "tet superedge id");
      const double* dd = dsupint0 + (e * 6 + k) * 3;
      E.push_back({int64_t(N[tp[k][0]]), int64_t(N[tp[k][1]]), {dd[0], dd[1], dd[2]}});
    }
  }
  for (int64_t e = 0; e < ntri; ++e) {
    const uint64_t* N = dsupedge1 + e * 3;
    for (int k = 0; k < 3; ++k) {
      if (bad(N[rp[k][0]]) || bad(N[rp[k][1]])) return fail(c, XG_ERR_ARG, "tri superedge id");
      const double* dd = dsupint1 + (e * 3 + k) * 3;
      E.push_back({int64_t(N[rp[k][0]]), int64_t(N[rp[k][1]]), {dd[0], dd[1], dd[2]}});
    }
  }
  for (int64_t e = 0; e < nedge; ++e) {
    const uint64_t* N = dsupedge2 + e * 2;
    if (bad(N[0]) || bad(N[1])) return fail(c, XG_ERR_ARG, "edge id");
    const double* dd = dsupint2 + e * 3;
    E.push_back({int64_t(N[0]), int64_t(N[1]), {dd[0], dd[1], dd[2]}});
  }
  const int64_t n = npoin;
  // per node degree, then entries sorted by neighbour id
  std::vector<int64_t> deg(n + 1, 0);
  for (auto& e : E) {
    if (e.a == e.b) return fail(c, XG_ERR_ARG, "degenerate edge");
    ++deg[e.a + 1];
    ++deg[e.b + 1];
  }
  std::vector<int64_t> start(deg);
  for (int64_t i = 0; i < n; ++i) start[i + 1] += start[i];
  struct Ent {
    int64_t q;
    int64_t eid;
    bool first;
  };
  std::vector<Ent> ent(static_cast<size_t>(start[n]));
  {
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    for (size_t k = 0; k < E.size(); ++k) {
      ent[fill[E[k].a]++] = {E[k].b, int64_t(k), true};
      ent[fill[E[k].b]++] = {E[k].a, int64_t(k), false};
    }
  }
  for (int64_t p = 0; p < n; ++p)
    std::sort(ent.begin() + start[p], ent.begin() + start[p + 1],
              [](const Ent& x, const Ent& y) { return x.q < y.q || (x.q == y.q && x.eid < y.eid); });
  // SELL-32 slices
  const int64_t nslice = (n + kSlice - 1) / kSlice;
  std::vector<int32_t> soff(nslice + 1), swidth(nslice);
  int64_t total = 0;
  for (int64_t s = 0; s < nslice; ++s) {
    int64_t w = 0;
    for (int64_t p = s * kSlice; p < std::min(n, (s + 1) * kSlice); ++p)
      w = std::max<int64_t>(w, start[p + 1] - start[p]);
    swidth[s] = static_cast<int32_t>(w);
    soff[s] = static_cast<int32_t>(total);
    total += w * kSlice;
    if (total >= (int64_t(1) << 31)) return fail(c, XG_ERR_ARG, "adjacency too large");
  }
  soff[nslice] = static_cast<int32_t>(total);
  std::vector<int32_t> nbr(static_cast<size_t>(total), kPad);
  std::vector<double> ddx(nbr.size(), 0.0), ddy(nbr.size(), 0.0), ddz(nbr.size(), 0.0);
  for (int64_t p = 0; p < n; ++p) {
    const int64_t s = p / kSlice, lane = p % kSlice;
    for (int64_t k = 0; k < start[p + 1] - start[p]; ++k) {
      const Ent& en = ent[start[p] + k];
      const int64_t idx = soff[s] + k * kSlice + lane;
      nbr[idx] = en.first ? static_cast<int32_t>(en.q) : ~static_cast<int32_t>(en.q);
      ddx[idx] = E[en.eid].d[0];
      ddy[idx] = E[en.eid].d[1];
      ddz[idx] = E[en.eid].d[2];
    }
  }
  // half-edge lists: every edge is owned by its end with the smaller local
  // id (with locality ordering that splits each node's edges about evenly);
  // the owner's entry (list 1) holds the other end (~id when the owner is the
  // canonical second end), D and the position of the edge in the other end's
  // list 2, where the owner deposits that end's signed flux
  HalfLists hl;
  {
    std::vector<int64_t> c1(n + 1, 0), c2(n + 1, 0);
    auto own = [&](const Edge& e) { return std::min(e.a, e.b); };
    auto oth = [&](const Edge& e) { return std::max(e.a, e.b); };
    for (auto& e : E) {
      ++c1[own(e) + 1];
      ++c2[oth(e) + 1];
    }
    for (int64_t i = 0; i < n; ++i) {
      c1[i + 1] += c1[i];
      c2[i + 1] += c2[i];
    }
    std::vector<int64_t> l1(E.size()), l2(E.size());
    {
      std::vector<int64_t> f1(c1.begin(), c1.end() - 1), f2(c2.begin(), c2.end() - 1);
      for (size_t k = 0; k < E.size(); ++k) {
        l1[f1[own(E[k])]++] = int64_t(k);
        l2[f2[oth(E[k])]++] = int64_t(k);
      }
    }
    for (int64_t p = 0; p < n; ++p) {
      std::sort(l1.begin() + c1[p], l1.begin() + c1[p + 1], [&](int64_t x, int64_t y) {
        return oth(E[x]) < oth(E[y]) || (oth(E[x]) == oth(E[y]) && x < y);
      });
      std::sort(l2.begin() + c2[p], l2.begin() + c2[p + 1], [&](int64_t x, int64_t y) {
        return own(E[x]) < own(E[y]) || (own(E[x]) == own(E[y]) && x < y);
      });
    }
    auto sell = [&](const std::vector<int64_t>& cnt, std::vector<int32_t>& off,
                    std::vector<int32_t>& wid, int64_t& total) -> bool {
      off.assign(nslice + 1, 0);
      wid.assign(nslice, 0);
      total = 0;
      for (int64_t s2 = 0; s2 < nslice; ++s2) {
        int64_t w = 0;
        for (int64_t p = s2 * kSlice; p < std::min(n, (s2 + 1) * kSlice); ++p)
          w = std::max<int64_t>(w, cnt[p + 1] - cnt[p]);
        wid[s2] = static_cast<int32_t>(w);
        off[s2] = static_cast<int32_t>(total);
        total += w * kSlice;
        if (total >= (int64_t(1) << 31)) return false;
      }
      off[nslice] = static_cast<int32_t>(total);
      return true;
    };
    if (!sell(c1, hl.soff1, hl.sw1, hl.nent1) || !sell(c2, hl.soff2, hl.sw2, hl.nent2))
      return fail(c, XG_ERR_ARG, "adjacency too large");
    hl.q1.assign(hl.nent1, kPad);
    hl.d1.assign(hl.nent1 * 3, 0.0);
    hl.pos1.assign(hl.nent1, kPad);
    std::vector<int32_t> slot1(E.size(), -1);
    for (int64_t p = 0; p < n; ++p) {
      const int64_t s2 = p / kSlice, lane = p % kSlice;
      for (int64_t k = 0; k < c1[p + 1] - c1[p]; ++k) {
        const int64_t eid = l1[c1[p] + k];
        const int64_t idx = hl.soff1[s2] + k * kSlice + lane;
        const int32_t q = static_cast<int32_t>(oth(E[eid]));
        hl.q1[idx] = (E[eid].a == p) ? q : ~q;
        for (int a = 0; a < 3; ++a) hl.d1[idx * 3 + a] = E[eid].d[a];
        slot1[eid] = static_cast<int32_t>(idx);
      }
    }
    for (int64_t p = 0; p < n; ++p) {
      const int64_t s2 = p / kSlice, lane = p % kSlice;
      for (int64_t k = 0; k < c2[p + 1] - c2[p]; ++k) {
        const int64_t eid = l2[c2[p] + k];
        hl.pos1[slot1[eid]] = static_cast<int32_t>(hl.soff2[s2] + k * kSlice + lane);
      }
    }
  }
  // boundary triangles: per boundary node, the (tri, position) pairs
  std::vector<int32_t> bidx(n, -1), btri(nbtri * 3);
  std::vector<uint8_t> bsym(nbtri * 3);
  std::vector<int64_t> bcount;
  int64_t nbn = 0;
  for (int64_t t = 0; t < nbtri; ++t)
    for (int a = 0; a < 3; ++a) {
      uint64_t p = triinpoel[t * 3 + a];
      if (bad(p)) return fail(c, XG_ERR_ARG, "triinpoel id");
      btri[t * 3 + a] = static_cast<int32_t>(p);
      bsym[t * 3 + a] = besym[t * 3 + a] ? 1 : 0;
      if (bidx[p] < 0) {
        bidx[p] = static_cast<int32_t>(nbn++);
        bcount.push_back(0);
      }
      ++bcount[bidx[p]];
    }
  std::vector<int32_t> bptr(nbn + 1, 0);
  std::vector<int4> bent4(nbtri * 3);
  for (int64_t i = 0; i < nbn; ++i) bptr[i + 1] = bptr[i] + static_cast<int32_t>(bcount[i]);
  {
    std::vector<int32_t> fill(bptr.begin(), bptr.end() - 1);
    for (int64_t t = 0; t < nbtri; ++t)
      for (int a = 0; a < 3; ++a) {
        int32_t bi = bidx[triinpoel[t * 3 + a]];
        const int32_t flags = a | (bsym[t * 3] << 2) | (bsym[t * 3 + 1] << 3) |
                              (bsym[t * 3 + 2] << 4);
        bent4[fill[bi]++] = make_int4(btri[t * 3], btri[t * 3 + 1], btri[t * 3 + 2], flags);
      }
  }
  // (re)create the device state
  if (c->riecg) {
    XG_CUDA(c, cudaStreamSynchronize(c->stream));
    destroy_riecg(c->riecg);
    c->riecg = nullptr;
  }
  auto* d = new RieCGDev;
  c->riecg = d;
  d->n = n;
  d->prm = *prm;
  d->fp32 = prm->precision == XG_FP32_FLUX;
  d->nslice = nslice;
  d->nent = total;
  d->nbn = nbn;
  d->nbt = nbtri;
  d->nbent = nbtri * 3;
  d->xyz_host.assign(coord, coord + 3 * n);
  if (d->fp32)
    rc = alloc_and_upload<float>(c, d, coord, vol, soff, swidth, nbr, ddx, ddy, ddz, bidx, bptr,
                                 bent4, hl);
  else
    rc = alloc_and_upload<double>(c, d, coord, vol, soff, swidth, nbr, ddx, ddy, ddz, bidx, bptr,
                                  bent4, hl);
  if (rc) {
    destroy_riecg(d);
    c->riecg = nullptr;
    return rc;
  }
  // bidx is also needed on the host to set BC flags later
  return XG_OK;
  XG_HOST_CATCH(c)
}

int xg_riecg_set_bc(xg_ctx* c, int64_t nsym, const uint64_t* symnodes, const double* symnorms,
                    int64_t nfar, const uint64_t* farnodes, const double* farnorms,
                    const double* far5, int64_t ndir, const uint64_t* dirnodes,
                    const int32_t* dirmask, const double* dirvals, int64_t npre,
                    const uint64_t* prenodes, const double* prevals) {
  XG_HOST_TRY
  int rc = use(c);
  if (rc) return rc;
  RieCGDev* d = c->riecg;
  if (!d) return fail(c, XG_ERR_STATE, "riecg_set_bc before riecg_setup");
  const int64_t n = d->n;
  auto chk = [&](int64_t cnt, const uint64_t* ids) {
    for (int64_t i = 0; i < cnt; ++i)
      if (ids[i] >= static_cast<uint64_t>(n)) return false;
    return true;
  };
  if ((nsym && (!symnodes || !symnorms)) || (nfar && (!farnodes || !farnorms || !far5)) ||
      (ndir && (!dirnodes || !dirmask || !dirvals)) || (npre && (!prenodes || !prevals)))
    return fail(c, XG_ERR_ARG, "riecg_set_bc: null array");
  if (!chk(nsym, symnodes) || !chk(nfar, farnodes) || !chk(ndir, dirnodes) || !chk(npre, prenodes))
    return fail(c, XG_ERR_ARG, "riecg_set_bc: node id out of range");
  // unique BC nodes in increasing id order, each with its ops
  std::vector<int64_t> ids;
  ids.insert(ids.end(), symnodes, symnodes + nsym);
  ids.insert(ids.end(), farnodes, farnodes + nfar);
  ids.insert(ids.end(), dirnodes, dirnodes + ndir);
  ids.insert(ids.end(), prenodes, prenodes + npre);
  std::sort(ids.begin(), ids.end());
  ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
  const int64_t nbc = static_cast<int64_t>(ids.size());
  std::vector<int32_t> node(nbc), dir(nbc, -1), far(nbc, -1), pre(nbc, -1), symp(nbc + 1, 0);
  auto pos = [&](uint64_t p) {
    return static_cast<int64_t>(std::lower_bound(ids.begin(), ids.end(), int64_t(p)) - ids.begin());
  };
  for (int64_t i = 0; i < nbc; ++i) node[i] = static_cast<int32_t>(ids[i]);
  for (int64_t k = 0; k < ndir; ++k) dir[pos(dirnodes[k])] = static_cast<int32_t>(k);
  for (int64_t k = 0; k < nfar; ++k) far[pos(farnodes[k])] = static_cast<int32_t>(k);
  for (int64_t k = 0; k < npre; ++k) pre[pos(prenodes[k])] = static_cast<int32_t>(k);
  // symmetry normals grouped per node, keeping the given order within a node
  std::vector<int64_t> cnt(nbc, 0);
  for (int64_t k = 0; k < nsym; ++k) ++cnt[pos(symnodes[k])];
  for (int64_t i = 0; i < nbc; ++i) symp[i + 1] = symp[i] + static_cast<int32_t>(cnt[i]);
  std::vector<double> symn(std::max<int64_t>(1, nsym) * 3, 0.0);
  {
    std::vector<int32_t> fill(symp.begin(), symp.end() - 1);
    for (int64_t k = 0; k < nsym; ++k) {
      int32_t j = fill[pos(symnodes[k])]++;
      for (int a = 0; a < 3; ++a) symn[j * 3 + a] = symnorms[k * 3 + a];
    }
  }
  // per boundary node: its BC program entry (the residual pass applies it)
  std::vector<int32_t> hbidx(n);
  XG_CUDA(c, cudaMemcpy(hbidx.data(), d->bidx, n * sizeof(int32_t), cudaMemcpyDeviceToHost));
  std::vector<int32_t> bcof(std::max<int64_t>(1, d->nbn), -1);
  for (int64_t i = 0; i < nbc; ++i) {
    int32_t bi = hbidx[ids[i]];
    if (bi < 0)
      return fail(c, XG_ERR_ARG, "riecg_set_bc: BC node not on a boundary triangle");
    bcof[bi] = static_cast<int32_t>(i);
  }
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  d->bcarena.release();
  for (int pass = 0; pass < 2; ++pass) {
    Arena& A = d->bcarena;
    A.plan(d->bcnode, std::max<int64_t>(1, nbc));
    A.plan(d->bcdir, std::max<int64_t>(1, nbc));
    A.plan(d->bcfar, std::max<int64_t>(1, nbc));
    A.plan(d->bcpre, std::max<int64_t>(1, nbc));
    A.plan(d->bcsymp, nbc + 1);
    A.plan(d->symn, symn.size());
    A.plan(d->dirmask, std::max<int64_t>(1, ndir) * 5);
    A.plan(d->dirval, std::max<int64_t>(1, ndir) * 5);
    A.plan(d->dirxyz, std::max<int64_t>(1, ndir) * 3);
    A.plan(d->farn, std::max<int64_t>(1, nfar) * 3);
    A.plan(d->preval, std::max<int64_t>(1, npre) * 2);
    if (pass == 0) XG_CUDA(c, A.reserve());
  }
  auto up = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
    return bytes ? cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) : cudaSuccess;
  };
  XG_CUDA(c, up(d->bcnode, node.data(), nbc * 4));
  XG_CUDA(c, up(d->bcdir, dir.data(), nbc * 4));
  XG_CUDA(c, up(d->bcfar, far.data(), nbc * 4));
  XG_CUDA(c, up(d->bcpre, pre.data(), nbc * 4));
  XG_CUDA(c, up(d->bcsymp, symp.data(), (nbc + 1) * 4));
  XG_CUDA(c, up(d->symn, symn.data(), symn.size() * 8));
  XG_CUDA(c, up(d->dirmask, dirmask, ndir * 5 * 4));
  XG_CUDA(c, up(d->dirval, dirvals, ndir * 5 * 8));
  {
    std::vector<double> dx(std::max<int64_t>(1, ndir) * 3, 0.0);
    for (int64_t k = 0; k < ndir; ++k)
      for (int j = 0; j < 3; ++j) dx[k * 3 + j] = d->xyz_host[j * d->n + dirnodes[k]];
    XG_CUDA(c, up(d->dirxyz, dx.data(), ndir * 3 * 8));
  }
  XG_CUDA(c, up(d->farn, farnorms, nfar * 3 * 8));
  XG_CUDA(c, up(d->preval, prevals, npre * 2 * 8));
  XG_CUDA(c, up(d->bcof, bcof.data(), bcof.size() * 4));
  if (far5)
    for (int i = 0; i < 5; ++i) d->far5[i] = far5[i];
  d->nbc = nbc;
  d->dt_valid = false;
  drop_graphs(d);
  return XG_OK;
  XG_HOST_CATCH(c)
}

int xg_riecg_set_state(xg_ctx* c, const double* U, double t) {
  int rc = use(c);
  if (rc) return rc;
  RieCGDev* d = c->riecg;
  if (!d) return fail(c, XG_ERR_STATE, "riecg_set_state before riecg_setup");
  if (!U) return fail(c, XG_ERR_ARG, "riecg_set_state: null U");
  // a pinned host buffer is read by k_state_in itself over the host link;
  // other memory goes through a staging copy
  const double* src = static_cast<const double*>(pinned_view(U));
  if (!src) {
    XG_CUDA(c, cudaMemcpyAsync(d->stage_buf, U, d->n * 5 * sizeof(double),
                               cudaMemcpyHostToDevice, c->stream));
    src = d->stage_buf;
  }
  // the state, its primitive records and its CFL minimum in one pass
  k_reset_min<<<1, 1, 0, c->stream>>>(d->scal);
  XG_CHECK_LAUNCH(c);
  if (d->fp32)
    k_state_in<float><<<blocks_for(d->n, kBlock), kBlock, 0, c->stream>>>(
        d->n, src, d->vol, aux_of(d), d->prm.gamma, d->U, static_cast<float*>(d->W[d->cur]),
        &d->scal->dtmin);
  else
    k_state_in<double><<<blocks_for(d->n, kBlock), kBlock, 0, c->stream>>>(
        d->n, src, d->vol, aux_of(d), d->prm.gamma, d->U, static_cast<double*>(d->W[d->cur]),
        &d->scal->dtmin);
  XG_CHECK_LAUNCH(c);
  d->t = t;
  d->dt_valid = true;
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}

int xg_riecg_get_state(xg_ctx* c, double* U, double* t) {
  int rc = use(c);
  if (rc) return rc;
  RieCGDev* d = c->riecg;
  if (!d) return fail(c, XG_ERR_STATE, "riecg_get_state before riecg_setup");
  if (U) {
    // into a pinned host buffer directly (coalesced stores over the host
    // link), otherwise through a staging copy
    double* dst = static_cast<double*>(pinned_view(U));
    k_soa_to_aos<<<blocks_for(d->n * 5, kBlock), kBlock, 0, c->stream>>>(
        d->n, 5, d->U, dst ? dst : d->stage_buf);
    XG_CHECK_LAUNCH(c);
    if (!dst)
      XG_CUDA(c, cudaMemcpyAsync(U, d->stage_buf, d->n * 5 * sizeof(double),
                                 cudaMemcpyDeviceToHost, c->stream));
  }
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (t) *t = d->t;
  return XG_OK;
}

}  // extern "C"

namespace {
template <class F>
int grad_dropin(xg_ctx* c, RieCGDev* d, const double* U, double* G) {
  F* W = static_cast<F*>(d->stage_W);
  F* Gr = static_cast<F*>(d->stage_G);
  XG_CUDA(c, cudaMemcpyAsync(d->stage_buf, U, d->n * 5 * sizeof(double), cudaMemcpyHostToDevice,
                             c->stream));
  k_prim_aos<F><<<blocks_for(d->n, kBlock), kBlock, 0, c->stream>>>(d->n, d->stage_buf, W, W);
  XG_CHECK_LAUNCH(c);
  int rc = launch_grad<F>(c, d, W, Gr, 0);
  if (rc) return rc;
  k_grec_to_aos<F><<<blocks_for(d->n * 15, kBlock), kBlock, 0, c->stream>>>(d->n, Gr, d->stage_buf);
  XG_CHECK_LAUNCH(c);
  XG_CUDA(c, cudaMemcpyAsync(G, d->stage_buf, d->n * 15 * sizeof(double), cudaMemcpyDeviceToHost,
                             c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}

template <class F>
int rhs_dropin(xg_ctx* c, RieCGDev* d, const double* G, const double* U, double* R) {
  F* W = static_cast<F*>(d->stage_W);
  F* Gr = static_cast<F*>(d->stage_G);
  XG_CUDA(c, cudaMemcpyAsync(d->stage_buf, G, d->n * 15 * sizeof(double), cudaMemcpyHostToDevice,
                             c->stream));
  k_aos_to_grec<F><<<blocks_for(d->n * 16, kBlock), kBlock, 0, c->stream>>>(d->n, d->stage_buf, Gr);
  XG_CHECK_LAUNCH(c);
  XG_CUDA(c, cudaMemcpyAsync(d->stage_buf, U, d->n * 5 * sizeof(double), cudaMemcpyHostToDevice,
                             c->stream));
  k_prim_aos<F><<<blocks_for(d->n, kBlock), kBlock, 0, c->stream>>>(d->n, d->stage_buf, W, W);
  XG_CHECK_LAUNCH(c);
  k_set_time<<<1, 1, 0, c->stream>>>(d->scal, d->t);
  XG_CHECK_LAUNCH(c);
  int rc = launch_src<F>(c, d, W);
  if (rc) return rc;
  rc = launch_rhs<F>(c, d, 0, false, false, W, Gr, nullptr, d->stage_buf);
  if (rc) return rc;
  XG_CUDA(c, cudaMemcpyAsync(R, d->stage_buf, d->n * 5 * sizeof(double), cudaMemcpyDeviceToHost,
                             c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}

// Greedy colouring of the owned edges (list 1, read back from the device):
// each edge, in owner order, takes the lowest colour neither end uses yet
// (at most 2 x max degree - 1 colours; 128 supported), then the edges are
// grouped by colour, owner order kept within a colour.
int build_colours(xg_ctx* c, RieCGDev* d) {
  if (!d->coff.empty()) return XG_OK;
  const int64_t n = d->n, nslice = (n + kSlice - 1) / kSlice;
  std::vector<int32_t> soff1(nslice + 1), sw1(nslice);
  std::vector<int4> e1(std::max<int64_t>(1, d->nent1));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  XG_CUDA(c, cudaMemcpy(soff1.data(), d->soff1, soff1.size() * 4, cudaMemcpyDeviceToHost));
  XG_CUDA(c, cudaMemcpy(sw1.data(), d->sw1, sw1.size() * 4, cudaMemcpyDeviceToHost));
  if (d->nent1)
    XG_CUDA(c, cudaMemcpy(e1.data(), d->ent1, d->nent1 * sizeof(int4), cudaMemcpyDeviceToHost));
  std::vector<int2> pq;
  std::vector<float4> dd;
  for (int64_t p = 0; p < n; ++p) {
    const int64_t s2 = p / kSlice, lane = p % kSlice;
    for (int64_t k = 0; k < sw1[s2]; ++k) {
      const int4 v = e1[soff1[s2] + k * kSlice + lane];
      if (v.x == kPad) continue;
      float x, y, z;
      std::memcpy(&x, &v.y, 4);
      std::memcpy(&y, &v.z, 4);
      std::memcpy(&z, &v.w, 4);
      const float sg = v.x >= 0 ? 1.f : -1.f;  // owner's orientation
      pq.push_back(make_int2(static_cast<int>(p), v.x >= 0 ? v.x : ~v.x));
      dd.push_back(make_float4(sg * x, sg * y, sg * z, 0.f));
    }
  }
  const int64_t m = static_cast<int64_t>(pq.size());
  std::vector<uint64_t> used(2 * n, 0);
  std::vector<int32_t> col(m);
  int ncol = 0;
  for (int64_t e = 0; e < m; ++e) {
    const int64_t a = pq[e].x, b = pq[e].y;
    int k = -1;
    for (int w = 0; w < 2 && k < 0; ++w) {
      const uint64_t busy = used[2 * a + w] | used[2 * b + w];
      if (~busy) k = 64 * w + __builtin_ctzll(~busy);
    }
    if (k < 0) return fail(c, XG_ERR_ARG, "rhs_coloured: more than 128 edge colours");
    used[2 * a + k / 64] |= uint64_t(1) << (k % 64);
    used[2 * b + k / 64] |= uint64_t(1) << (k % 64);
    col[e] = k;
    ncol = std::max(ncol, k + 1);
  }
  std::vector<int64_t> off(ncol + 1, 0);
  for (int64_t e = 0; e < m; ++e) ++off[col[e] + 1];
  for (int k = 0; k < ncol; ++k) off[k + 1] += off[k];
  std::vector<int2> spq(std::max<int64_t>(1, m));
  std::vector<float4> sdd(std::max<int64_t>(1, m));
  {
    std::vector<int64_t> fill(off.begin(), off.end() - 1);
    for (int64_t e = 0; e < m; ++e) {
      const int64_t to = fill[col[e]]++;
      spq[to] = pq[e];
      sdd[to] = dd[e];
    }
  }
  d->colarena.release();
  for (int pass = 0; pass < 2; ++pass) {
    Arena& A = d->colarena;
    A.plan(d->cpq, spq.size());
    A.plan(d->cd, sdd.size());
    A.plan(d->cR, n * 8);
    if (pass == 0) XG_CUDA(c, A.reserve());
  }
  XG_CUDA(c, cudaMemcpy(d->cpq, spq.data(), spq.size() * sizeof(int2), cudaMemcpyHostToDevice));
  XG_CUDA(c, cudaMemcpy(d->cd, sdd.data(), sdd.size() * sizeof(float4), cudaMemcpyHostToDevice));
  d->coff = off;
  return XG_OK;
}

template <int FLUX>
int launch_colours(xg_ctx* c, RieCGDev* d, const float* W, const float* G) {
  for (size_t k = 0; k + 1 < d->coff.size(); ++k) {
    const int64_t m = d->coff[k + 1] - d->coff[k];
    if (m == 0) continue;
    XG_PROF_LAUNCH(c, d, "riecg_flux_colour",
                   (k_flux_colour<FLUX><<<blocks_for(m, kBlock), kBlock, 0, c->stream>>>(
                       m, d->cpq + d->coff[k], d->cd + d->coff[k], W, G, d->prm.gamma,
                       d->prm.stab2, d->prm.stab2coef, d->cR)));
  }
  return XG_OK;
}

// xg_riecg_rhs with the edge-coloured scatter (FP32 mode).
int rhs_dropin_coloured(xg_ctx* c, RieCGDev* d, const double* G, const double* U, double* R) {
  int rc = build_colours(c, d);
  if (rc) return rc;
  float* W = static_cast<float*>(d->stage_W);
  float* Gr = static_cast<float*>(d->stage_G);
  XG_CUDA(c, cudaMemcpyAsync(d->stage_buf, G, d->n * 15 * sizeof(double), cudaMemcpyHostToDevice,
                             c->stream));
  k_aos_to_grec<float><<<blocks_for(d->n * 16, kBlock), kBlock, 0, c->stream>>>(d->n, d->stage_buf,
                                                                                 Gr);
  XG_CHECK_LAUNCH(c);
  XG_CUDA(c, cudaMemcpyAsync(d->stage_buf, U, d->n * 5 * sizeof(double), cudaMemcpyHostToDevice,
                             c->stream));
  k_prim_aos<float><<<blocks_for(d->n, kBlock), kBlock, 0, c->stream>>>(d->n, d->stage_buf, W, W);
  XG_CHECK_LAUNCH(c);
  XG_CUDA(c, cudaMemsetAsync(d->cR, 0, d->n * 8 * sizeof(float), c->stream));
  k_set_time<<<1, 1, 0, c->stream>>>(d->scal, d->t);
  XG_CHECK_LAUNCH(c);
  rc = launch_src<float>(c, d, W);
  if (rc) return rc;
  rc = d->prm.flux == XG_HLLC ? launch_colours<XG_HLLC>(c, d, W, Gr)
                              : launch_colours<XG_RUSANOV>(c, d, W, Gr);
  if (rc) return rc;
  XG_PROF_LAUNCH(c, d, "riecg_colour_out",
                 (k_colour_out<<<blocks_for(d->n, kBlock), kBlock, 0, c->stream>>>(
                     d->n, d->cR, bnd_of(d), W, d->prm.gamma, src_of<float>(d), d->stage_buf)));
  XG_CUDA(c, cudaMemcpyAsync(R, d->stage_buf, d->n * 5 * sizeof(double), cudaMemcpyDeviceToHost,
                             c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}
}  // namespace

extern "C" {

int xg_riecg_grad(xg_ctx* c, const double* U, double* G) {
  int rc = use(c);
  if (rc) return rc;
  RieCGDev* d = c->riecg;
  if (!d) return fail(c, XG_ERR_STATE, "riecg_grad before riecg_setup");
  if (!U || !G) return fail(c, XG_ERR_ARG, "riecg_grad: null array");
  return d->fp32 ? grad_dropin<float>(c, d, U, G) : grad_dropin<double>(c, d, U, G);
}

int xg_riecg_rhs(xg_ctx* c, const double* G, const double* U, double* R) {
  int rc = use(c);
  if (rc) return rc;
  RieCGDev* d = c->riecg;
  if (!d) return fail(c, XG_ERR_STATE, "riecg_rhs before riecg_setup");
  if (!U || !G || !R) return fail(c, XG_ERR_ARG, "riecg_rhs: null array");
  return d->fp32 ? rhs_dropin<float>(c, d, G, U, R) : rhs_dropin<double>(c, d, G, U, R);
}

int xg_riecg_rhs_coloured(xg_ctx* c, const double* G, const double* U, double* R, int* ncolours) {
  XG_HOST_TRY
  int rc = use(c);
  if (rc) return rc;
  RieCGDev* d = c->riecg;
  if (!d) return fail(c, XG_ERR_STATE, "riecg_rhs_coloured before riecg_setup");
  if (!d->fp32) return fail(c, XG_ERR_STATE, "riecg_rhs_coloured: FP32 mode only");
  if (!U || !G || !R) return fail(c, XG_ERR_ARG, "riecg_rhs_coloured: null array");
  rc = rhs_dropin_coloured(c, d, G, U, R);
  if (rc) return rc;
  if (ncolours) *ncolours = static_cast<int>(d->coff.size()) - 1;
  return XG_OK;
  XG_HOST_CATCH(c)
}

int xg_riecg_set_source(xg_ctx* c, int problem, const double* prm) {
  XG_HOST_TRY
  int rc = use(c);
  if (rc) return rc;
  RieCGDev* d = c->riecg;
  if (!d) return fail(c, XG_ERR_STATE, "riecg_set_source before riecg_setup");
  if (problem < XG_SRC_NONE || problem > XG_SRC_RAYLEIGH_TAYLOR)
    return fail(c, XG_ERR_ARG, "riecg_set_source: unknown problem");
  if (problem != XG_SRC_NONE && !d->Sv) {
    XG_CUDA(c, cudaStreamSynchronize(c->stream));
    for (int pass = 0; pass < 2; ++pass) {
      double* p64 = nullptr;
      float* p32 = nullptr;
      if (d->fp32)
        d->srcarena.plan(p32, d->n * 5);
      else
        d->srcarena.plan(p64, d->n * 5);
      if (pass == 0) XG_CUDA(c, d->srcarena.reserve());
      d->Sv = d->fp32 ? static_cast<void*>(p32) : static_cast<void*>(p64);
    }
  }
  d->src.problem = problem;
  for (int k = 0; k < 8; ++k) d->src.p[k] = prm ? prm[k] : 0.0;
  d->src.gamma = d->prm.gamma;
  // the captured time loop holds the source launch or not: capture again
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  drop_graphs(d);
  return XG_OK;
  XG_HOST_CATCH(c)
}

int xg_riecg_bc(xg_ctx* c) {
  int rc = use(c);
  if (rc) return rc;
  RieCGDev* d = c->riecg;
  if (!d) return fail(c, XG_ERR_STATE, "riecg_bc before riecg_setup");
  if (d->fp32)
    rc = launch_bc<float>(c, d, static_cast<float*>(d->W[d->cur]), 0);
  else
    rc = launch_bc<double>(c, d, static_cast<double*>(d->W[d->cur]), 0);
  if (rc) return rc;
  rc = refresh_dt(c, d);
  if (rc) return rc;
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}

int xg_riecg_dt(xg_ctx* c, double* dt) {
  int rc = use(c);
  if (rc) return rc;
  RieCGDev* d = c->riecg;
  if (!d) return fail(c, XG_ERR_STATE, "riecg_dt before riecg_setup");
  if (!dt) return fail(c, XG_ERR_ARG, "riecg_dt: null dt");
  if (!d->dt_valid) {
    rc = refresh_dt(c, d);
    if (rc) return rc;
  }
  Scalars s;
  XG_CUDA(c, cudaMemcpyAsync(&s, d->scal, sizeof(s), cudaMemcpyDeviceToHost, c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  double m;
  std::memcpy(&m, &s.dtmin, sizeof(double));
  if (std::fabs(d->prm.const_dt) > std::numeric_limits<double>::epsilon())
    *dt = d->prm.const_dt;
  else
    *dt = m * d->prm.cfl;
  return XG_OK;
}

int xg_riecg_stage(xg_ctx* c, int stage, double dt) {
  int rc = use(c);
  if (rc) return rc;
  RieCGDev* d = c->riecg;
  if (!d) return fail(c, XG_ERR_STATE, "riecg_stage before riecg_setup");
  if (stage < 0 || stage > 2) return fail(c, XG_ERR_ARG, "riecg_stage: stage must be 0..2");
  k_set_dt<<<1, 1, 0, c->stream>>>(d->scal, dt);
  XG_CHECK_LAUNCH(c);
  if (stage == 2) {
    k_reset_min<<<1, 1, 0, c->stream>>>(d->scal);
    XG_CHECK_LAUNCH(c);
  }
  // every stage's source at the context's time (the start of the step)
  k_set_time<<<1, 1, 0, c->stream>>>(d->scal, d->t);
  XG_CHECK_LAUNCH(c);
  rc = d->fp32 ? launch_src<float>(c, d, static_cast<const float*>(d->W[d->cur]))
               : launch_src<double>(c, d, static_cast<const double*>(d->W[d->cur]));
  if (rc) return rc;
  rc = d->fp32 ? do_stage<float>(c, d, stage, false) : do_stage<double>(c, d, stage, false);
  if (rc) return rc;
  d->dt_valid = stage == 2;
  if (stage == 2) d->t += dt;  // the step is complete
  rc = flush_profile(c, d);
  if (rc) return rc;
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}

int xg_riecg_run(xg_ctx* c, int64_t nstep, double* dts, float* ms) {
  int rc = use(c);
  if (rc) return rc;
  RieCGDev* d = c->riecg;
  if (!d) return fail(c, XG_ERR_STATE, "riecg_run before riecg_setup");
  if (nstep < 0) return fail(c, XG_ERR_ARG, "riecg_run: negative step count");
  if (nstep == 0) {
    if (ms) *ms = 0.f;
    return XG_OK;
  }
  if (!d->dt_valid) {
    rc = refresh_dt(c, d);
    if (rc) return rc;
  }
  if (d->dthist_cap < nstep) {
    XG_CUDA(c, cudaStreamSynchronize(c->stream));
    if (d->dthist) cudaFree(d->dthist);
    d->dthist = nullptr;
    const int64_t cap = std::max<int64_t>(nstep, 1024);
    XG_CUDA(c, cudaMalloc(&d->dthist, cap * sizeof(double)));
    d->dthist_cap = cap;
    drop_graphs(d);
  }
  XG_CUDA(c, cudaMemsetAsync(&d->scal->step, 0, sizeof(long long), c->stream));
  k_set_time<<<1, 1, 0, c->stream>>>(d->scal, d->t);
  XG_CHECK_LAUNCH(c);
  auto one_step = [&]() -> int {
    XG_PROF_LAUNCH(c, d, "riecg_step_begin",
                   (k_step_begin<<<1, 1, 0, c->stream>>>(d->scal, d->prm.cfl, d->prm.const_dt,
                                                         d->dthist)));
    // the source of the whole step at its start time (RieCG::rhs)
    const int r1 = d->fp32 ? launch_src<float>(c, d, static_cast<const float*>(d->W[d->cur]))
                           : launch_src<double>(c, d, static_cast<const double*>(d->W[d->cur]));
    if (r1) return r1;
    for (int st = 0; st < 3; ++st) {
      int r2 = d->fp32 ? do_stage<float>(c, d, st, true) : do_stage<double>(c, d, st, true);
      if (r2) return r2;
    }
    return XG_OK;
  };
  // replay two whole steps at a time from a captured graph (the primitive
  // buffers swap once per stage, so two steps return to the same buffer),
  // and single steps from a one-step graph of the current parity;
  // profiling runs launch kernel by kernel
  auto capture = [&](int steps, int parity, cudaGraphExec_t* out) -> int {
    const int saved = d->cur;
    d->cur = parity;
    cudaGraph_t g = nullptr;
    XG_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int r = XG_OK;
    for (int k = 0; k < steps && !r; ++k) r = one_step();
    cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
    d->cur = saved;
    if (r) {
      if (g) cudaGraphDestroy(g);
      return r;
    }
    if (ce != cudaSuccess) return fail(c, XG_ERR_CUDA, cudaGetErrorString(ce));
    ce = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
      *out = nullptr;
      return fail(c, XG_ERR_CUDA, cudaGetErrorString(ce));
    }
    return XG_OK;
  };
  auto single = [&]() -> int {
    if (d->prof) return one_step();
    const int par = d->cur;
    if (!d->graph1[par]) {
      const int r = capture(1, par, &d->graph1[par]);
      if (r) return r;
    }
    XG_CUDA(c, cudaGraphLaunch(d->graph1[par], c->stream));
    d->cur ^= 1;  // three buffer swaps
    return XG_OK;
  };
  const bool use_graph = !d->prof && nstep >= 2;
  int64_t done = 0;
  if (use_graph && !d->graph) {
    rc = capture(2, 0, &d->graph);
    if (rc) return rc;
  }
  cudaEvent_t e0, e1;
  XG_CUDA(c, cudaEventCreate(&e0));
  XG_CUDA(c, cudaEventCreate(&e1));
  XG_CUDA(c, cudaEventRecord(e0, c->stream));
  if (use_graph) {
    if (d->cur != 0) {
      rc = single();  // three buffer swaps bring cur back to 0
      if (rc) return rc;
      ++done;
    }
    while (nstep - done >= 2) {
      XG_CUDA(c, cudaGraphLaunch(d->graph, c->stream));
      done += 2;
    }
  }
  for (; done < nstep; ++done) {
    rc = single();
    if (rc) return rc;
  }
  XG_CUDA(c, cudaEventRecord(e1, c->stream));
  XG_CUDA(c, cudaEventSynchronize(e1));
  float el = 0.f;
  XG_CUDA(c, cudaEventElapsedTime(&el, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ms) *ms = el;
  rc = flush_profile(c, d);
  if (rc) return rc;
  std::vector<double> h(nstep);
  XG_CUDA(c, cudaMemcpy(h.data(), d->dthist, nstep * sizeof(double), cudaMemcpyDeviceToHost));
  for (double v : h) d->t += v;
  if (dts) std::memcpy(dts, h.data(), nstep * sizeof(double));
  d->dt_valid = true;
  Scalars s;
  XG_CUDA(c, cudaMemcpy(&s, d->scal, sizeof(s), cudaMemcpyDeviceToHost));
  if (s.blowup) return fail(c, XG_ERR_BLOWUP, "dt below machine epsilon");
  return XG_OK;
}

int xg_riecg_profile(xg_ctx* c, int enable) {
  if (!c || !c->riecg) return fail(c, XG_ERR_STATE, "riecg_profile before riecg_setup");
  RieCGDev* d = c->riecg;
  if (enable) {
    // a fresh record: launches still pending from an earlier one are dropped
    XG_CUDA(c, cudaStreamSynchronize(c->stream));
    for (auto& p : d->pending) {
      cudaEventDestroy(p.second.first);
      cudaEventDestroy(p.second.second);
    }
    d->pending.clear();
    d->ktimes.clear();
  }
  d->prof = enable != 0;
  return XG_OK;
}

int xg_riecg_kernel_times(xg_ctx* c, int cap, const char** names, double* ms, int64_t* launches,
                          int* n) {
  if (!c || !c->riecg) return fail(c, XG_ERR_STATE, "riecg_kernel_times before riecg_setup");
  // launches of the drop-in entry points are still pending here
  const int rc = flush_profile(c, c->riecg);
  if (rc) return rc;
  auto& kt = c->riecg->ktimes;
  if (n) *n = static_cast<int>(kt.size());
  for (int i = 0; i < cap && i < static_cast<int>(kt.size()); ++i) {
    if (names) names[i] = kt[i].name;
    if (ms) ms[i] = kt[i].ms;
    if (launches) launches[i] = kt[i].launches;
  }
  return XG_OK;
}

}  // extern "C"
