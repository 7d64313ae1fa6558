// KozCG on one GB300: element Taylor-Galerkin residual and flux-corrected
// transport, FP64, or with FP32 element arithmetic (XG_FP32_FLUX).
//
// Reference path (paths relative to the reference project root):
//   kozak::rhs      src/Physics/Kozak.cpp:29-180
//   KozCG::dt       src/Inciter/KozCG.cpp:613-688
//   KozCG::aec      src/Inciter/KozCG.cpp:772-843
//   KozCG::alw      src/Inciter/KozCG.cpp:865-948
//   KozCG::lim      src/Inciter/KozCG.cpp:978-1097
//   KozCG::solve    src/Inciter/KozCG.cpp:1119-1197
//   KozCG::BC       src/Inciter/KozCG.cpp:590-611 (Dirichlet and symmetry)
//
// Layout: node arrays SoA [ncomp][n] (U, R = rhs then low-order solution,
// P = antidiffusive sums +/- per component, A = limited contributions),
// elements as int32 [T][4].  Element kernels (one thread per tet) hand their
// four nodes' contributions on: in FP64 as plain stores into element-major
// slots that k_node_gather sums per node in ascending element order (the
// reference's order, the same bits on every run), in FP32 as vector atomic
// adds into node records.  The allowed limits Q+/- (extremes over
// the elements holding a node) are taken per node over the node adjacency,
// which holds the same nodes, and kept as order-preserving keys.  Node
// kernels (one thread per node) do the per-node algebra between the element
// passes.  One step is:
//   step_begin -> node_prim -> elem_rhs_aec -> [gather] -> bc_p -> node_lo -> node_alw ->
//   node_lim -> elem_lim -> [gather] -> node_solve -> bc (+ CFL minimum for the next step)
// ([gather]: FP64; FP32 zeroes its records first instead)
//
// FP32-element mode: the element passes read an FP32 copy of the state (made
// by node_prim) and FP32 element geometry (made at setup), and add into FP32
// node records [n][16] / [n][8] with vector atomics; the allowed limits are
// 32-bit keys of floats.  The node passes (low-order solution, limit
// coefficients, update, dt) stay FP64 on the FP64 state.  GB300's FP64 rate
// is a small fraction of its FP32 rate, and FP32/FP64 conversions run at the
// FP64 rate, so this mode converts per node, not per element.

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "xg_internal.hpp"
#include "xg_source.cuh"

namespace xg {

namespace {
constexpr int kBlock = 256;

struct KScalars {
  double dt;
  unsigned long long dtmin;
  int32_t blowup;
  int32_t pad;
  double t, tnext;  // the current step's start time, the next step's
};
}  // namespace

struct KozCGDev {
  Arena arena;
  Arena bcarena;
  int64_t n = 0, ne = 0;
  xg_kozcg_params prm{};
  int32_t* inpoel = nullptr;
  double *xyz = nullptr, *vol = nullptr;
  double *U = nullptr, *R = nullptr, *P = nullptr, *A = nullptr;
  unsigned long long* Q = nullptr;
  double* stage = nullptr;
  double* V = nullptr;  // [n][4] velocity and pressure per node (FP32 packed in the first half)
  // FP32-element mode: element sums, the FP32 state, the low-order solution
  // as the allowed-limit pass reads it, 32-bit limit keys, element geometry
  float *R32 = nullptr, *A32 = nullptr, *U32 = nullptr, *lo32 = nullptr;
  unsigned int* Q32 = nullptr;
  float* geo32 = nullptr;
  // FP64 mode: residual and limited slot records (10 and 6 doubles per
  // (element, local node) slot) and each node's slots in element order,
  // SELL-32 like the adjacency
  double *E = nullptr, *L = nullptr;
  int32_t *soff = nullptr, *sw = nullptr, *sslot = nullptr;
  // node adjacency (every pair of nodes sharing a tet) as SELL-32: slice s
  // of 32 nodes, entry k of node i at aoff[s] + 32 k + lane, -1 padding
  int64_t nslice = 0;
  int32_t *aoff = nullptr, *aw = nullptr, *anbr = nullptr;
  // BC program: one thread per BC node
  int64_t nbc = 0;
  int32_t *bcnode = nullptr, *bcdir = nullptr, *bcsymp = nullptr, *dirmask = nullptr;
  double *symn = nullptr, *dirval = nullptr;
  uint8_t* isbc = nullptr;  // per node
  KScalars* scal = nullptr;
  double* dthist = nullptr;
  int64_t dthist_cap = 0;
  double t = 0.0;
  bool dt_valid = false;
  // manufactured source (kozak::rhs with problems::SRC): per step the
  // sources at the nodes at the step's start time S [5][n] and at the
  // element centroids half a step later Se [ne][5]
  SrcPrm src{};
  double *S = nullptr, *Se = nullptr;
};

void destroy_kozcg(KozCGDev* d) {
  if (!d) return;
  if (d->dthist) cudaFree(d->dthist);
  if (d->S) cudaFree(d->S);
  if (d->Se) cudaFree(d->Se);
  delete d;
}
size_t bytes_kozcg(const KozCGDev* d) { return d ? d->arena.bytes() + d->bcarena.bytes() : 0; }

namespace {

// order-preserving map of doubles to unsigned 64-bit keys
__device__ __forceinline__ unsigned long long dkey(double v) {
  unsigned long long b = __double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double dval(unsigned long long k) {
  unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double(b);
}

__device__ __forceinline__ double node_dt(const double u[5], double vol, double g) {
  double r = u[0];
  double uu = u[1] / r, vv = u[2] / r, ww = u[3] / r;
  double pr = (u[4] - 0.5 * r * (uu * uu + vv * vv + ww * ww)) * (g - 1.0);
  double c = sqrt(g * fmax(pr, 0.0) / r);
  double L = cbrt(vol);
  double vel = sqrt(uu * uu + vv * vv + ww * ww);
  return L / fmax(vel + c, 1.0e-8);
}

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

template <class F>
struct Geo {
  F J;
  F g[4][3];
};

// Element geometry (Kozak.cpp:76-89): coordinate differences in FP64, the
// cross products and Jacobian in F.
template <class F>
__device__ __forceinline__ Geo<F> tetgeo(const double* xyz, int64_t n, const int32_t N[4]) {
  const double* x = xyz;
  const double* y = xyz + n;
  const double* z = xyz + 2 * n;
  const F ba[3] = {F(x[N[1]] - x[N[0]]), F(y[N[1]] - y[N[0]]), F(z[N[1]] - z[N[0]])};
  const F ca[3] = {F(x[N[2]] - x[N[0]]), F(y[N[2]] - y[N[0]]), F(z[N[2]] - z[N[0]])};
  const F da[3] = {F(x[N[3]] - x[N[0]]), F(y[N[3]] - y[N[0]]), F(z[N[3]] - z[N[0]])};
  Geo<F> t;
  t.g[1][0] = ca[1] * da[2] - da[1] * ca[2];
  t.g[1][1] = ca[2] * da[0] - da[2] * ca[0];
  t.g[1][2] = ca[0] * da[1] - da[0] * ca[1];
  t.g[2][0] = da[1] * ba[2] - ba[1] * da[2];
  t.g[2][1] = da[2] * ba[0] - ba[2] * da[0];
  t.g[2][2] = da[0] * ba[1] - ba[0] * da[1];
  t.g[3][0] = ba[1] * ca[2] - ca[1] * ba[2];
  t.g[3][1] = ba[2] * ca[0] - ca[2] * ba[0];
  t.g[3][2] = ba[0] * ca[1] - ca[0] * ba[1];
  for (int i = 0; i < 3; ++i) t.g[0][i] = -t.g[1][i] - t.g[2][i] - t.g[3][i];
  t.J = ba[0] * t.g[1][0] + ba[1] * t.g[1][1] + ba[2] * t.g[1][2];
  return t;
}

// Types of a precision mode: F is the element arithmetic; FP64 mode sums in
// FP64 and keeps the allowed limits as 64-bit keys of doubles, the
// FP32-element mode sums in FP32 and keys floats in 32 bits.
template <class F>
struct KozT;
template <>
struct KozT<double> {
  using Key = unsigned long long;
};
template <>
struct KozT<float> {
  using Key = unsigned int;
};

__device__ __forceinline__ unsigned long long okey(double v) { return dkey(v); }
__device__ __forceinline__ unsigned int okey(float v) {
  const unsigned int b = __float_as_uint(v);
  return (b >> 31) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ double oval(unsigned long long k) { return dval(k); }
__device__ __forceinline__ float oval(unsigned int k) {
  return __uint_as_float((k >> 31) ? (k & 0x7fffffffu) : ~k);
}
__device__ __forceinline__ double kbits(unsigned long long k) { return __longlong_as_double(k); }
__device__ __forceinline__ float kbits(unsigned int k) { return __uint_as_float(k); }
__device__ __forceinline__ unsigned long long tobits(double v) { return __double_as_longlong(v); }
__device__ __forceinline__ unsigned int tobits(float v) { return __float_as_uint(v); }

// Where component c of node i lives in the element sums: FP64 mode SoA
// [5][n] (R, A) and [10][n] (P), written whole by k_node_gather from the
// slot records; FP32 mode node records, so that one element
// adds a node's contribution with 16-byte vector atomics
// (red.global.add.v4.f32) instead of one atomic per component: R and P share
// a [n][16] record (R at 0..4, P+/- at 5..14, P addressed from R + 5), A has
// [n][8].
constexpr int kRP = 16;   // FP32 R+P record
constexpr int kAR = 8;    // FP32 A record
constexpr int kGB = 4;    // FP64 node gather: slots loaded together
template <class F, int S>
__device__ __forceinline__ int64_t ridx(int64_t n, int c, int64_t i) {
  return sizeof(F) == 4 ? i * S + c : c * n + i;
}
template <class F>
__device__ __forceinline__ int64_t pidx(int64_t n, int cs, int64_t i) {
  return sizeof(F) == 4 ? i * kRP + cs : cs * n + i;
}

// FP32 mode: r[5] added to node i's record of R (S = kRP) or A (S = kAR).
template <int S>
__device__ __forceinline__ void add5(float* R, int64_t, int64_t i, const float r[5]) {
  atomicAdd(reinterpret_cast<float4*>(R + i * S), make_float4(r[0], r[1], r[2], r[3]));
  atomicAdd(R + i * S + 4, r[4]);
}

// Per-node velocity and pressure (the node-wise quotients kozak::rhs forms
// for every element holding the node, Kozak.cpp:93-118): computed once per
// node, the same expressions, so the element pass gathers bit-identical
// values instead of repeating the FP64 divisions per element.  In FP32 mode
// the state itself is also stored in FP32 (Uf), so that the element passes
// read it without conversions.
template <class F>
__global__ void __launch_bounds__(kBlock) k_node_prim(int64_t n, const double* __restrict__ U,
                                                       double gamma_d, F* __restrict__ V,
                                                       F* __restrict__ Uf) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const F gamma = F(gamma_d);
  F u[5];
#pragma unroll
  for (int c = 0; c < 5; ++c) u[c] = F(U[c * n + i]);
  F o[4];
#pragma unroll
  for (int j = 0; j < 3; ++j) o[j] = u[j + 1] / u[0];
  o[3] = (gamma - F(1.0)) * (u[4] - F(0.5) * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) / u[0]);
#pragma unroll
  for (int k = 0; k < 4; ++k) V[i * 4 + k] = o[k];
  if (Uf) {
#pragma unroll
    for (int c = 0; c < 5; ++c) Uf[c * n + i] = u[c];
  }
}

// Element geometry in FP32 for the FP32 mode, formed once at setup from the
// FP64 coordinates (tetgeo<double>, then rounded): J and g1, g2, g3 as
// [10][T] (g0 = -g1 - g2 - g3 is re-formed in the element passes).
__global__ void k_geo32(int64_t n, int64_t ne, const int32_t* __restrict__ inpoel,
                        const double* __restrict__ xyz, float* __restrict__ geo) {
  const int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (e >= ne) return;
  int32_t N[4];
  for (int a = 0; a < 4; ++a) N[a] = inpoel[e * 4 + a];
  const Geo<double> t = tetgeo<double>(xyz, n, N);
  geo[e] = float(t.J);
  for (int a = 1; a < 4; ++a)
    for (int j = 0; j < 3; ++j) geo[(1 + (a - 1) * 3 + j) * ne + e] = float(t.g[a][j]);
}

template <class F>
__device__ __forceinline__ Geo<F> elem_geo(const double* __restrict__ xyz,
                                           const float* __restrict__ geo, int64_t n, int64_t ne,
                                           int64_t e, const int32_t N[4]) {
  if constexpr (sizeof(F) == 8) {
    return tetgeo<double>(xyz, n, N);
  } else {
    Geo<float> t;
    t.J = __ldg(geo + e);
    for (int a = 1; a < 4; ++a)
      for (int j = 0; j < 3; ++j) t.g[a][j] = __ldg(geo + (1 + (a - 1) * 3 + j) * ne + e);
    for (int j = 0; j < 3; ++j) t.g[0][j] = -t.g[1][j] - t.g[2][j] - t.g[3][j];
    return t;
  }
}

// Component c of the state at a node, as the element arithmetic reads it.
template <class F>
__device__ __forceinline__ F ust(const double* __restrict__ U, const F* __restrict__ Uf, int64_t n,
                                 int c, int32_t node) {
  if constexpr (sizeof(F) == 8)
    return U[c * n + node];
  else
    return __ldg(Uf + c * n + node);
}

// kozak::rhs for one tet (Kozak.cpp:73-173) plus the antidiffusive element
// contributions of KozCG::aec (KozCG.cpp:794-814), scattered to the nodes.
// V holds each node's velocity and pressure (k_node_prim).
template <class F>
__device__ __forceinline__ void load_v4(const F* V, int64_t i, F o[4]) {
  if constexpr (sizeof(F) == 8) {
    const double2* q = reinterpret_cast<const double2*>(V + i * 4);
    const double2 a = __ldg(q), b = __ldg(q + 1);
    o[0] = a.x;
    o[1] = a.y;
    o[2] = b.x;
    o[3] = b.y;
  } else {
    const float4 a = __ldg(reinterpret_cast<const float4*>(V + i * 4));
    o[0] = a.x;
    o[1] = a.y;
    o[2] = a.z;
    o[3] = a.w;
  }
}

// kozak::rhs for one tet (Kozak.cpp:73-173): the residual r[a][c] of its
// four nodes, and with fct the antidiffusive element contributions of
// KozCG::aec (KozCG.cpp:794-814) aec[a][c] (zero without).  V holds each
// node's velocity and pressure (k_node_prim).
template <class F>
__device__ __forceinline__ void elem_terms(int64_t n, int64_t ne, int64_t e,
                                           const int32_t* __restrict__ inpoel,
                                           const double* __restrict__ xyz,
                                           const float* __restrict__ geo,
                                           const double* __restrict__ U, const F* __restrict__ Uf,
                                           const F* __restrict__ V,
                                           const KScalars* __restrict__ sc, F gamma, F ctau,
                                           int fct, const double* __restrict__ S,
                                           const double* __restrict__ Se, int32_t N[4],
                                           F r[4][5], F aec[4][5]) {
  for (int a = 0; a < 4; ++a) N[a] = inpoel[e * 4 + a];
  const Geo<F> t = elem_geo<F>(xyz, geo, n, ne, e, N);
  F u[4][5], vel[4][3], p[4];
  for (int a = 0; a < 4; ++a) {
    for (int c = 0; c < 5; ++c) u[a][c] = ust<F>(U, Uf, n, c, N[a]);
    F v4[4];
    load_v4(V, N[a], v4);
    vel[a][0] = v4[0];
    vel[a][1] = v4[1];
    vel[a][2] = v4[2];
    p[a] = v4[3];
  }
  const F dt = F(sc->dt);
  F ue[5];
  for (int c = 0; c < 5; ++c) ue[c] = (u[0][c] + u[1][c] + u[2][c] + u[3][c]) / F(4.0);
  F coef = dt / t.J / F(2.0);
  for (int j = 0; j < 3; ++j)
    for (int a = 0; a < 4; ++a) {
      const F cg = coef * t.g[a][j];
      const F uj = vel[a][j];
      ue[0] -= cg * u[a][j + 1];
      ue[1] -= cg * u[a][1] * uj;
      ue[2] -= cg * u[a][2] * uj;
      ue[3] -= cg * u[a][3] * uj;
      ue[j + 1] -= cg * p[a];
      ue[4] -= cg * (u[a][4] + p[a]) * uj;
    }
  if (S) {  // the nodes' sources at the step's start time, dt/8 each
    const F c8 = dt / F(8.0);
    for (int a = 0; a < 4; ++a)
      for (int c = 0; c < 5; ++c) ue[c] += c8 * F(__ldg(S + c * n + N[a]));
  }
  const F pr =
      (gamma - F(1.0)) * (ue[4] - F(0.5) * (ue[1] * ue[1] + ue[2] * ue[2] + ue[3] * ue[3]) / ue[0]);
  for (int a = 0; a < 4; ++a)
    for (int c = 0; c < 5; ++c) r[a][c] = F(0.0);
  coef = F(1.0) / F(6.0);
  for (int j = 0; j < 3; ++j) {
    const F uj = ue[j + 1] / ue[0];
    for (int a = 0; a < 4; ++a) {
      const F cg = coef * t.g[a][j];
      r[a][0] += cg * ue[j + 1];
      r[a][1] += cg * ue[1] * uj;
      r[a][2] += cg * ue[2] * uj;
      r[a][3] += cg * ue[3] * uj;
      r[a][j + 1] += cg * pr;
      r[a][4] += cg * (ue[4] + pr) * uj;
    }
  }
  if (Se) {  // the centroid's source half a step later, J/24 to each node
    const F cj = t.J / F(24.0);
    F se[5];
    for (int c = 0; c < 5; ++c) se[c] = F(__ldg(Se + e * 5 + c));
    for (int a = 0; a < 4; ++a)
      for (int c = 0; c < 5; ++c) r[a][c] += cj * se[c];
  }
  for (int c = 0; c < 5; ++c)
    for (int a = 0; a < 4; ++a) {
      F s = F(0.0);
      if (fct)
        for (int b = 0; b < 4; ++b) {
          const F m = t.J / F(120.0) * ((a == b) ? F(3.0) : F(-1.0));
          s += m * ctau * u[b][c];
        }
      aec[a][c] = s;
    }
}

// FP32 element pass: per node its residual and its ten antidiffusive sums
// (+, - per component; the sign that does not apply adds 0) in one [16]
// record, four vector atomics (one per 4 floats); without FCT the residual
// alone.
__global__ void __launch_bounds__(kBlock) k_elem_rhs_aec32(int64_t n, int64_t ne,
                                                            const int32_t* __restrict__ inpoel,
                                                            const float* __restrict__ geo,
                                                            const float* __restrict__ Uf,
                                                            const float* __restrict__ V,
                                                            const KScalars* __restrict__ sc,
                                                            double gamma, double ctau, int fct,
                                                            const double* __restrict__ S,
                                                            const double* __restrict__ Se,
                                                            float* R) {
  const int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (e >= ne) return;
  int32_t N[4];
  float r[4][5], aec[4][5];
  elem_terms<float>(n, ne, e, inpoel, nullptr, geo, nullptr, Uf, V, sc, float(gamma),
                    float(ctau), fct, S, Se, N, r, aec);
  if (!fct) {
    for (int a = 0; a < 4; ++a) add5<kRP>(R, n, N[a], r[a]);
    return;
  }
  for (int a = 0; a < 4; ++a) {
    float v[16];
    for (int c = 0; c < 5; ++c) v[c] = r[a][c];
    for (int c = 0; c < 5; ++c) {
      v[5 + c * 2 + 0] = aec[a][c] > 0.f ? aec[a][c] : 0.f;
      v[5 + c * 2 + 1] = aec[a][c] < 0.f ? aec[a][c] : 0.f;
    }
    v[15] = 0.f;
    float* q = R + int64_t(N[a]) * kRP;
    for (int k = 0; k < 4; ++k)
      atomicAdd(reinterpret_cast<float4*>(q + 4 * k),
                make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]));
  }
}

// FP64 element passes hand their node contributions to k_node_gather through
// slot records, one per (element e, local node a), slot q = 4 e + a: the
// residual pass writes 10 doubles (the five contributions, then the five
// antidiffusive ones), the limiting pass 6 (the five limited contributions
// and a zero).  A warp's 32 elements own 128 consecutive records; each lane
// builds its four in shared memory (kStW double2 per lane: 16-byte stores
// of 8 lanes fall in distinct banks) and the warp moves the run to or from
// global memory with contiguous 512-byte accesses.
constexpr int kEB = 128;   // FP64 element-pass block: 4 warps
constexpr int kStW = 21;   // staged double2 per lane
constexpr int kRecD2 = 5;  // residual slot record, double2
constexpr int kLimD2 = 3;  // limited slot record, double2

template <int D2>  // double2 per element
__device__ __forceinline__ void warp_put(double2* __restrict__ g, const double2* buf, int nv,
                                         int lane) {
  for (int k = lane; k < nv * D2; k += 32) g[k] = buf[(k / D2) * kStW + k % D2];
}
template <int D2>
__device__ __forceinline__ void warp_get(const double2* __restrict__ g, double2* buf, int nv,
                                         int lane) {
  for (int k = lane; k < nv * D2; k += 32) buf[(k / D2) * kStW + k % D2] = __ldg(g + k);
}

__global__ void __launch_bounds__(kEB) k_elem_rhs64(int64_t n, int64_t ne,
                                                     const int32_t* __restrict__ inpoel,
                                                     const double* __restrict__ xyz,
                                                     const double* __restrict__ U,
                                                     const double* __restrict__ V,
                                                     const KScalars* __restrict__ sc,
                                                     double gamma, double ctau, int fct,
                                                     const double* __restrict__ S,
                                                     const double* __restrict__ Se,
                                                     double* __restrict__ E) {
  __shared__ double2 st[kEB / 32][32 * kStW];
  const int lane = threadIdx.x & 31;
  const int64_t e = blockIdx.x * int64_t(kEB) + threadIdx.x;
  const int64_t e0 = e - lane;
  if (e0 >= ne) return;  // the whole warp is past the last element
  double2* buf = st[threadIdx.x >> 5];
  if (e < ne) {
    int32_t N[4];
    double r[4][5], aec[4][5];
    elem_terms<double>(n, ne, e, inpoel, xyz, nullptr, U, nullptr, V, sc, gamma, ctau, fct, S, Se,
                       N, r, aec);
    for (int a = 0; a < 4; ++a) {
      double2* b = buf + lane * kStW + a * kRecD2;
      b[0] = make_double2(r[a][0], r[a][1]);
      b[1] = make_double2(r[a][2], r[a][3]);
      b[2] = make_double2(r[a][4], aec[a][0]);
      b[3] = make_double2(aec[a][1], aec[a][2]);
      b[4] = make_double2(aec[a][3], aec[a][4]);
    }
  }
  __syncwarp();
  const int nv = static_cast<int>(ne - e0 < 32 ? ne - e0 : 32);
  warp_put<4 * kRecD2>(reinterpret_cast<double2*>(E) + e0 * 4 * kRecD2, buf, nv, lane);
}

struct KBC {
  int64_t nbc;
  const int32_t* node;
  const int32_t* dir;
  const int32_t* symp;
  const int32_t* dirmask;
  const double* dirval;
  const double* symn;
  SrcPrm prob;         // the problem whose analytic state mask-1 Dirichlet values take
  const double* xyz;   // [3][n] node coordinates
};

// Symmetry projection of the momentum antidiffusive sums (KozCG.cpp:816-830).
template <class F>
__global__ void k_bc_p(int64_t n, KBC bc, F* P) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= bc.nbc) return;
  const int64_t p = bc.node[i];
  for (int32_t k = bc.symp[i]; k < bc.symp[i + 1]; ++k) {
    const F nx = F(bc.symn[3 * k]), ny = F(bc.symn[3 * k + 1]), nz = F(bc.symn[3 * k + 2]);
    F* P2 = P + pidx<F>(n, 2, p);  // comp 1 (+)
    F* P3 = P + pidx<F>(n, 3, p);  // comp 1 (-)
    F* P4 = P + pidx<F>(n, 4, p);
    F* P5 = P + pidx<F>(n, 5, p);
    F* P6 = P + pidx<F>(n, 6, p);
    F* P7 = P + pidx<F>(n, 7, p);
    const F rvnp = *P2 * nx + *P4 * ny + *P6 * nz;
    const F rvnn = *P3 * nx + *P5 * ny + *P7 * nz;
    *P2 -= rvnp * nx;
    *P3 -= rvnn * nx;
    *P4 -= rvnp * ny;
    *P5 -= rvnn * ny;
    *P6 -= rvnp * nz;
    *P7 -= rvnn * nz;
  }
}

// KozCG::alw node part (KozCG.cpp:887-912): P /= vol, low-order solution
// lo = U + dt R/vol - P+ - P-.
// Without FCT the update of KozCG::solve (KozCG.cpp:1151-1160) goes straight
// to A.  Racc/Pacc are the element sums (in F); lo and P/vol go to the FP64
// arrays Rlo/Pout (the same arrays as Racc/Pacc in FP64 mode), and in FP32
// mode lo also to lo32 for the element pass of the allowed limits.
template <class F>
__global__ void k_node_lo(int64_t n, const double* __restrict__ vol, const double* __restrict__ U,
                          const KScalars* __restrict__ sc, int fct, const F* Racc, const F* Pacc,
                          double* Rlo, double* Pout, F* lo32, double* A) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const double dt = sc->dt;
  const double v = vol[i];
  // FP32 mode: one FP64 division per node (GB300's FP64 divisions are slow);
  // FP64 mode divides as the reference does
  const double iv = sizeof(F) == 4 ? 1.0 / v : 0.0;
  auto per_vol = [&](double x) { return sizeof(F) == 4 ? x * iv : x / v; };
  for (int c = 0; c < 5; ++c) {
    if (fct) {
      double pp = per_vol(double(Pacc[pidx<F>(n, c * 2 + 0, i)]));
      double pn = per_vol(double(Pacc[pidx<F>(n, c * 2 + 1, i)]));
      Pout[(c * 2 + 0) * n + i] = pp;
      Pout[(c * 2 + 1) * n + i] = pn;
      const double lo = U[c * n + i] + per_vol(dt * double(Racc[ridx<F, kRP>(n, c, i)])) - pp - pn;
      Rlo[c * n + i] = lo;
      if (lo32) lo32[c * n + i] = F(lo);
    } else {
      A[c * n + i] = U[c * n + i] + per_vol(dt * double(Racc[ridx<F, kRP>(n, c, i)]));
    }
  }
}

// KozCG::alw element part (KozCG.cpp:914-935): the allowed limits of a node
// are the maximum / minimum, over the elements holding it, of the element's
// extremes of the low-order solution lo (and of the state U unless clip).
// The nodes of those elements are the node and its adjacency, so the same
// extremes are taken here per node over {i} and its neighbours: max and min
// are exact, so the bounds are the element loop's, without atomics.  Stored
// as order-preserving keys (the node pass of the limits reads keys).
template <class F>
__global__ void __launch_bounds__(kBlock) k_node_alw(int64_t n, const int32_t* __restrict__ aoff,
                                                      const int32_t* __restrict__ aw,
                                                      const int32_t* __restrict__ nbr,
                                                      const F* __restrict__ U,
                                                      const F* __restrict__ lo, int clip,
                                                      typename KozT<F>::Key* __restrict__ Q) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int lane = static_cast<int>(i & 31);
  const int64_t s = i >> 5;
  const int32_t off = __ldg(aoff + s), w = __ldg(aw + s);
  F mx[5], mn[5];
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    const F l = lo[c * n + i];
    mx[c] = l;
    mn[c] = l;
    if (!clip) {
      const F u = U[c * n + i];
      mx[c] = fmax(mx[c], u);
      mn[c] = fmin(mn[c], u);
    }
  }
#pragma unroll 4
  for (int k = 0; k < w; ++k) {
    const int32_t q = __ldg(nbr + off + k * 32 + lane);
    if (q < 0) continue;
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      const F l = __ldg(lo + c * n + q);
      mx[c] = fmax(mx[c], l);
      mn[c] = fmin(mn[c], l);
      if (!clip) {
        const F u = __ldg(U + c * n + q);
        mx[c] = fmax(mx[c], u);
        mn[c] = fmin(mn[c], u);
      }
    }
  }
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    Q[(c * 2 + 0) * n + i] = okey(mx[c]);
    Q[(c * 2 + 1) * n + i] = okey(mn[c]);
  }
}

// KozCG::lim node part (KozCG.cpp:1004-1024): Q -= low-order solution, limit
// coefficients C+/- stored back into Q as F values (reinterpreted).
template <class F>
__global__ void k_node_lim(int64_t n, const double* __restrict__ R, const double* __restrict__ P,
                           typename KozT<F>::Key* Q) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const double eps = DBL_EPSILON;
  for (int c = 0; c < 5; ++c) {
    double qp = double(oval(Q[(c * 2 + 0) * n + i])) - R[c * n + i];
    double qn = double(oval(Q[(c * 2 + 1) * n + i])) - R[c * n + i];
    const double pp = P[(c * 2 + 0) * n + i], pn = P[(c * 2 + 1) * n + i];
    // the coefficient's quotient in F (an FP32 division in FP32 mode)
    const F cp = pp < eps ? F(0) : fmin(F(1), F(qp) / F(pp));
    const F cn = pn > -eps ? F(0) : fmin(F(1), F(qn) / F(pn));
    Q[(c * 2 + 0) * n + i] = tobits(cp);
    Q[(c * 2 + 1) * n + i] = tobits(cn);
  }
}

// KozCG::lim element part (KozCG.cpp:1049-1078): limited antidiffusive
// element contributions, system-limited over the components in sysmask.
// Limit coefficients of one element from its antidiffusive contributions
// aec[a][c] and the nodes' C+/- (Q, as F bits); ca = the limited ones.
template <class F>
__device__ __forceinline__ void elem_limit(int64_t n, const int32_t N[4],
                                           const typename KozT<F>::Key* __restrict__ Q,
                                           int sysmask, const F aec[4][5], F ca[4][5]) {
  F coef[5];
  for (int c = 0; c < 5; ++c) {
    coef[c] = F(1.0);
    for (int a = 0; a < 4; ++a) {
      const F s = aec[a][c];
      const F lim = kbits(Q[(c * 2 + (s > F(0.0) ? 0 : 1)) * n + N[a]]);
      coef[c] = coef[c] < lim ? coef[c] : lim;
    }
  }
  F cs = F(1.0);
  for (int c = 0; c < 5; ++c)
    if (sysmask & (1 << c)) cs = cs < coef[c] ? cs : coef[c];
  for (int c = 0; c < 5; ++c)
    if (sysmask & (1 << c)) coef[c] = cs;
  for (int a = 0; a < 4; ++a)
    for (int c = 0; c < 5; ++c) ca[a][c] = coef[c] * aec[a][c];
}

// FP32: the antidiffusive contributions formed again from the FP32 state and
// geometry (as KozCG::lim does), the limited ones added atomically.
__global__ void __launch_bounds__(kBlock) k_elem_lim32(int64_t n, int64_t ne,
                                                        const int32_t* __restrict__ inpoel,
                                                        const float* __restrict__ geo,
                                                        const float* __restrict__ Uf,
                                                        const unsigned int* __restrict__ Q,
                                                        double ctau_d, int sysmask, float* A) {
  const int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (e >= ne) return;
  const float ctau = float(ctau_d);
  int32_t N[4];
  for (int a = 0; a < 4; ++a) N[a] = inpoel[e * 4 + a];
  const Geo<float> t = elem_geo<float>(nullptr, geo, n, ne, e, N);
  float aec[4][5], ca[4][5];
  for (int c = 0; c < 5; ++c)
    for (int a = 0; a < 4; ++a) {
      float s = 0.f;
      for (int b = 0; b < 4; ++b) {
        const float m = t.J / 120.f * ((a == b) ? 3.f : -1.f);
        s += m * ctau * ust<float>(nullptr, Uf, n, c, N[b]);
      }
      aec[a][c] = s;
    }
  elem_limit<float>(n, N, Q, sysmask, aec, ca);
  for (int a = 0; a < 4; ++a) add5<kAR>(A, n, N[a], ca[a]);
}

// FP64: the antidiffusive contributions are the ones the residual pass
// stored in the residual slot records E (the values KozCG::lim forms again
// from the same state and geometry); the limited ones go to the limited slot
// records L.
__global__ void __launch_bounds__(kEB) k_elem_lim64(int64_t n, int64_t ne,
                                                     const int32_t* __restrict__ inpoel,
                                                     const double* __restrict__ E,
                                                     const unsigned long long* __restrict__ Q,
                                                     int sysmask, double* __restrict__ L) {
  __shared__ double2 st[kEB / 32][32 * kStW];
  const int lane = threadIdx.x & 31;
  const int64_t e = blockIdx.x * int64_t(kEB) + threadIdx.x;
  const int64_t e0 = e - lane;
  if (e0 >= ne) return;  // the whole warp is past the last element
  double2* buf = st[threadIdx.x >> 5];
  const int nv = static_cast<int>(ne - e0 < 32 ? ne - e0 : 32);
  warp_get<4 * kRecD2>(reinterpret_cast<const double2*>(E) + e0 * 4 * kRecD2, buf, nv, lane);
  __syncwarp();
  double ca[4][5];
  const bool live = e < ne;
  if (live) {
    int32_t N[4];
    for (int a = 0; a < 4; ++a) N[a] = inpoel[e * 4 + a];
    double aec[4][5];
    for (int a = 0; a < 4; ++a) {
      const double* rec = reinterpret_cast<const double*>(buf + lane * kStW + a * kRecD2);
      for (int c = 0; c < 5; ++c) aec[a][c] = rec[5 + c];
    }
    elem_limit<double>(n, N, Q, sysmask, aec, ca);
  }
  __syncwarp();
  if (live)
    for (int a = 0; a < 4; ++a) {
      double2* b = buf + lane * kStW + a * kLimD2;
      b[0] = make_double2(ca[a][0], ca[a][1]);
      b[1] = make_double2(ca[a][2], ca[a][3]);
      b[2] = make_double2(ca[a][4], 0.0);
    }
  __syncwarp();
  warp_put<4 * kLimD2>(reinterpret_cast<double2*>(L) + e0 * 4 * kLimD2, buf, nv, lane);
}

// FP64 node sums of the element contributions, in a fixed order: node i
// adds the slots (element e, local node a) of the elements holding it in
// ascending e -- the order of the reference's serial element loop
// (Kozak.cpp:73-173 adds R[N[a]] per element, KozCG.cpp:794-814 and
// 1049-1078 likewise P and A) -- so the sums are the same on every run, with
// no atomics.  Slot q's record is RD2 double2 at E + q * RD2: entries 0..4
// the contributions to the node's five components, and with WP entries
// 5..9 the antidiffusive ones, summed by sign into P+ / P- (zero goes to
// neither).  Slots as SELL-32: slice s of 32 nodes, entry k of node i at
// soff[s] + 32 k + lane, value q, -1 padding.  The slots are taken kGB at a
// time, their loads issued together before the adds (in slot order), so
// that a node's loads overlap.
template <int RD2, bool WP>
__global__ void __launch_bounds__(kBlock) k_node_gather(int64_t n,
                                                         const int32_t* __restrict__ soff,
                                                         const int32_t* __restrict__ sw,
                                                         const int32_t* __restrict__ slot,
                                                         const double* __restrict__ E,
                                                         double* __restrict__ R,
                                                         double* __restrict__ P) {
  constexpr int LD2 = WP ? 5 : 3;  // double2 read per slot
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int lane = static_cast<int>(i & 31);
  const int64_t s = i >> 5;
  const int32_t off = __ldg(soff + s), w = __ldg(sw + s);
  const double2* E2 = reinterpret_cast<const double2*>(E);
  double r[5], pp[5], pn[5];
#pragma unroll
  for (int c = 0; c < 5; ++c) r[c] = pp[c] = pn[c] = 0.0;
  for (int k0 = 0; k0 < w; k0 += kGB) {
    int32_t q[kGB];
#pragma unroll
    for (int j = 0; j < kGB; ++j) q[j] = k0 + j < w ? __ldg(slot + off + (k0 + j) * 32 + lane) : -1;
    double x[kGB][2 * LD2];
#pragma unroll
    for (int j = 0; j < kGB; ++j) {
      const int64_t qq = q[j] >= 0 ? q[j] : 0;  // padding reads slot 0, unused
#pragma unroll
      for (int k = 0; k < LD2; ++k) {
        const double2 t = __ldg(E2 + qq * RD2 + k);
        x[j][2 * k] = t.x;
        x[j][2 * k + 1] = t.y;
      }
    }
#pragma unroll
    for (int j = 0; j < kGB; ++j) {
      if (q[j] < 0) break;  // padding only after a node's last slot
#pragma unroll
      for (int c = 0; c < 5; ++c) r[c] += x[j][c];
      if constexpr (WP) {
#pragma unroll
        for (int c = 0; c < 5; ++c) {
          // v > 0 and v < 0 as integer tests of the bits (NaN and -0 in
          // neither), off GB300's narrow FP64 pipe
          const double v = x[j][5 + c];
          const long long b = __double_as_longlong(v);
          const long long mag = b & 0x7fffffffffffffffll;
          if (mag != 0 && mag <= 0x7ff0000000000000ll) {
            if (b > 0)
              pp[c] += v;
            else
              pn[c] += v;
          }
        }
      }
    }
  }
#pragma unroll
  for (int c = 0; c < 5; ++c) R[c * n + i] = r[c];
  if constexpr (WP) {
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      P[(c * 2 + 0) * n + i] = pp[c];
      P[(c * 2 + 1) * n + i] = pn[c];
    }
  }
}

// KozCG::solve (KozCG.cpp:1144-1150): A = low-order + A/vol, then U = A and
// the CFL minimum of the new state for nodes without BCs.  Aacc: the limited
// sums (F, with FCT); A: the update itself (FP64, without FCT).
template <class F>
__global__ void __launch_bounds__(kBlock) k_node_solve(int64_t n, const double* __restrict__ vol,
                                                        const double* __restrict__ R,
                                                        const F* __restrict__ Aacc,
                                                        const double* __restrict__ A, int fct,
                                                        const uint8_t* __restrict__ isbc,
                                                        double gamma, double* U,
                                                        unsigned long long* dtmin) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  double dtp = DBL_MAX;
  if (i < n) {
    double u[5];
    const double v = vol[i];
    const double iv = sizeof(F) == 4 ? 1.0 / v : 0.0;  // FP32 mode: one division
    for (int c = 0; c < 5; ++c) {
      const double a = double(Aacc[ridx<F, kAR>(n, c, i)]);
      u[c] = fct ? R[c * n + i] + (sizeof(F) == 4 ? a * iv : a / v) : A[c * n + i];
      U[c * n + i] = u[c];
    }
    if (!isbc[i]) dtp = node_dt(u, vol[i], gamma);
  }
  block_min_atomic(dtp, dtmin);
}

// KozCG::BC: Dirichlet then symmetry (physics::dirbc/symbc), one thread per
// BC node, with the node's CFL dt.
// Nodal BCs (KozCG::BC) at time t: after a step t + dt (sc->tnext,
// KozCG.cpp:1167), otherwise the caller's t_host (sc null).
__global__ void __launch_bounds__(kBlock) k_bc(int64_t n, KBC bc, double gamma, double* U,
                                                const double* __restrict__ vol, int want_dt,
                                                unsigned long long* dtmin,
                                                const KScalars* __restrict__ sc, double t_host) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  double dtp = DBL_MAX;
  if (i < bc.nbc) {
    const int64_t p = bc.node[i];
    double u[5];
    for (int c = 0; c < 5; ++c) u[c] = U[c * n + p];
    const int32_t d = bc.dir[i];
    if (d >= 0)
      dirichlet(bc.prob, bc.xyz[p], bc.xyz[n + p], bc.xyz[2 * n + p], sc ? sc->tnext : t_host,
                bc.dirmask + d * 5, bc.dirval + d * 5, u);
    for (int32_t k = bc.symp[i]; k < bc.symp[i + 1]; ++k) {
      const double* nn = bc.symn + 3 * k;
      double vn = u[1] * nn[0] + u[2] * nn[1] + u[3] * nn[2];
      u[1] -= vn * nn[0];
      u[2] -= vn * nn[1];
      u[3] -= vn * nn[2];
    }
    for (int c = 0; c < 5; ++c) U[c * n + p] = u[c];
    if (want_dt) dtp = node_dt(u, vol[p], gamma);
  }
  if (want_dt) block_min_atomic(dtp, dtmin);
}

__global__ void k_dt(int64_t n, const double* __restrict__ U, const double* __restrict__ vol,
                     double gamma, unsigned long long* dtmin) {
  int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  double dtp = DBL_MAX;
  if (p < n) {
    double u[5];
    for (int c = 0; c < 5; ++c) u[c] = U[c * n + p];
    dtp = node_dt(u, vol[p], gamma);
  }
  block_min_atomic(dtp, dtmin);
}

__global__ void k_step_begin(KScalars* s, double cfl, double const_dt, double* hist, int64_t k) {
  double dt;
  if (fabs(const_dt) > DBL_EPSILON)
    dt = const_dt;
  else
    dt = __longlong_as_double(s->dtmin) * cfl;
  if (dt < DBL_EPSILON) s->blowup = 1;
  s->dt = dt;
  s->t = s->tnext;
  s->tnext = s->t + dt;
  s->dtmin = __double_as_longlong(DBL_MAX);
  if (hist) hist[k] = dt;
}
// A step of the caller's dt from time t (its CFL minimum starts afresh).
__global__ void k_set_step(KScalars* s, double t, double dt) {
  s->t = t;
  s->dt = dt;
  s->tnext = t + dt;
  s->dtmin = __double_as_longlong(DBL_MAX);
}
__global__ void k_set_time(KScalars* s, double t) {
  s->t = t;
  s->tnext = t;
}

// The sources kozak::rhs adds (src/Physics/Kozak.cpp:125-132, 161-170): at
// every node at the step's start time, S [5][n], and at every element's
// centroid (the mean of its nodes' coordinates) half a step later, Se [ne][5].
__global__ void k_src_nodes(int64_t n, SrcPrm q, const KScalars* __restrict__ sc,
                            const double* __restrict__ xyz, double* __restrict__ S) {
  const int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (p >= n) return;
  double o[5];
  problem_source(q, xyz[p], xyz[n + p], xyz[2 * n + p], sc->t, o);
  for (int c = 0; c < 5; ++c) S[c * n + p] = o[c];
}
__global__ void k_src_elems(int64_t n, int64_t ne, SrcPrm q, const KScalars* __restrict__ sc,
                            const int32_t* __restrict__ inpoel, const double* __restrict__ xyz,
                            double* __restrict__ Se) {
  const int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (e >= ne) return;
  const int32_t* N = inpoel + e * 4;
  double c3[3];
  for (int j = 0; j < 3; ++j) {
    const double* x = xyz + j * n;
    c3[j] = (x[N[0]] + x[N[1]] + x[N[2]] + x[N[3]]) / 4.0;
  }
  double o[5];
  problem_source(q, c3[0], c3[1], c3[2], sc->t + sc->dt / 2.0, o);
  for (int c = 0; c < 5; ++c) Se[e * 5 + c] = o[c];
}

__global__ void k_reset_min(KScalars* s) { s->dtmin = __double_as_longlong(DBL_MAX); }

__global__ void k_aos_to_soa(int64_t n, int nc, const double* __restrict__ a,
                             double* __restrict__ s) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n * nc) return;
  int64_t p = i / nc;
  int c = static_cast<int>(i - p * nc);
  s[c * n + p] = a[i];
}
__global__ void k_soa_to_aos(int64_t n, int nc, const double* __restrict__ s,
                             double* __restrict__ a) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n * nc) return;
  int64_t p = i / nc;
  int c = static_cast<int>(i - p * nc);
  a[i] = s[c * n + p];
}

KBC kbc_of(KozCGDev* d) {
  return KBC{d->nbc,   d->bcnode, d->bcdir, d->bcsymp, d->dirmask,
             d->dirval, d->symn,  d->src,   d->xyz};
}

int refresh_dt(xg_ctx* c, KozCGDev* d) {
  k_reset_min<<<1, 1, 0, c->stream>>>(d->scal);
  XG_CHECK_LAUNCH(c);
  k_dt<<<blocks_for(d->n, kBlock), kBlock, 0, c->stream>>>(d->n, d->U, d->vol, d->prm.gamma,
                                                            &d->scal->dtmin);
  XG_CHECK_LAUNCH(c);
  d->dt_valid = true;
  return XG_OK;
}

// The arrays of precision F: element sums (R, P, A accumulators), the state
// the element passes read, the per-node primitives, the limit keys.
template <class F>
struct KArrays {
  F *R, *P, *A, *Uf, *V, *lo;
  typename KozT<F>::Key* Q;
  const float* geo;
};
KArrays<double> arrays64(KozCGDev* d) {
  return KArrays<double>{d->R, d->P, d->A, nullptr, d->V, d->R, d->Q, nullptr};
}
KArrays<float> arrays32(KozCGDev* d) {
  return KArrays<float>{d->R32, d->R32 + 5, d->A32, d->U32, reinterpret_cast<float*>(d->V),
                        d->lo32, d->Q32, d->geo32};
}

// Node primitives and the element Galerkin (+ antidiffusive) pass on state U
// into the node sums R, P: in FP64 the element pass fills the residual slot
// records and k_node_gather forms R (and P with FCT) in the FP64 arrays; in
// FP32 it adds into the zeroed node records k.R directly.
template <class F>
void galerkin(cudaStream_t s, KozCGDev* d, const KArrays<F>& k, const double* U, int fct) {
  const int64_t n = d->n, ne = d->ne;
  const double *S = nullptr, *Se = nullptr;
  if (d->src.problem != XG_SRC_NONE) {
    k_src_nodes<<<blocks_for(n, kBlock), kBlock, 0, s>>>(n, d->src, d->scal, d->xyz, d->S);
    k_src_elems<<<blocks_for(ne, kBlock), kBlock, 0, s>>>(n, ne, d->src, d->scal, d->inpoel,
                                                          d->xyz, d->Se);
    S = d->S;
    Se = d->Se;
  }
  k_node_prim<F><<<blocks_for(n, kBlock), kBlock, 0, s>>>(n, U, d->prm.gamma, k.V, k.Uf);
  if constexpr (sizeof(F) == 8) {
    k_elem_rhs64<<<blocks_for(ne, kEB), kEB, 0, s>>>(n, ne, d->inpoel, d->xyz, U, k.V, d->scal,
                                                     d->prm.gamma, d->prm.ctau, fct, S, Se,
                                                     d->E);
    if (fct)
      k_node_gather<kRecD2, true><<<blocks_for(n, kBlock), kBlock, 0, s>>>(
          n, d->soff, d->sw, d->sslot, d->E, d->R, d->P);
    else
      k_node_gather<kRecD2, false><<<blocks_for(n, kBlock), kBlock, 0, s>>>(
          n, d->soff, d->sw, d->sslot, d->E, d->R, nullptr);
  } else {
    k_elem_rhs_aec32<<<blocks_for(ne, kBlock), kBlock, 0, s>>>(n, ne, d->inpoel, k.geo, k.Uf, k.V,
                                                                d->scal, d->prm.gamma,
                                                                d->prm.ctau, fct, S, Se, k.R);
  }
}

// One KozCG step with the dt already in the device scalars, element
// arithmetic in F.
template <class F>
int step_impl(xg_ctx* c, KozCGDev* d, const KArrays<F>& k) {
  cudaStream_t s = c->stream;
  const int64_t n = d->n, ne = d->ne;
  const int fct = d->prm.fct;
  // FP32: R with P [n][16], A [n][8] accumulate atomically from zero; FP64:
  // R, A [5][n], P [10][n] are written whole by k_node_gather
  if (sizeof(F) == 4) {
    XG_CUDA(c, cudaMemsetAsync(k.R, 0, n * kRP * 4, s));
    if (fct) XG_CUDA(c, cudaMemsetAsync(k.A, 0, n * kAR * 4, s));
  }
  galerkin<F>(s, d, k, d->U, fct);
  XG_CHECK_LAUNCH(c);
  if (fct && d->nbc) {
    k_bc_p<F><<<blocks_for(d->nbc, kBlock), kBlock, 0, s>>>(n, kbc_of(d), k.P);
    XG_CHECK_LAUNCH(c);
  }
  const bool f32 = sizeof(F) == 4;
  k_node_lo<F><<<blocks_for(n, kBlock), kBlock, 0, s>>>(n, d->vol, d->U, d->scal, fct, k.R, k.P,
                                                         d->R, d->P, f32 ? k.lo : nullptr, d->A);
  XG_CHECK_LAUNCH(c);
  if (fct) {
    const F* Ust = f32 ? k.Uf : reinterpret_cast<const F*>(d->U);
    k_node_alw<F><<<blocks_for(n, kBlock), kBlock, 0, s>>>(n, d->aoff, d->aw, d->anbr, Ust,
                                                            k.lo, d->prm.fctclip, k.Q);
    XG_CHECK_LAUNCH(c);
    k_node_lim<F><<<blocks_for(n, kBlock), kBlock, 0, s>>>(n, d->R, d->P, k.Q);
    XG_CHECK_LAUNCH(c);
    if constexpr (sizeof(F) == 4) {
      k_elem_lim32<<<blocks_for(ne, kBlock), kBlock, 0, s>>>(n, ne, d->inpoel, k.geo, k.Uf, k.Q,
                                                              d->prm.ctau, d->prm.fctsys, k.A);
      XG_CHECK_LAUNCH(c);
    } else {
      k_elem_lim64<<<blocks_for(ne, kEB), kEB, 0, s>>>(n, ne, d->inpoel, d->E, k.Q,
                                                       d->prm.fctsys, d->L);
      XG_CHECK_LAUNCH(c);
      k_node_gather<kLimD2, false><<<blocks_for(n, kBlock), kBlock, 0, s>>>(
          n, d->soff, d->sw, d->sslot, d->L, d->A, nullptr);
      XG_CHECK_LAUNCH(c);
    }
  }
  k_node_solve<F><<<blocks_for(n, kBlock), kBlock, 0, s>>>(n, d->vol, d->R, k.A, d->A, fct,
                                                            d->isbc, d->prm.gamma, d->U,
                                                            &d->scal->dtmin);
  XG_CHECK_LAUNCH(c);
  if (d->nbc) {
    k_bc<<<blocks_for(d->nbc, kBlock), kBlock, 0, s>>>(n, kbc_of(d), d->prm.gamma, d->U, d->vol,
                                                        1, &d->scal->dtmin, d->scal, 0.0);
    XG_CHECK_LAUNCH(c);
  }
  return XG_OK;
}

int step(xg_ctx* c, KozCGDev* d) {
  if (d->prm.precision == XG_FP32_FLUX) return step_impl<float>(c, d, arrays32(d));
  return step_impl<double>(c, d, arrays64(d));
}

// The residual of FP32 node records [n][16] to FP64 [5][n].
__global__ void k_rec_to_soa(int64_t n, const float* __restrict__ a, double* __restrict__ b) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n * 5) return;
  const int64_t c = i / n, p = i - c * n;
  b[i] = double(a[p * kRP + c]);
}

}  // namespace
}  // namespace xg

using namespace xg;

extern "C" {

int xg_kozcg_setup(xg_ctx* c, const xg_kozcg_params* prm, int64_t npoin, const double* coord,
                   const double* vol, int64_t nelem, const uint64_t* inpoel) {
  XG_HOST_TRY
  int rc = use(c);
  if (rc) return rc;
  if (!prm || npoin <= 0 || nelem <= 0 || !coord || !vol || !inpoel)
    return fail(c, XG_ERR_ARG, "kozcg_setup: bad mesh");
  if (npoin >= (int64_t(1) << 31) - 64) return fail(c, XG_ERR_ARG, "kozcg_setup: too many nodes");
  if (prm->fctsys & ~31) return fail(c, XG_ERR_ARG, "kozcg_setup: fctsys mask beyond 5 components");
  if (prm->precision != XG_FP64 && prm->precision != XG_FP32_FLUX)
    return fail(c, XG_ERR_ARG, "kozcg_setup: unknown precision");
  for (int64_t i = 0; i < nelem * 4; ++i)
    if (inpoel[i] >= static_cast<uint64_t>(npoin))
      return fail(c, XG_ERR_ARG, "kozcg_setup: element node id out of range");
  // Elements in the order of their smallest node id (stable counting sort),
  // so that consecutive elements share nearby nodes: the element passes then
  // read nearby node data, and the elements holding a run of nodes (the
  // slots one warp of k_node_gather reads) lie in a window of the slot
  // records about the mesh's node bandwidth wide, instead of across the
  // whole array.  Results do not depend on the element order beyond the
  // order of each node's sums, which stays fixed.
  std::vector<int32_t> ip(nelem * 4);
  {
    std::vector<int64_t> cnt(npoin + 1, 0);
    std::vector<int32_t> key(nelem);
    for (int64_t e = 0; e < nelem; ++e) {
      uint64_t m = inpoel[e * 4];
      for (int a = 1; a < 4; ++a) m = std::min(m, inpoel[e * 4 + a]);
      key[e] = static_cast<int32_t>(m);
      ++cnt[m + 1];
    }
    for (int64_t i = 0; i < npoin; ++i) cnt[i + 1] += cnt[i];
    for (int64_t e = 0; e < nelem; ++e) {
      const int64_t to = cnt[key[e]]++;
      for (int a = 0; a < 4; ++a) ip[to * 4 + a] = static_cast<int32_t>(inpoel[e * 4 + a]);
    }
  }
  // node adjacency for the allowed limits: the elements of each node
  // (counting sort), then each node's sorted distinct element neighbours,
  // laid out as SELL-32
  const int64_t nslice = (npoin + 31) / 32;
  const bool f64 = prm->precision == XG_FP64;
  if (f64 && nelem * 4 >= (int64_t(1) << 31))
    return fail(c, XG_ERR_ARG, "kozcg_setup: too many elements for FP64 slots");
  std::vector<int32_t> aoff(nslice + 1), aw(nslice), anbr;
  // FP64 node sums: per node its (element, local node) slots e * 4 + a in
  // ascending e, SELL-32 (slice offsets soff, widths sw, -1 padding)
  std::vector<int32_t> soff(nslice + 1), sw(nslice), sslot;
  {
    std::vector<int64_t> eptr(npoin + 1, 0);
    for (int64_t i = 0; i < nelem * 4; ++i) ++eptr[ip[i] + 1];
    for (int64_t i = 0; i < npoin; ++i) eptr[i + 1] += eptr[i];
    std::vector<int32_t> eln(nelem * 4), els(f64 ? nelem * 4 : 0);
    {
      std::vector<int64_t> fill(eptr.begin(), eptr.end() - 1);
      for (int64_t e = 0; e < nelem; ++e)
        for (int a = 0; a < 4; ++a) {
          const int64_t k = fill[ip[e * 4 + a]]++;
          eln[k] = static_cast<int32_t>(e);
          if (f64) els[k] = static_cast<int32_t>(e * 4 + a);
        }
    }
    if (f64) {
      int64_t tot = 0;
      for (int64_t sl = 0; sl < nslice; ++sl) {
        int64_t w = 0;
        for (int64_t i = sl * 32; i < std::min<int64_t>(npoin, sl * 32 + 32); ++i)
          w = std::max(w, eptr[i + 1] - eptr[i]);
        soff[sl] = static_cast<int32_t>(tot);
        sw[sl] = static_cast<int32_t>(w);
        tot += 32 * w;
        if (tot >= (int64_t(1) << 31)) return fail(c, XG_ERR_ARG, "kozcg_setup: slots too many");
      }
      soff[nslice] = static_cast<int32_t>(tot);
      sslot.assign(static_cast<size_t>(std::max<int64_t>(1, tot)), -1);
      for (int64_t i = 0; i < npoin; ++i) {
        const int64_t sl = i / 32, lane = i % 32;
        for (int64_t k = eptr[i]; k < eptr[i + 1]; ++k)
          sslot[soff[sl] + (k - eptr[i]) * 32 + lane] = els[k];
      }
    }
    std::vector<int64_t> nptr(npoin + 1, 0);
    std::vector<int32_t> nb;
    nb.reserve(static_cast<size_t>(npoin) * 16);
    std::vector<int32_t> tmp;
    for (int64_t i = 0; i < npoin; ++i) {
      tmp.clear();
      for (int64_t k = eptr[i]; k < eptr[i + 1]; ++k)
        for (int a = 0; a < 4; ++a) {
          const int32_t j = ip[int64_t(eln[k]) * 4 + a];
          if (j != i) tmp.push_back(j);
        }
      std::sort(tmp.begin(), tmp.end());
      tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
      nb.insert(nb.end(), tmp.begin(), tmp.end());
      nptr[i + 1] = static_cast<int64_t>(nb.size());
    }
    int64_t tot = 0;
    for (int64_t sl = 0; sl < nslice; ++sl) {
      int64_t w = 0;
      for (int64_t i = sl * 32; i < std::min<int64_t>(npoin, sl * 32 + 32); ++i)
        w = std::max(w, nptr[i + 1] - nptr[i]);
      aoff[sl] = static_cast<int32_t>(tot);
      aw[sl] = static_cast<int32_t>(w);
      tot += 32 * w;
      if (tot >= (int64_t(1) << 31)) return fail(c, XG_ERR_ARG, "kozcg_setup: adjacency too large");
    }
    aoff[nslice] = static_cast<int32_t>(tot);
    anbr.assign(static_cast<size_t>(std::max<int64_t>(1, tot)), -1);
    for (int64_t i = 0; i < npoin; ++i) {
      const int64_t sl = i / 32, lane = i % 32;
      for (int64_t k = nptr[i]; k < nptr[i + 1]; ++k)
        anbr[aoff[sl] + (k - nptr[i]) * 32 + lane] = nb[k];
    }
  }
  if (c->kozcg) {
    XG_CUDA(c, cudaStreamSynchronize(c->stream));
    destroy_kozcg(c->kozcg);
    c->kozcg = nullptr;
  }
  auto* d = new KozCGDev;
  c->kozcg = d;
  d->n = npoin;
  d->ne = nelem;
  d->prm = *prm;
  d->nslice = nslice;
  for (int pass = 0; pass < 2; ++pass) {
    Arena& A = d->arena;
    A.plan(d->inpoel, nelem * 4);
    A.plan(d->xyz, npoin * 3);
    A.plan(d->vol, npoin);
    A.plan(d->U, npoin * 5);
    A.plan(d->R, npoin * 5);
    A.plan(d->P, npoin * 10);
    A.plan(d->Q, npoin * 10);
    A.plan(d->A, npoin * 5);
    A.plan(d->stage, npoin * 5);
    A.plan(d->V, npoin * 4);
    A.plan(d->aoff, aoff.size());
    A.plan(d->aw, aw.size());
    A.plan(d->anbr, anbr.size());
    if (prm->precision == XG_FP32_FLUX) {
      A.plan(d->R32, npoin * 16);  // R and P records
      A.plan(d->A32, npoin * 8);
      A.plan(d->U32, npoin * 5);
      A.plan(d->lo32, npoin * 5);
      A.plan(d->Q32, npoin * 10);
      A.plan(d->geo32, nelem * 10);
    } else {
      A.plan(d->E, nelem * 4 * kRecD2 * 2);
      if (prm->fct) A.plan(d->L, nelem * 4 * kLimD2 * 2);
      A.plan(d->soff, soff.size());
      A.plan(d->sw, sw.size());
      A.plan(d->sslot, sslot.size());
    }
    A.plan(d->isbc, npoin);
    A.plan(d->scal, 1);
    if (pass == 0) {
      cudaError_t e = A.reserve();
      if (e != cudaSuccess) {
        destroy_kozcg(d);
        c->kozcg = nullptr;
        return fail(c, XG_ERR_CUDA, std::string("kozcg_setup: ") + cudaGetErrorString(e));
      }
    }
  }
  cudaStream_t s = c->stream;
  XG_CUDA(c, cudaMemcpy(d->inpoel, ip.data(), ip.size() * 4, cudaMemcpyHostToDevice));
  XG_CUDA(c, cudaMemcpy(d->xyz, coord, npoin * 3 * 8, cudaMemcpyHostToDevice));
  XG_CUDA(c, cudaMemcpy(d->vol, vol, npoin * 8, cudaMemcpyHostToDevice));
  XG_CUDA(c, cudaMemcpy(d->aoff, aoff.data(), aoff.size() * 4, cudaMemcpyHostToDevice));
  XG_CUDA(c, cudaMemcpy(d->aw, aw.data(), aw.size() * 4, cudaMemcpyHostToDevice));
  XG_CUDA(c, cudaMemcpy(d->anbr, anbr.data(), anbr.size() * 4, cudaMemcpyHostToDevice));
  if (f64) {
    XG_CUDA(c, cudaMemcpy(d->soff, soff.data(), soff.size() * 4, cudaMemcpyHostToDevice));
    XG_CUDA(c, cudaMemcpy(d->sw, sw.data(), sw.size() * 4, cudaMemcpyHostToDevice));
    XG_CUDA(c, cudaMemcpy(d->sslot, sslot.data(), sslot.size() * 4, cudaMemcpyHostToDevice));
  }
  XG_CUDA(c, cudaMemsetAsync(d->U, 0, npoin * 5 * 8, s));
  XG_CUDA(c, cudaMemsetAsync(d->isbc, 0, npoin, s));
  if (d->geo32) {
    k_geo32<<<blocks_for(nelem, kBlock), kBlock, 0, s>>>(npoin, nelem, d->inpoel, d->xyz,
                                                          d->geo32);
    XG_CHECK_LAUNCH(c);
  }
  KScalars k0{};  // every member zero
  double big = DBL_MAX;
  std::memcpy(&k0.dtmin, &big, sizeof(double));
  XG_CUDA(c, cudaMemcpyAsync(d->scal, &k0, sizeof(k0), cudaMemcpyHostToDevice, s));
  XG_CUDA(c, cudaStreamSynchronize(s));
  return XG_OK;
  XG_HOST_CATCH(c)
}

int xg_kozcg_set_bc(xg_ctx* c, int64_t nsym, const uint64_t* symnodes, const double* symnorms,
                    int64_t ndir, const uint64_t* dirnodes, const int32_t* dirmask,
                    const double* dirvals) {
  XG_HOST_TRY
  int rc = use(c);
  if (rc) return rc;
  KozCGDev* d = c->kozcg;
  if (!d) return fail(c, XG_ERR_STATE, "kozcg_set_bc before kozcg_setup");
  if ((nsym && (!symnodes || !symnorms)) || (ndir && (!dirnodes || !dirmask || !dirvals)))
    return fail(c, XG_ERR_ARG, "kozcg_set_bc: null array");
  const int64_t n = d->n;
  std::vector<int64_t> ids;
  for (int64_t i = 0; i < nsym; ++i) {
    if (symnodes[i] >= uint64_t(n)) return fail(c, XG_ERR_ARG, "kozcg_set_bc: node id");
    ids.push_back(int64_t(symnodes[i]));
  }
  for (int64_t i = 0; i < ndir; ++i) {
    if (dirnodes[i] >= uint64_t(n)) return fail(c, XG_ERR_ARG, "kozcg_set_bc: node id");
    ids.push_back(int64_t(dirnodes[i]));
  }
  std::sort(ids.begin(), ids.end());
  ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
  const int64_t nbc = static_cast<int64_t>(ids.size());
  auto pos = [&](uint64_t p) {
    return static_cast<int64_t>(std::lower_bound(ids.begin(), ids.end(), int64_t(p)) - ids.begin());
  };
  std::vector<int32_t> node(nbc), dir(nbc, -1), symp(nbc + 1, 0);
  for (int64_t i = 0; i < nbc; ++i) node[i] = static_cast<int32_t>(ids[i]);
  for (int64_t k = 0; k < ndir; ++k) dir[pos(dirnodes[k])] = static_cast<int32_t>(k);
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
  std::vector<uint8_t> isbc(n, 0);
  for (auto p : ids) isbc[p] = 1;
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  d->bcarena.release();
  for (int pass = 0; pass < 2; ++pass) {
    Arena& A = d->bcarena;
    A.plan(d->bcnode, std::max<int64_t>(1, nbc));
    A.plan(d->bcdir, std::max<int64_t>(1, nbc));
    A.plan(d->bcsymp, nbc + 1);
    A.plan(d->symn, symn.size());
    A.plan(d->dirmask, std::max<int64_t>(1, ndir) * 5);
    A.plan(d->dirval, std::max<int64_t>(1, ndir) * 5);
    if (pass == 0) XG_CUDA(c, A.reserve());
  }
  auto up = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
    return bytes ? cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) : cudaSuccess;
  };
  XG_CUDA(c, up(d->bcnode, node.data(), nbc * 4));
  XG_CUDA(c, up(d->bcdir, dir.data(), nbc * 4));
  XG_CUDA(c, up(d->bcsymp, symp.data(), (nbc + 1) * 4));
  XG_CUDA(c, up(d->symn, symn.data(), symn.size() * 8));
  XG_CUDA(c, up(d->dirmask, dirmask, ndir * 5 * 4));
  XG_CUDA(c, up(d->dirval, dirvals, ndir * 5 * 8));
  XG_CUDA(c, up(d->isbc, isbc.data(), n));
  d->nbc = nbc;
  d->dt_valid = false;
  return XG_OK;
  XG_HOST_CATCH(c)
}

int xg_kozcg_set_state(xg_ctx* c, const double* U, double t) {
  int rc = use(c);
  if (rc) return rc;
  KozCGDev* d = c->kozcg;
  if (!d) return fail(c, XG_ERR_STATE, "kozcg_set_state before kozcg_setup");
  if (!U) return fail(c, XG_ERR_ARG, "kozcg_set_state: null U");
  XG_CUDA(c, cudaMemcpyAsync(d->stage, U, d->n * 5 * 8, cudaMemcpyHostToDevice, c->stream));
  k_aos_to_soa<<<blocks_for(d->n * 5, kBlock), kBlock, 0, c->stream>>>(d->n, 5, d->stage, d->U);
  XG_CHECK_LAUNCH(c);
  d->t = t;
  rc = refresh_dt(c, d);
  if (rc) return rc;
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}

int xg_kozcg_get_state(xg_ctx* c, double* U, double* t) {
  int rc = use(c);
  if (rc) return rc;
  KozCGDev* d = c->kozcg;
  if (!d) return fail(c, XG_ERR_STATE, "kozcg_get_state before kozcg_setup");
  if (U) {
    k_soa_to_aos<<<blocks_for(d->n * 5, kBlock), kBlock, 0, c->stream>>>(d->n, 5, d->U, d->stage);
    XG_CHECK_LAUNCH(c);
    XG_CUDA(c, cudaMemcpyAsync(U, d->stage, d->n * 5 * 8, cudaMemcpyDeviceToHost, c->stream));
  }
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (t) *t = d->t;
  return XG_OK;
}

int xg_kozcg_rhs(xg_ctx* c, const double* U, double dt, double* R) {
  int rc = use(c);
  if (rc) return rc;
  KozCGDev* d = c->kozcg;
  if (!d) return fail(c, XG_ERR_STATE, "kozcg_rhs before kozcg_setup");
  if (!U || !R) return fail(c, XG_ERR_ARG, "kozcg_rhs: null array");
  cudaStream_t s = c->stream;
  // use A as scratch for the caller's state so the device state is untouched
  XG_CUDA(c, cudaMemcpyAsync(d->stage, U, d->n * 5 * 8, cudaMemcpyHostToDevice, s));
  k_aos_to_soa<<<blocks_for(d->n * 5, kBlock), kBlock, 0, s>>>(d->n, 5, d->stage, d->A);
  XG_CHECK_LAUNCH(c);
  k_set_step<<<1, 1, 0, s>>>(d->scal, d->t, dt);  // the sources at the context's time
  XG_CHECK_LAUNCH(c);
  if (d->prm.precision == XG_FP32_FLUX) {
    const KArrays<float> k = arrays32(d);
    XG_CUDA(c, cudaMemsetAsync(k.R, 0, d->n * kRP * 4, s));
    galerkin<float>(s, d, k, d->A, 0);
    k_rec_to_soa<<<blocks_for(d->n * 5, kBlock), kBlock, 0, s>>>(d->n, k.R, d->R);
  } else {
    galerkin<double>(s, d, arrays64(d), d->A, 0);
  }
  XG_CHECK_LAUNCH(c);
  k_soa_to_aos<<<blocks_for(d->n * 5, kBlock), kBlock, 0, s>>>(d->n, 5, d->R, d->stage);
  XG_CHECK_LAUNCH(c);
  XG_CUDA(c, cudaMemcpyAsync(R, d->stage, d->n * 5 * 8, cudaMemcpyDeviceToHost, s));
  XG_CUDA(c, cudaStreamSynchronize(s));
  d->dt_valid = false;
  return XG_OK;
}

int xg_kozcg_dt(xg_ctx* c, double* dt) {
  int rc = use(c);
  if (rc) return rc;
  KozCGDev* d = c->kozcg;
  if (!d) return fail(c, XG_ERR_STATE, "kozcg_dt before kozcg_setup");
  if (!dt) return fail(c, XG_ERR_ARG, "kozcg_dt: null dt");
  if (!d->dt_valid) {
    rc = refresh_dt(c, d);
    if (rc) return rc;
  }
  KScalars h;
  XG_CUDA(c, cudaMemcpyAsync(&h, d->scal, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  double m;
  std::memcpy(&m, &h.dtmin, sizeof(double));
  *dt = std::fabs(d->prm.const_dt) > std::numeric_limits<double>::epsilon() ? d->prm.const_dt
                                                                             : m * d->prm.cfl;
  return XG_OK;
}

int xg_kozcg_bc(xg_ctx* c) {
  int rc = use(c);
  if (rc) return rc;
  KozCGDev* d = c->kozcg;
  if (!d) return fail(c, XG_ERR_STATE, "kozcg_bc before kozcg_setup");
  if (d->nbc) {
    k_bc<<<blocks_for(d->nbc, kBlock), kBlock, 0, c->stream>>>(
        d->n, kbc_of(d), d->prm.gamma, d->U, d->vol, 0, &d->scal->dtmin, nullptr, d->t);
    XG_CHECK_LAUNCH(c);
  }
  rc = refresh_dt(c, d);
  if (rc) return rc;
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}

int xg_kozcg_run(xg_ctx* c, int64_t nstep, double* dts, float* ms) {
  int rc = use(c);
  if (rc) return rc;
  KozCGDev* d = c->kozcg;
  if (!d) return fail(c, XG_ERR_STATE, "kozcg_run before kozcg_setup");
  if (nstep < 0) return fail(c, XG_ERR_ARG, "kozcg_run: negative step count");
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
    XG_CUDA(c, cudaMalloc(&d->dthist, nstep * sizeof(double)));
    d->dthist_cap = nstep;
  }
  k_set_time<<<1, 1, 0, c->stream>>>(d->scal, d->t);
  XG_CHECK_LAUNCH(c);
  cudaEvent_t e0, e1;
  XG_CUDA(c, cudaEventCreate(&e0));
  XG_CUDA(c, cudaEventCreate(&e1));
  XG_CUDA(c, cudaEventRecord(e0, c->stream));
  for (int64_t k = 0; k < nstep; ++k) {
    k_step_begin<<<1, 1, 0, c->stream>>>(d->scal, d->prm.cfl, d->prm.const_dt, d->dthist, k);
    XG_CHECK_LAUNCH(c);
    rc = step(c, d);
    if (rc) return rc;
  }
  XG_CUDA(c, cudaEventRecord(e1, c->stream));
  XG_CUDA(c, cudaEventSynchronize(e1));
  float el = 0.f;
  XG_CUDA(c, cudaEventElapsedTime(&el, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ms) *ms = el;
  std::vector<double> h(nstep);
  XG_CUDA(c, cudaMemcpy(h.data(), d->dthist, nstep * 8, cudaMemcpyDeviceToHost));
  for (double v : h) d->t += v;
  if (dts) std::memcpy(dts, h.data(), nstep * 8);
  d->dt_valid = true;
  KScalars s;
  XG_CUDA(c, cudaMemcpy(&s, d->scal, sizeof(s), cudaMemcpyDeviceToHost));
  if (s.blowup) return fail(c, XG_ERR_BLOWUP, "dt below machine epsilon");
  return XG_OK;
}

int xg_kozcg_step(xg_ctx* c, double dt) {
  int rc = use(c);
  if (rc) return rc;
  KozCGDev* d = c->kozcg;
  if (!d) return fail(c, XG_ERR_STATE, "kozcg_step before kozcg_setup");
  if (!(dt > 0.0) || !std::isfinite(dt)) return fail(c, XG_ERR_ARG, "kozcg_step: dt must be > 0");
  k_set_step<<<1, 1, 0, c->stream>>>(d->scal, d->t, dt);
  XG_CHECK_LAUNCH(c);
  rc = step(c, d);
  if (rc) return rc;
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  d->t += dt;
  d->dt_valid = true;  // the step's solve formed the next CFL minimum
  return XG_OK;
}

int xg_kozcg_set_source(xg_ctx* c, int problem, const double* prm) {
  int rc = use(c);
  if (rc) return rc;
  KozCGDev* d = c->kozcg;
  if (!d) return fail(c, XG_ERR_STATE, "kozcg_set_source before kozcg_setup");
  if (problem < XG_SRC_NONE || problem > XG_SRC_RAYLEIGH_TAYLOR)
    return fail(c, XG_ERR_ARG, "kozcg_set_source: unknown problem");
  if (problem != XG_SRC_NONE && problem != XG_SRC_TAYLOR_GREEN && !prm)
    return fail(c, XG_ERR_ARG, "kozcg_set_source: this problem needs its parameters");
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (problem != XG_SRC_NONE && !d->S) {
    XG_CUDA(c, cudaMalloc(&d->S, d->n * 5 * sizeof(double)));
    XG_CUDA(c, cudaMalloc(&d->Se, std::max<int64_t>(1, d->ne) * 5 * sizeof(double)));
  }
  d->src.problem = problem;
  for (int k = 0; k < 8; ++k) d->src.p[k] = prm ? prm[k] : 0.0;
  d->src.gamma = d->prm.gamma;
  return XG_OK;
}

}  // extern "C"
