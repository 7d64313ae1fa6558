// Sparse matrix and preconditioned conjugate gradients on one GB300.
//
// Reference path (paths relative to the reference project root):
//   tk::CSR                         src/LinearSolver/CSR.{hpp,cpp}
//   CSR::mult                       src/LinearSolver/CSR.cpp:154-172
//   CSR::dirichlet                  src/LinearSolver/CSR.cpp:106-152
//   ConjugateGradients::init/apply/r/setup/next/qAp/q/pq/rz/x
//                                   src/LinearSolver/ConjugateGradients.cpp:105-823
//
// Layout: the matrix is stored as SELL-32 (slices of 32 rows, each padded to
// the slice's longest row; entry k of row i at off[s] + k*32 + lane) with
// int32 columns and FP64 values.  Dirichlet elimination never rewrites the
// host matrix: a device pass builds the working values from the original
// ones and the Dirichlet mask, which is what the reference's sequential
// elimination produces (rows and columns of Dirichlet nodes zeroed, 1 on
// their diagonal), and the right-hand side correction sum_i a_ji * val_i is
// summed per row in the reference's order (decreasing node id).
//
// One PCG iteration (the reference's FP64 algorithm) is three kernels:
//   k_cg_p: p = z + beta p (beta = rho/rho0)
//   k_cg_a: q = A p, partial (p, q)
//   k_cg_b: alpha = rho/(p,q); r -= alpha q; x += alpha p; z = r/d (Jacobi,
//           as r times the stored inverse diagonal);
//           partial (r,z), (r,r); convergence test
// plus, for the factored preconditioner (pc 2, no reference counterpart),
// z = -S (I+N)(I+N)^T S r in two passes over the lower and upper triangles.
// GB300 runs FP64 arithmetic at a small fraction of its FP32 rate, so the
// FP64 kernels keep FP64 operations per row to what the algorithm needs
// (p is formed once per row, scalar divisions once per block).
// Kernels loop over rows with a grid of one wave of resident blocks, so a
// reduction has one partial per block; the last block to finish (an atomic
// ticket, no spinning) adds them in block order, so every reduction is
// deterministic.  Kernels return at once when the solve is done, so the host
// launches iterations in batches and reads the done flag once per batch.
//
// Mixed precision (xg_cg_solve_mixed): the same iteration in FP32 on an FP32
// copy of the working matrix, its columns stored as 16-bit offsets from the
// row (when every |j - i| < 32768) and the factor values in FP16, with FP64
// dot products and reliable updates: the FP32 correction e = sum alpha p' is
// folded into the FP64 x and the FP32 residual replaced by the true FP64
// residual b - A x whenever the recursive residual has fallen by the factor
// `inner_tol` since the last replacement.  The search direction is kept
// across replacements, so the FP32 iteration follows the FP64 one instead of
// restarting.  The FP32 iteration is three kernels: k_cg_a forms
// p' = z + beta p per gathered entry (FP32 arithmetic is cheap; no p pass),
// k_pc_upper_res updates r and e and applies (I+N)^T S, k_pc_lower applies
// -S (I+N) and closes the iteration.

#include <cuda_fp16.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "xg_internal.hpp"

namespace xg {

namespace {
constexpr int kSlice = 32;
constexpr int32_t kPad = -1;
constexpr int16_t kPad16 = std::numeric_limits<int16_t>::min();
constexpr int kBlock = 256;
constexpr int kBatch = 16;

struct CGScalars {
  double rho, rho0, pq, alpha, rr, normb, tol, delta, rlast;
  double pad0;
  int64_t it, maxit;
  int32_t done, finished, converged, pc;
  int32_t guard, pad1;  // 0: |(p,q)| < DBL_EPSILON ends the solve; 1: underflow only
  unsigned int ticket[4];
};
}  // namespace

struct CGDev {
  Arena arena;
  int64_t n = 0, nslice = 0, nent = 0, maxgrid = 0;
  int32_t *soff = nullptr, *swidth = nullptr, *col = nullptr;
  int16_t* col16 = nullptr;            // column - row, kPad16 for padding
  double* a0 = nullptr;                // original values (SELL order)
  double* a = nullptr;                 // working values (after Dirichlet elimination)
  float* a32 = nullptr;
  float* rs32 = nullptr;               // per row: exact (FP64) working row sum, in FP32
  int32_t* diagpos = nullptr;          // SELL index of each row's diagonal
  uint8_t* bcmask = nullptr;
  double* bcval = nullptr;
  double *x = nullptr, *b = nullptr, *r = nullptr, *q = nullptr, *z = nullptr, *d = nullptr;
  double* p[2] = {nullptr, nullptr};
  float *r32 = nullptr, *q32 = nullptr, *z32 = nullptr, *d32 = nullptr;
  double* e64 = nullptr;  // the mixed solve's correction sum alpha p', accumulated in FP64
  float* r32b = nullptr;  // second FP32 residual (factored mixed iteration, alternating)
  float* p32[2] = {nullptr, nullptr};
  double* partial = nullptr;  // 3 * maxgrid
  CGScalars* scal = nullptr;
  bool apply = false;
  bool ready = false;
  bool use16 = false;  // every |j - i| fits a 16-bit offset
  int pc = 1;
  int64_t last_it = 0;
  double last_normr = 0, last_normb = 0;
  int last_conv = 0;
  // factored approximate inverse M^-1 = -S (I+N)(I+N)^T S (pc 2): lower and
  // upper triangles of the matrix graph as SELL-32, the factor values (FP32,
  // and FP16 for the mixed solver), the row scales s = 1/sqrt|a_ii| and the
  // normalised couplings e_ij = a_ij s_i s_j
  int64_t nentL = 0, nentU = 0;
  int32_t *soffL = nullptr, *swL = nullptr, *colL = nullptr, *posL = nullptr, *tposU = nullptr;
  int32_t *soffU = nullptr, *swU = nullptr, *colU = nullptr;
  int16_t *colL16 = nullptr, *colU16 = nullptr;
  float *nvL = nullptr, *nvU = nullptr, *srow = nullptr, *eL = nullptr, *eU = nullptr;
  __half *hvL = nullptr, *hvU = nullptr;
  float* eF = nullptr;  // e_ij in the full layout (0 on the diagonal and at Dirichlet nodes)
  double *v = nullptr, *u = nullptr, *t = nullptr;  // S r, (I+N)^T S r; t: xg_cg_precondition
  float *v32 = nullptr, *u32 = nullptr;
  bool geom_set = false;
  bool factor_set = false;
  uint64_t bc_key = 0;  // hash of the Dirichlet mask the geometry was built for
  int guard = 0;        // breakdown guard of the FP64 solver (xg_cg_set_guard)
  xg_lpc* factor_model = nullptr;  // network emitting N, or null: N = factor_c * e
  double factor_c = 1.0;
};

void destroy_cg(CGDev* d) { delete d; }
size_t bytes_cg(const CGDev* d) { return d ? d->arena.bytes() : 0; }

namespace {

// ---------------------------------------------------------------- reductions

// Sum of one value per thread into partial[k * gridDim.x + blockIdx.x];
// returns true in the block that completes last (its threads then see every
// partial).  The warp sums run in A (FP32 for the FP32 solver, whose values
// are FP32: FP64 shuffles and adds per thread load GB300's narrow FP64
// pipe); the warp totals are summed in FP64.
template <int K, class A>
__device__ __forceinline__ bool block_partials(const A (&v)[K], double* partial,
                                               unsigned int* ticket) {
  __shared__ double sm[K][32];
  __shared__ bool last;
  A s[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    s[k] = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s[k] += __shfl_xor_sync(0xffffffffu, s[k], o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) sm[k][wid] = double(s[k]);
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    for (int k = 0; k < K; ++k) {
      double t = 0.0;
      for (int w = 0; w < nw; ++w) t += sm[k][w];
      partial[k * gridDim.x + blockIdx.x] = t;
    }
    __threadfence();
    unsigned int prev = atomicAdd(ticket, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  return last;
}

// In the last block: deterministic sum of the partials of component k, four
// independent lane-strided chains, then a fixed-order tree.
__device__ double sum_partials(const double* partial, int k) {
  __shared__ double red[kBlock];
  __threadfence();
  const int64_t nb = gridDim.x;
  const double* base = partial + k * nb;
  double t0 = 0.0, t1 = 0.0, t2 = 0.0, t3 = 0.0;
  int64_t i = threadIdx.x;
  for (; i + 3 * kBlock < nb; i += 4 * kBlock) {
    t0 += __ldcg(base + i);
    t1 += __ldcg(base + i + kBlock);
    t2 += __ldcg(base + i + 2 * kBlock);
    t3 += __ldcg(base + i + 3 * kBlock);
  }
  for (; i < nb; i += kBlock) t0 += __ldcg(base + i);
  red[threadIdx.x] = (t0 + t1) + (t2 + t3);
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  double r = red[0];
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------- row access

// Column of SELL entry e of row i (or -1 for padding), from int32 columns or
// 16-bit offsets.  The int32 columns and FP64 values (the FP64 solver's
// matrix stream, larger than L2) are read with the evict-first hint so that
// the gathered vectors stay in L2; the FP32 solver's narrower stream is read
// through the non-coherent cache (measured faster for it).
struct Cols32 {
  const int32_t* c;
  __device__ __forceinline__ int32_t at(int32_t e, int32_t) const { return __ldcs(c + e); }
};
struct Cols16 {
  const int16_t* c;
  __device__ __forceinline__ int32_t at(int32_t e, int32_t i) const {
    const int16_t dlt = __ldg(c + e);
    return dlt == kPad16 ? -1 : i + int32_t(dlt);
  }
};

__device__ __forceinline__ float ldv(const __half* p) { return __half2float(p[0]); }
__device__ __forceinline__ float ldv(const float* p) { return __ldg(p); }
__device__ __forceinline__ double ldv(const double* p) { return __ldcs(p); }

// sum_k val[e_k] * g(col[e_k]) over row i of a SELL-32 layout, in entry
// order, issued in groups of U entries so that U column / value loads and
// then U gathers are in flight at once (padding reads the row's own entry
// with weight 0).
template <int U, class T, class CI, class V, class G>
__device__ __forceinline__ T sell_row(CI ci, const V* __restrict__ val, int32_t off, int w,
                                      int lane, int32_t i, G g) {
  T s = T(0);
  int k = 0;
  for (; k + U <= w; k += U) {
    int32_t cc[U];
    T vv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int32_t e = off + (k + u) * kSlice + lane;
      const int32_t c = ci.at(e, i);
      vv[u] = c < 0 ? T(0) : T(ldv(val + e));
      cc[u] = c < 0 ? i : c;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) s += vv[u] * g(cc[u]);
  }
  for (; k < w; ++k) {
    const int32_t e = off + k * kSlice + lane;
    const int32_t c = ci.at(e, i);
    if (c >= 0) s += T(ldv(val + e)) * g(c);
  }
  return s;
}

// The same sum with each round fully unrolled to the exact number of entries
// left (at most XM): a row of w <= XM entries is one round, its column /
// value loads and then its gathers all in flight at once, with no predicated
// or sequential tail (the slice width is uniform across the warp, so the
// dispatch does not diverge).  Wider rows take rounds of XM.  XM bounds the
// registers of the kernel: 16 for whole rows (15 entries on a tetrahedral
// mesh of a cube), 8 for the strict triangles (7).

template <int W, class T, class CI, class V, class G>
__device__ __forceinline__ T sell_fixed(CI ci, const V* __restrict__ val, int32_t off, int lane,
                                        int32_t i, G g, T s) {
  int32_t cc[W];
  T vv[W];
#pragma unroll
  for (int u = 0; u < W; ++u) {
    const int32_t e = off + u * kSlice + lane;
    const int32_t c = ci.at(e, i);
    vv[u] = c < 0 ? T(0) : T(ldv(val + e));
    cc[u] = c < 0 ? i : c;
  }
#pragma unroll
  for (int u = 0; u < W; ++u) s += vv[u] * g(cc[u]);
  return s;
}

template <int W, int XM, class T, class CI, class V, class G>
__device__ __forceinline__ T sell_tail(int r, CI ci, const V* __restrict__ val, int32_t off,
                                       int lane, int32_t i, G g, T s) {
  if constexpr (W <= XM) {
    if (r == W) return sell_fixed<W, T>(ci, val, off, lane, i, g, s);
    return sell_tail<W + 1, XM, T>(r, ci, val, off, lane, i, g, s);
  } else {
    return s;
  }
}

template <class T, int XM = 16, class CI, class V, class G>
__device__ __forceinline__ T sell_row_x(CI ci, const V* __restrict__ val, int32_t off, int w,
                                        int lane, int32_t i, G g) {
  T s = T(0);
  int k = 0;
  for (; w - k > XM; k += XM) s = sell_fixed<XM, T>(ci, val, off + k * kSlice, lane, i, g, s);
  if (w > k) s = sell_tail<1, XM, T>(w - k, ci, val, off + k * kSlice, lane, i, g, s);
  return s;
}

// One wave of resident blocks of kernel K for n rows.
int g_nsm = 0;
template <auto K>
unsigned pgrid(int64_t n) {
  static const int per_sm = [] {
    int v = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, K, kBlock, 0) != cudaSuccess) v = 1;
    return v < 1 ? 1 : v;
  }();
  const int64_t want = (n + kBlock - 1) / kBlock;
  return static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>(want, int64_t(per_sm) * g_nsm)));
}

#define XG_ROWS(i, n) \
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < (n); \
       i += int64_t(gridDim.x) * blockDim.x)

// ---------------------------------------------------------------- launches

// The iteration kernels are launched as programmatic dependents of the
// kernel before them in the stream: their blocks may be scheduled while that
// kernel drains (its blocks trigger after their row loop, before the
// reduction tail) and wait in griddep_wait() until it has completed and its
// writes are visible.  Every kernel launched with launch_dep() calls
// griddep_wait() before it reads anything.
__device__ __forceinline__ void griddep_wait() {
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
}
__device__ __forceinline__ void griddep_trigger() {
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}

template <class... P, class... A>
void launch_dep_k(void (*k)(P...), unsigned grid, cudaStream_t s, A&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kBlock);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  (void)cudaLaunchKernelEx(&cfg, k, std::forward<A>(args)...);  // errors: cudaGetLastError
}

// Kernel K over n rows, one wave of resident blocks, as a dependent launch.
template <auto K, class... A>
void launch_dep(int64_t n, cudaStream_t s, A&&... args) {
  launch_dep_k(K, pgrid<K>(n), s, std::forward<A>(args)...);
}

// ---------------------------------------------------------------- kernels

// CSR::mult on the original values: y = A x.
__global__ void __launch_bounds__(kBlock) k_spmv(int64_t n, const int32_t* __restrict__ soff,
                                                 const int32_t* __restrict__ sw,
                                                 const int32_t* __restrict__ col,
                                                 const double* __restrict__ a,
                                                 const double* __restrict__ x,
                                                 double* __restrict__ y) {
  XG_ROWS(i, n) {
    const int lane = int(i & 31);
    y[i] = sell_row_x<double>(Cols32{col}, a, soff[i >> 5], sw[i >> 5], lane, int32_t(i),
                               [&](int32_t c) { return __ldg(x + c); });
  }
}

// Working values from the original ones and the Dirichlet mask; the
// right-hand-side correction of every non-Dirichlet row (sum over its
// Dirichlet columns in decreasing column order, CSR.cpp:130-138 as driven by
// ConjugateGradients.cpp:475-485); Dirichlet rows of b take their values
// (ConjugateGradients.cpp:542-552); Neumann contributions are added first
// (ConjugateGradients.cpp:472-473).
__global__ void k_apply_bc(int64_t n, const int32_t* __restrict__ soff,
                           const int32_t* __restrict__ sw, const int32_t* __restrict__ col,
                           const double* __restrict__ a0, double* __restrict__ a,
                           float* __restrict__ a32, const uint8_t* __restrict__ mask,
                           const double* __restrict__ val, const double* __restrict__ neu,
                           double* __restrict__ b) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int lane = int(i & 31);
  const int32_t off = soff[i >> 5], w = sw[i >> 5];
  const bool rowbc = mask[i] != 0;
  double corr = 0.0;
  for (int k = w - 1; k >= 0; --k) {
    const int32_t e = off + k * kSlice + lane;
    const int32_t c = col[e];
    if (c < 0) continue;
    double v = a0[e];
    double nv;
    if (rowbc) {
      nv = (c == i) ? 1.0 : 0.0;
    } else if (mask[c]) {
      corr += v * val[c];
      nv = 0.0;
    } else {
      nv = v;
    }
    a[e] = nv;
    a32[e] = float(nv);
  }
  double bi = b[i] + (neu ? neu[i] : 0.0);
  bi -= corr;
  if (rowbc) bi = val[i];
  b[i] = bi;
}

// rs_i = sum_j a_ij of the working matrix (FP64), stored in FP32.
__global__ void k_row_sums(int64_t n, const int32_t* __restrict__ soff,
                           const int32_t* __restrict__ sw, const int32_t* __restrict__ col,
                           const double* __restrict__ a, float* __restrict__ rs) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int lane = int(i & 31);
  const int32_t off = soff[i >> 5], w = sw[i >> 5];
  double sum = 0.0;
  for (int k = 0; k < w; ++k) {
    const int32_t e = off + k * kSlice + lane;
    if (col[e] >= 0) sum += a[e];
  }
  rs[i] = float(sum);
}

__global__ void k_copy_values(int64_t nent, const double* __restrict__ a0, double* __restrict__ a,
                              float* __restrict__ a32) {
  int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (e >= nent) return;
  a[e] = a0[e];
  a32[e] = float(a0[e]);
}

// ConjugateGradients::setup + pc + initres (ConjugateGradients.cpp:105-319):
// r = b - A x, d = 1/diag(A) (Jacobi) or 1 (none, factor), z = r d, p = r,
// partials of (b,b) and (r,z).
__global__ void __launch_bounds__(kBlock) k_setup(int64_t n, const int32_t* __restrict__ soff,
                                                   const int32_t* __restrict__ sw,
                                                   const int32_t* __restrict__ col,
                                                   const double* __restrict__ a,
                                                   const int32_t* __restrict__ diagpos,
                                                   const double* __restrict__ x,
                                                   const double* __restrict__ b,
                                                   double* __restrict__ r, double* __restrict__ d,
                                                   double* __restrict__ z, double* __restrict__ p,
                                                   float* __restrict__ d32, double* partial,
                                                   CGScalars* sc) {
  double v[2] = {0.0, 0.0};
  const int pc = sc->pc;
  XG_ROWS(i, n) {
    const int lane = int(i & 31);
    const double s = sell_row_x<double>(Cols32{col}, a, soff[i >> 5], sw[i >> 5], lane,
                                         int32_t(i), [&](int32_t c) { return x[c]; });
    const double ri = b[i] - s;
    // the inverse Jacobi diagonal: one multiply per row and iteration in
    // place of an FP64 division (the slow FP64 pipe of this GPU)
    const double di = pc == 1 ? 1.0 / a[diagpos[i]] : 1.0;
    r[i] = ri;
    d[i] = di;
    d32[i] = float(di);
    const double zi = ri * di;
    z[i] = zi;
    p[i] = ri;
    v[0] += b[i] * b[i];
    v[1] += ri * zi;
  }
  if (block_partials<2>(v, partial, &sc->ticket[0])) {
    double bb = sum_partials(partial, 0);
    double rz = sum_partials(partial, 1);
    if (threadIdx.x == 0) {
      sc->normb = sqrt(bb);
      sc->rho = rz;
      sc->it = 0;
      sc->done = 0;
      sc->finished = 0;
      sc->converged = 0;
      sc->ticket[0] = 0;
    }
  }
}

// next + qAp + q (ConjugateGradients.cpp:584-669): p' = z + beta p,
// q = A p', partial (p', q); the last block sets alpha = rho / (p', q).
// T is the vector type, V the matrix value type, CI the column encoding.
//
// beta = rho/rho0 (0 in the first iteration), formed once per block: an FP64
// division per thread would load GB300's narrow FP64 pipe.
template <class T>
__device__ __forceinline__ T block_beta(const CGScalars* sc) {
  __shared__ T beta_s;
  if (threadIdx.x == 0) beta_s = sc->it == 0 ? T(0) : T(sc->rho / sc->rho0);
  __syncthreads();
  return beta_s;
}

// p = z + beta p in place (the FP64 solver; its SpMV then gathers p alone,
// with half the FP64 operations of forming p per gathered entry).
template <class T>
__global__ void __launch_bounds__(kBlock) k_cg_p(int64_t n, const T* __restrict__ z,
                                                  T* __restrict__ p, const CGScalars* sc) {
  griddep_wait();
  if (sc->done) return;
  const T beta = block_beta<T>(sc);
  XG_ROWS(i, n) p[i] = z[i] + beta * p[i];
  griddep_trigger();
}

// q = A p', (p', q).  PF: p' = z + beta p formed per gathered entry and
// stored for the row (the FP32 solver: two gathers, no extra pass; p0/p1
// alternate with the count); otherwise p' = p0 = p1 (k_cg_p).  The FP32
// solver sums (p', q) per thread in FP32 and widens once, and forms each row
// as sum_j a_ij (p'_j - p'_i) + rs_i p'_i (rs: the row's exact sum, zero for
// an interior row of the pressure Laplacian): on a smooth p' the terms
// a_ij p'_j of the plain sum cancel to a result about 1/kappa(A) of their
// size, which FP32 cannot hold, while the differences p'_j - p'_i are
// formed exactly and nothing large cancels.
template <class T, class V, class CI, bool PF>
__global__ void __launch_bounds__(kBlock) k_cg_a(int64_t n, const int32_t* __restrict__ soff,
                                                  const int32_t* __restrict__ sw, CI ci,
                                                  const V* __restrict__ a,
                                                  const T* __restrict__ z, T* p0, T* p1,
                                                  T* __restrict__ q, double* partial,
                                                  CGScalars* sc, const float* __restrict__ rs) {
  griddep_wait();
  if (sc->done) return;
  const int64_t it = sc->it;
  const T beta = PF ? block_beta<T>(sc) : T(0);
  const T* __restrict__ pold = (it & 1) ? p1 : p0;
  T* __restrict__ pnew = (it & 1) ? p0 : p1;
  T dot = T(0);
  XG_ROWS(i, n) {
    const int lane = int(i & 31);
    if (PF) {
      const T pi = z[i] + beta * pold[i];
      const T s = sell_row_x<T>(ci, a, soff[i >> 5], sw[i >> 5], lane, int32_t(i),
                                 [&](int32_t c) {
                                   return (__ldg(z + c) + beta * __ldg(pold + c)) - pi;
                                 }) +
                  T(rs[i]) * pi;
      pnew[i] = pi;
      q[i] = s;
      dot += pi * s;
    } else {
      const T s = sell_row_x<T>(ci, a, soff[i >> 5], sw[i >> 5], lane, int32_t(i),
                                 [&](int32_t c) { return __ldg(p0 + c); });
      q[i] = s;
      dot += p0[i] * s;
    }
  }
  griddep_trigger();
  T v[1] = {dot};
  if (block_partials<1>(v, partial, &sc->ticket[1])) {
    double pq = sum_partials(partial, 0);
    if (threadIdx.x == 0) {
      sc->rho0 = sc->rho;
      sc->pq = pq;
      // the reference's breakdown guard is an absolute epsilon
      // (ConjugateGradients.cpp:681-690); the FP32 solver, and the FP64 one
      // with guard 1, guard underflow only
      const double eps = (sizeof(T) == 8 && sc->guard == 0) ? DBL_EPSILON : DBL_MIN;
      if (fabs(pq) < eps) {
        sc->finished = 1;
        sc->alpha = 0.0;
      } else {
        sc->alpha = sc->rho / pq;
      }
      sc->ticket[1] = 0;
    }
  }
}

// The end of an iteration, in the last block: (r,r), the count and the
// stopping test (ConjugateGradients.cpp:772-823):
//   FP64: ||r|| < tol ||b||, or maxit iterations (the reference's test);
//   MIXED: ||r|| < max(tol ||b||, delta * rlast) asks for a residual
//   replacement (rlast: the last true residual norm), as does maxit.
template <bool MIXED>
__device__ __forceinline__ void end_iteration(double rr, CGScalars* sc) {
  sc->rr = rr;
  sc->it += 1;
  const double nr = sqrt(rr);
  const double nb = sc->normb > 1.0e-14 ? sc->normb : 1.0;
  if (MIXED) {
    const double lim = fmax(sc->tol * nb, sc->delta * sc->rlast);
    if (sc->finished || nr < lim || sc->it >= sc->maxit) sc->done = 1;
  } else {
    if (sc->finished || nr < sc->tol * nb || sc->it >= sc->maxit) {
      sc->done = 1;
      sc->converged = nr > sc->tol * nb ? 0 : 1;
    }
  }
}

// pq + rz + x (ConjugateGradients.cpp:671-823), fused: r -= alpha q,
// x += alpha p'; Jacobi z = r d (d the inverse diagonal), rho = (r, z), or
// (FACTOR) v = S r for
// the factor passes that follow; (r, r) and the stopping test:
//   FP64: ||r|| < tol ||b||, or maxit iterations (the reference's test);
//   MIXED: ||r|| < max(tol ||b||, delta * rlast) asks for a residual
//   replacement (rlast: the last true residual norm), as does maxit.
// x is the FP64 solution (FP64 solver) or the mixed solver's FP64 correction
// e, summed with exact FP64 products alpha p'.
template <class T, bool FACTOR, bool MIXED>
__global__ void __launch_bounds__(kBlock) k_cg_b(int64_t n, const T* __restrict__ q,
                                                  const T* __restrict__ d, const T* p0,
                                                  const T* p1, const float* __restrict__ srow,
                                                  T* __restrict__ r, T* __restrict__ z,
                                                  T* __restrict__ vs, double* __restrict__ x,
                                                  double* partial, CGScalars* sc) {
  griddep_wait();
  if (sc->done) return;
  const T alpha = T(sc->alpha);
  // the p' of this iteration (k_cg_a wrote it; the count advances below, or
  // at the end of the factor passes)
  const T* __restrict__ p = (sc->it & 1) ? p0 : p1;
  if (FACTOR) {
    // no reduction here: (r,z), (r,r) and the stopping test close the
    // iteration in k_pc_lower
    XG_ROWS(i, n) {
      const T ri = r[i] - alpha * q[i];
      r[i] = ri;
      x[i] += double(alpha) * double(p[i]);
      vs[i] = T(srow[i]) * ri;
    }
    griddep_trigger();
    return;
  }
  T rz = T(0), rr = T(0);  // per thread in T, widened in block_partials
  XG_ROWS(i, n) {
    const T ri = r[i] - alpha * q[i];
    r[i] = ri;
    x[i] += double(alpha) * double(p[i]);
    const T zi = ri * d[i];
    z[i] = zi;
    rz += ri * zi;
    rr += ri * ri;
  }
  griddep_trigger();
  const T v[2] = {rz, rr};
  if (block_partials<2>(v, partial, &sc->ticket[2])) {
    double rz = sum_partials(partial, 0);
    double rr = sum_partials(partial, 1);
    if (threadIdx.x == 0) {
      sc->rho = rz;
      end_iteration<MIXED>(rr, sc);
      sc->ticket[2] = 0;
    }
  }
}

// ---- factored approximate inverse (pc 2)

// u = (I+N)^T v: u_i = v_i + sum_{j>i} N_ji v_j (upper layout of N).
template <class T, class V, class CI>
__global__ void __launch_bounds__(kBlock) k_pc_upper(int64_t n, const int32_t* __restrict__ soffU,
                                                      const int32_t* __restrict__ swU, CI ci,
                                                      const V* __restrict__ nvU,
                                                      const T* __restrict__ vs,
                                                      T* __restrict__ u,
                                                      const CGScalars* __restrict__ sc) {
  griddep_wait();
  if (sc->done) return;
  XG_ROWS(i, n) {
    const int lane = int(i & 31);
    u[i] = vs[i] + sell_row_x<T, 8>(ci, nvU, soffU[i >> 5], swU[i >> 5], lane, int32_t(i),
                                  [&](int32_t c) { return __ldg(vs + c); });
  }
}

// The update of a factored FP32 iteration fused with the first factor pass:
// r' = r - alpha q, e += alpha p' (in FP64: FP32 rounding noise in the
// correction would be amplified by A's largest eigenvalues into the residual
// the outer loop replaces), u = (I+N)^T S r', with the neighbours'
// S r' formed from their r and q.  The residual alternates between ra and rb
// with the count (the current one is ra at even counts): the pass reads one
// and writes the other, so no row reads a residual that another row of the
// same pass has replaced.
template <class CI>
__global__ void __launch_bounds__(kBlock, 5) k_pc_upper_res(
    int64_t n, const int32_t* __restrict__ soffU, const int32_t* __restrict__ swU, CI ci,
    const __half* __restrict__ nvU, const float* __restrict__ srow, const float* __restrict__ q,
    const float* p0, const float* p1, float* ra, float* rb, double* __restrict__ e,
    float* __restrict__ u, const CGScalars* __restrict__ sc) {
  griddep_wait();
  if (sc->done) return;
  const float alpha = float(sc->alpha);
  const int64_t it = sc->it;
  const float* __restrict__ p = (it & 1) ? p0 : p1;
  const float* __restrict__ rold = (it & 1) ? rb : ra;
  float* __restrict__ rnew = (it & 1) ? ra : rb;
  XG_ROWS(i, n) {
    const int lane = int(i & 31);
    const float ri = rold[i] - alpha * q[i];
    rnew[i] = ri;
    e[i] += double(alpha) * double(p[i]);
    u[i] = srow[i] * ri +
           sell_row_x<float, 8>(ci, nvU, soffU[i >> 5], swU[i >> 5], lane, int32_t(i),
                              [&](int32_t c) {
                                return __ldg(srow + c) * (__ldg(rold + c) - alpha * __ldg(q + c));
                              });
  }
}

// z = -S (I+N) u (Dirichlet rows: z = r), partial (r,z); the last block
// stores rho = (r,z).  MODE 0 applies the preconditioner only; MODE 1 (FP64)
// and MODE 2 (mixed) also close a CG iteration: partial (r,r), the count and
// the stopping test.
template <class T, class V, class CI, int MODE>
__global__ void __launch_bounds__(kBlock, sizeof(T) == 4 ? 6 : 1) k_pc_lower(int64_t n, const int32_t* __restrict__ soffL,
                                                      const int32_t* __restrict__ swL, CI ci,
                                                      const V* __restrict__ nvL,
                                                      const float* __restrict__ srow,
                                                      const uint8_t* __restrict__ mask,
                                                      const T* __restrict__ u,
                                                      const T* r_even, const T* r_odd,
                                                      T* __restrict__ z, double* partial,
                                                      CGScalars* sc) {
  griddep_wait();
  if (sc->done) return;
  // the residual: r_even unless it alternates (r_odd given), then the one
  // k_pc_upper_res wrote (MODE 2) or the current one (MODE 0)
  const bool odd = r_odd && (((sc->it + (MODE == 2 ? 1 : 0)) & 1) != 0);
  const T* __restrict__ r = odd ? r_odd : r_even;
  T rz = T(0), rr = T(0);  // per thread in T (FP32 for the mixed solver), widened once
  XG_ROWS(i, n) {
    const int lane = int(i & 31);
    const T acc = u[i] + sell_row_x<T, 8>(ci, nvL, soffL[i >> 5], swL[i >> 5], lane, int32_t(i),
                                        [&](int32_t c) { return __ldg(u + c); });
    const T ri = r[i];
    const T zi = mask[i] ? ri : -T(srow[i]) * acc;
    z[i] = zi;
    rz += ri * zi;
    if (MODE > 0) rr += ri * ri;
  }
  griddep_trigger();
  T v[2] = {rz, rr};
  if (MODE == 0) {
    T w[1] = {v[0]};
    if (block_partials<1>(w, partial, &sc->ticket[3])) {
      double rz = sum_partials(partial, 0);
      if (threadIdx.x == 0) {
        sc->rho = rz;
        sc->ticket[3] = 0;
      }
    }
  } else if (block_partials<2>(v, partial, &sc->ticket[3])) {
    double rz = sum_partials(partial, 0);
    double rr = sum_partials(partial, 1);
    if (threadIdx.x == 0) {
      sc->rho = rz;
      end_iteration<MODE == 2>(rr, sc);
      sc->ticket[3] = 0;
    }
  }
}

// v = S r
template <class T>
__global__ void k_scale(int64_t n, const float* __restrict__ srow, const T* __restrict__ r,
                        T* __restrict__ v) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i < n) v[i] = T(srow[i]) * r[i];
}

// ---- mixed precision: residual replacement

// r = b - A x in FP64 (true residual), r32 = r; Jacobi: z32 = r32 d32 and
// rho = (r32, z32); factor (srow given): v32 = S r32.  Partial (r,r) -> rr.
// FIRST starts the FP32 iteration (it = 0, so beta = 0); otherwise it
// continues with the kept search direction.
__global__ void __launch_bounds__(kBlock) k_outer_res(int64_t n, const int32_t* __restrict__ soff,
                                                       const int32_t* __restrict__ sw,
                                                       const int32_t* __restrict__ col,
                                                       const double* __restrict__ a,
                                                       const double* __restrict__ x,
                                                       const double* __restrict__ b,
                                                       const float* __restrict__ d32,
                                                       const float* __restrict__ srow,
                                                       float* r32, float* r32b,
                                                       float* __restrict__ z32,
                                                       float* __restrict__ v32, int first,
                                                       double* partial, CGScalars* sc) {
  // the current residual buffer (it alternates in the factored iteration)
  float* __restrict__ rout = (r32b && !first && (sc->it & 1)) ? r32b : r32;
  double v[2] = {0.0, 0.0};
  XG_ROWS(i, n) {
    const int lane = int(i & 31);
    const double s = sell_row_x<double>(Cols32{col}, a, soff[i >> 5], sw[i >> 5], lane,
                                         int32_t(i), [&](int32_t c) { return __ldg(x + c); });
    const double ri = b[i] - s;
    const float rf = float(ri);
    rout[i] = rf;
    if (srow) {
      v32[i] = srow[i] * rf;
    } else {
      const float zf = rf * d32[i];
      z32[i] = zf;
      v[1] += double(rf) * double(zf);
    }
    v[0] += ri * ri;
  }
  if (block_partials<2>(v, partial, &sc->ticket[0])) {
    double rr = sum_partials(partial, 0);
    double rz = sum_partials(partial, 1);
    if (threadIdx.x == 0) {
      sc->rr = rr;
      if (!srow) sc->rho = rz;
      if (first) sc->it = 0;
      sc->done = 0;
      sc->finished = 0;
      sc->ticket[0] = 0;
    }
  }
}

// x += e, e = 0
__global__ void k_add_correction(int64_t n, double* __restrict__ e, double* __restrict__ x) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i < n) {
    x[i] += e[i];
    e[i] = 0.0;
  }
}

__global__ void k_jacobi_apply(int64_t n, const double* __restrict__ r, const double* __restrict__ d,
                               double* __restrict__ z) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i < n) z[i] = r[i] * d[i];
}

// ---- factor construction

// Row scales s_i = 1/sqrt|a_ii| of the working matrix.
__global__ void k_factor_geom(int64_t n, const double* __restrict__ a,
                              const int32_t* __restrict__ diagpos, float* __restrict__ srow) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  srow[i] = float(1.0 / sqrt(fabs(a[diagpos[i]])));
}
// e_ij = a_ij s_i s_j (0 when i or j is a Dirichlet node) in the lower and
// upper layouts.
__global__ void k_factor_e(int64_t n, const int32_t* __restrict__ soffL,
                           const int32_t* __restrict__ swL, const int32_t* __restrict__ colL,
                           const int32_t* __restrict__ posL, const int32_t* __restrict__ tposU,
                           const double* __restrict__ a, const float* __restrict__ srow,
                           const uint8_t* __restrict__ mask, float* __restrict__ eL,
                           float* __restrict__ eU) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int lane = int(i & 31);
  const int32_t off = soffL[i >> 5], w = swL[i >> 5];
  for (int k = 0; k < w; ++k) {
    const int32_t e = off + k * kSlice + lane;
    const int32_t j = colL[e];
    if (j < 0) continue;
    const float v = (mask[i] || mask[j]) ? 0.f : float(a[posL[e]]) * srow[i] * srow[j];
    eL[e] = v;
    eU[tposU[e]] = v;
  }
}
// e_ij in the full layout.
__global__ void k_factor_efull(int64_t n, const int32_t* __restrict__ soff,
                               const int32_t* __restrict__ sw, const int32_t* __restrict__ col,
                               const double* __restrict__ a, const float* __restrict__ srow,
                               const uint8_t* __restrict__ mask, float* __restrict__ eF) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int lane = int(i & 31);
  const int32_t off = soff[i >> 5], w = sw[i >> 5];
  for (int k = 0; k < w; ++k) {
    const int32_t e = off + k * kSlice + lane;
    const int32_t j = col[e];
    eF[e] = (j < 0 || j == i || mask[i] || mask[j]) ? 0.f : float(a[e]) * srow[i] * srow[j];
  }
}
// N_ij = c e_ij (the first-order factor, c = 1, or any uniform scaling), in
// the lower layout and, transposed, the upper one.
__global__ void k_factor_scaled(int64_t n, const int32_t* __restrict__ soffL,
                                const int32_t* __restrict__ swL, const int32_t* __restrict__ colL,
                                const int32_t* __restrict__ tposU, const float* __restrict__ eL,
                                float c, float* __restrict__ nvL, float* __restrict__ nvU) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int lane = int(i & 31);
  const int32_t off = soffL[i >> 5], w = swL[i >> 5];
  for (int k = 0; k < w; ++k) {
    const int32_t e = off + k * kSlice + lane;
    const int32_t j = colL[e];
    if (j < 0) continue;
    const float v = c * eL[e];
    nvL[e] = v;
    nvU[tposU[e]] = v;
  }
}
__global__ void k_to_half(int64_t m, const float* __restrict__ a, __half* __restrict__ h) {
  int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (e < m) h[e] = __float2half_rn(a[e]);
}

// ---------------------------------------------------------------- host helpers

int read_scal(xg_ctx* c, CGDev* d, CGScalars* h) {
  XG_CUDA(c, cudaMemcpyAsync(h, d->scal, sizeof(CGScalars), cudaMemcpyDeviceToHost, c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}
int write_scal(xg_ctx* c, CGDev* d, const CGScalars* h) {
  XG_CUDA(c, cudaMemcpyAsync(d->scal, h, sizeof(CGScalars), cudaMemcpyHostToDevice, c->stream));
  // h lives on the caller's stack frame: complete the copy before returning
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}

// Row scales and normalised couplings of the current working matrix.
int build_geom(xg_ctx* c, CGDev* d) {
  cudaStream_t s = c->stream;
  const unsigned nb = blocks_for(d->n, kBlock);
  k_factor_geom<<<nb, kBlock, 0, s>>>(d->n, d->a, d->diagpos, d->srow);
  XG_CHECK_LAUNCH(c);
  k_factor_e<<<nb, kBlock, 0, s>>>(d->n, d->soffL, d->swL, d->colL, d->posL, d->tposU, d->a,
                                   d->srow, d->bcmask, d->eL, d->eU);
  XG_CHECK_LAUNCH(c);
  k_factor_efull<<<nb, kBlock, 0, s>>>(d->n, d->soff, d->swidth, d->col, d->a, d->srow, d->bcmask,
                                       d->eF);
  XG_CHECK_LAUNCH(c);
  d->geom_set = true;
  return XG_OK;
}

LpcGraph graph_of(const CGDev* d) {
  LpcGraph g;
  g.n = d->n;
  g.nslice = d->nslice;
  g.soff = d->soff;
  g.sw = d->swidth;
  g.col = d->col;
  g.eF = d->eF;
  g.soffL = d->soffL;
  g.swL = d->swL;
  g.colL = d->colL;
  g.eL = d->eL;
  g.tposU = d->tposU;
  g.soffU = d->soffU;
  g.swU = d->swU;
  g.colU = d->colU;
  g.eU = d->eU;
  g.srow = d->srow;
  g.mask = d->bcmask;
  g.nentL = d->nentL;
  g.nentU = d->nentU;
  return g;
}

// Scales, couplings and factor values (FP32 and FP16) of the current
// working matrix.
int build_factor(xg_ctx* c, CGDev* d) {
  cudaStream_t s = c->stream;
  const unsigned nb = blocks_for(d->n, kBlock);
  if (!d->geom_set) {
    int rg = build_geom(c, d);
    if (rg) return rg;
  }
  if (d->factor_model) {
    int rc = lpc_factor(c, d->factor_model, graph_of(d), d->nvL, d->nvU);
    if (rc) return rc;
  } else {
    k_factor_scaled<<<nb, kBlock, 0, s>>>(d->n, d->soffL, d->swL, d->colL, d->tposU, d->eL,
                                          float(d->factor_c), d->nvL, d->nvU);
    XG_CHECK_LAUNCH(c);
  }
  k_to_half<<<blocks_for(std::max<int64_t>(1, d->nentL), kBlock), kBlock, 0, s>>>(d->nentL, d->nvL,
                                                                                  d->hvL);
  k_to_half<<<blocks_for(std::max<int64_t>(1, d->nentU), kBlock), kBlock, 0, s>>>(d->nentU, d->nvU,
                                                                                  d->hvU);
  XG_CHECK_LAUNCH(c);
  d->factor_set = true;
  return XG_OK;
}

// z = M^-1 r with the factor in FP64 vectors (FP32 values): v = S r, then the
// two passes; rho = (r, z).
int factor_apply64(xg_ctx* c, CGDev* d, const double* r, double* z) {
  cudaStream_t s = c->stream;
  const int64_t n = d->n;
  k_scale<double><<<blocks_for(n, kBlock), kBlock, 0, s>>>(n, d->srow, r, d->v);
  launch_dep<k_pc_upper<double, float, Cols32>>(n, s, n, d->soffU, d->swU, Cols32{d->colU}, d->nvU,
      d->v, d->u, d->scal);
  launch_dep<k_pc_lower<double, float, Cols32, 0>>(n, s, n, d->soffL, d->swL, Cols32{d->colL},
      d->nvL, d->srow, d->bcmask, d->u, r, nullptr, z, d->partial, d->scal);
  XG_CHECK_LAUNCH(c);
  return XG_OK;
}

// The FP32 factor passes on v32 = S r (already written, r the current
// residual): z32 and rho = (r, z32).
template <class CI>
void factor_apply32(xg_ctx* c, CGDev* d, CI cu, CI cl) {
  cudaStream_t s = c->stream;
  const int64_t n = d->n;
  launch_dep<k_pc_upper<float, __half, CI>>(n, s, n, d->soffU, d->swU, cu, d->hvU, d->v32, d->u32,
      d->scal);
  launch_dep<k_pc_lower<float, __half, CI, 0>>(n, s, n, d->soffL, d->swL, cl, d->hvL, d->srow,
      d->bcmask, d->u32, d->r32, d->r32b, d->z32, d->partial, d->scal);
}

int cg_iterate(xg_ctx* c, CGDev* d, int64_t maxit, double tol, CGScalars* h) {
  cudaStream_t s = c->stream;
  // tol and maxit into the device scalars without touching the rest
  XG_CUDA(c, cudaMemcpyAsync(&d->scal->tol, &tol, sizeof(double), cudaMemcpyHostToDevice, s));
  XG_CUDA(c, cudaMemcpyAsync(&d->scal->maxit, &maxit, sizeof(int64_t), cudaMemcpyHostToDevice, s));
  const int64_t n = d->n;
  for (;;) {
    for (int k = 0; k < kBatch; ++k) {
      double* p0 = d->p[0];
      launch_dep<k_cg_p<double>>(n, s, n, d->z, p0, d->scal);
      launch_dep<k_cg_a<double, double, Cols32, false>>(n, s, n, d->soff, d->swidth, Cols32{d->col},
          d->a, d->z, p0, p0, d->q, d->partial, d->scal, static_cast<const float*>(nullptr));
      if (d->pc == 2) {
        launch_dep<k_cg_b<double, true, false>>(n, s, n, d->q, d->d, p0, p0, d->srow, d->r, d->z,
            d->v, d->x, d->partial, d->scal);
        launch_dep<k_pc_upper<double, float, Cols32>>(n, s, n, d->soffU, d->swU, Cols32{d->colU},
            d->nvU, d->v, d->u, d->scal);
        launch_dep<k_pc_lower<double, float, Cols32, 1>>(n, s, n, d->soffL, d->swL, Cols32{d->colL},
            d->nvL, d->srow, d->bcmask, d->u, d->r, nullptr, d->z, d->partial, d->scal);
      } else {
        launch_dep<k_cg_b<double, false, false>>(n, s, n, d->q, d->d, p0, p0, d->srow, d->r, d->z,
            d->v, d->x, d->partial, d->scal);
      }
    }
    XG_CHECK_LAUNCH(c);
    int rc = read_scal(c, d, h);
    if (rc) return rc;
    if (h->done) break;
  }
  return XG_OK;
}

// A batch of FP32 iterations with column encoding CI.  Factored: q = A p'
// (k_cg_a), the update with u = (I+N)^T S r' (k_pc_upper_res), then
// z = -S (I+N) u closing the iteration (k_pc_lower); Jacobi: k_cg_a, k_cg_b.
template <class CI>
int mixed_batch(xg_ctx* c, CGDev* d, CI ca, CI cu, CI cl) {
  cudaStream_t s = c->stream;
  const int64_t n = d->n;
  for (int k = 0; k < kBatch; ++k) {
    float *p0 = d->p32[0], *p1 = d->p32[1];
    launch_dep<k_cg_a<float, float, CI, true>>(n, s, n, d->soff, d->swidth, ca, d->a32, d->z32, p0,
        p1, d->q32, d->partial, d->scal, static_cast<const float*>(d->rs32));
    if (d->pc == 2) {
      launch_dep<k_pc_upper_res<CI>>(n, s, n, d->soffU, d->swU, cu, d->hvU, d->srow, d->q32, p0, p1,
          d->r32, d->r32b, d->e64, d->u32, d->scal);
      launch_dep<k_pc_lower<float, __half, CI, 2>>(n, s, n, d->soffL, d->swL, cl, d->hvL, d->srow,
          d->bcmask, d->u32, d->r32, d->r32b, d->z32, d->partial, d->scal);
    } else {
      launch_dep<k_cg_b<float, false, true>>(n, s, n, d->q32, d->d32, p0, p1, d->srow, d->r32,
          d->z32, d->v32, d->e64, d->partial, d->scal);
    }
  }
  XG_CHECK_LAUNCH(c);
  return XG_OK;
}

// True residual into the FP32 iteration (and the factor passes for z32).
int replace_residual(xg_ctx* c, CGDev* d, int first) {
  cudaStream_t s = c->stream;
  const int64_t n = d->n;
  k_outer_res<<<pgrid<k_outer_res>(n), kBlock, 0, s>>>(
      n, d->soff, d->swidth, d->col, d->a, d->x, d->b, d->d32, d->pc == 2 ? d->srow : nullptr,
      d->r32, d->pc == 2 ? d->r32b : nullptr, d->z32, d->v32, first, d->partial, d->scal);
  XG_CHECK_LAUNCH(c);
  if (d->pc == 2) {
    if (d->use16)
      factor_apply32(c, d, Cols16{d->colU16}, Cols16{d->colL16});
    else
      factor_apply32(c, d, Cols32{d->colU}, Cols32{d->colL});
    XG_CHECK_LAUNCH(c);
  }
  return XG_OK;
}

}  // namespace

int cg_graph(xg_ctx* c, LpcGraph* g) {
  CGDev* d = c->cg;
  if (!d || !d->ready) return fail(c, XG_ERR_STATE, "learned preconditioner: no initialised CG system");
  if (!d->geom_set) {
    int rc = build_geom(c, d);
    if (rc) return rc;
  }
  *g = graph_of(d);
  return XG_OK;
}

int cg_set_dirichlet(xg_ctx* c, const uint8_t* mask, const double* val) {
  CGDev* d = c->cg;
  if (!d) return fail(c, XG_ERR_STATE, "pressure Dirichlet data before cg_setup");
  const int64_t n = d->n;
  uint64_t key = 1469598103934665603ull;  // FNV-1a over the mask, as xg_cg_init
  for (int64_t i = 0; i < n; ++i) key = (key ^ mask[i]) * 1099511628211ull;
  XG_CUDA(c, cudaMemcpyAsync(d->bcmask, mask, n, cudaMemcpyHostToDevice, c->stream));
  XG_CUDA(c, cudaMemcpyAsync(d->bcval, val, n * 8, cudaMemcpyHostToDevice, c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (key != d->bc_key || !d->ready) {
    d->geom_set = false;
    d->factor_set = false;
  }
  d->bc_key = key;
  return XG_OK;
}

int cg_zero_solution(xg_ctx* c) {
  CGDev* d = c->cg;
  if (!d) return fail(c, XG_ERR_STATE, "cg_zero_solution before cg_setup");
  XG_CUDA(c, cudaMemsetAsync(d->x, 0, d->n * 8, c->stream));
  return XG_OK;
}

int cg_init_device(xg_ctx* c, const double* b_dev, int zero_values, int pc) {
  CGDev* d = c->cg;
  if (!d) return fail(c, XG_ERR_STATE, "cg_init_device before cg_setup");
  if (pc != 0 && pc != 1 && pc != 2) return fail(c, XG_ERR_ARG, "unknown preconditioner");
  cudaStream_t s = c->stream;
  const int64_t n = d->n;
  XG_CUDA(c, cudaMemcpyAsync(d->b, b_dev, n * 8, cudaMemcpyDeviceToDevice, s));
  const double* val = d->bcval;
  if (zero_values) {  // r is free until k_setup writes it
    XG_CUDA(c, cudaMemsetAsync(d->r, 0, n * 8, s));
    val = d->r;
  }
  d->pc = pc;
  d->apply = true;
  k_apply_bc<<<blocks_for(n, kBlock), kBlock, 0, s>>>(n, d->soff, d->swidth, d->col, d->a0, d->a,
                                                       d->a32, d->bcmask, val, nullptr, d->b);
  XG_CHECK_LAUNCH(c);
  k_row_sums<<<blocks_for(n, kBlock), kBlock, 0, s>>>(n, d->soff, d->swidth, d->col, d->a,
                                                      d->rs32);
  XG_CHECK_LAUNCH(c);
  CGScalars h{};
  h.pc = pc;
  h.guard = d->guard;
  XG_CUDA(c, cudaMemcpyAsync(d->scal, &h, sizeof(h), cudaMemcpyHostToDevice, s));
  k_setup<<<pgrid<k_setup>(n), kBlock, 0, s>>>(n, d->soff, d->swidth, d->col, d->a, d->diagpos,
                                               d->x, d->b, d->r, d->d, d->z, d->p[0], d->d32,
                                               d->partial, d->scal);
  XG_CHECK_LAUNCH(c);
  d->ready = true;
  if (pc == 2) {
    int rf = d->factor_set ? XG_OK : build_factor(c, d);
    if (rf) return rf;
    rf = factor_apply64(c, d, d->r, d->z);
    if (rf) return rf;
  }
  return XG_OK;
}

const double* cg_solution_device(xg_ctx* c) { return c->cg ? c->cg->x : nullptr; }
int64_t cg_rows(xg_ctx* c) { return c->cg ? c->cg->n : 0; }

// Values in CSR order, on the row pattern ia (zero-based, the pattern the
// context's system was set up with), into that system's SELL-32 layout: entry
// j of row i at soff[i / 32] + (j - ia[i]) 32 + i % 32, with the slice widths
// xg_cg_setup forms; padding entries 0.  dev_out holds nent() doubles.
int cg_to_sell(xg_ctx* c, const uint64_t* ia, const double* csr, double* dev_out) {
  CGDev* d = c->cg;
  if (!d) return fail(c, XG_ERR_STATE, "cg_to_sell before cg_setup");
  const int64_t nrow = d->n, nslice = (nrow + kSlice - 1) / kSlice;
  std::vector<int64_t> soff(nslice + 1, 0);
  for (int64_t s = 0; s < nslice; ++s) {
    uint64_t w = 0;
    for (int64_t i = s * kSlice; i < std::min(nrow, (s + 1) * kSlice); ++i)
      w = std::max<uint64_t>(w, ia[i + 1] - ia[i]);
    soff[s + 1] = soff[s] + int64_t(w) * kSlice;
  }
  if (soff[nslice] != d->nent) return fail(c, XG_ERR_ARG, "cg_to_sell: pattern mismatch");
  std::vector<double> v(static_cast<size_t>(d->nent), 0.0);
  for (int64_t i = 0; i < nrow; ++i) {
    const int64_t s = i / kSlice, lane = i % kSlice;
    for (uint64_t j = ia[i]; j < ia[i + 1]; ++j)
      v[soff[s] + int64_t(j - ia[i]) * kSlice + lane] = csr[j];
  }
  XG_CUDA(c, cudaMemcpy(dev_out, v.data(), v.size() * 8, cudaMemcpyHostToDevice));
  return XG_OK;
}
int64_t cg_nent(xg_ctx* c) { return c->cg ? c->cg->nent : 0; }
// The working values the solves read are formed from these originals.
double* cg_values_device(xg_ctx* c) { return c->cg ? c->cg->a0 : nullptr; }

}  // namespace xg

using namespace xg;

extern "C" {

int xg_cg_setup(xg_ctx* c, int64_t nrow, const uint64_t* ia, const uint64_t* ja, const double* a,
                int base) {
  XG_HOST_TRY
  int rc = use(c);
  if (rc) return rc;
  if (nrow <= 0 || !ia || !ja || !a || (base != 0 && base != 1))
    return fail(c, XG_ERR_ARG, "cg_setup: bad matrix");
  if (nrow >= (int64_t(1) << 31) - 64) return fail(c, XG_ERR_ARG, "cg_setup: too many rows");
  const uint64_t b0 = static_cast<uint64_t>(base);
  if (ia[0] != b0) return fail(c, XG_ERR_ARG, "cg_setup: ia[0] must equal the index base");
  std::vector<int32_t> diagk(nrow, -1);
  bool fits16 = true;
  for (int64_t i = 0; i < nrow; ++i) {
    if (ia[i + 1] < ia[i]) return fail(c, XG_ERR_ARG, "cg_setup: ia not monotonic");
    for (uint64_t j = ia[i]; j < ia[i + 1]; ++j) {
      uint64_t cc = ja[j - b0] - b0;
      if (cc >= static_cast<uint64_t>(nrow)) return fail(c, XG_ERR_ARG, "cg_setup: column id");
      if (static_cast<int64_t>(cc) == i) diagk[i] = static_cast<int32_t>(j - ia[i]);
      const int64_t dl = static_cast<int64_t>(cc) - i;
      if (dl <= int64_t(kPad16) || dl > int64_t(std::numeric_limits<int16_t>::max()))
        fits16 = false;
    }
    if (diagk[i] < 0) return fail(c, XG_ERR_ARG, "cg_setup: row without diagonal entry");
  }
  if (g_nsm == 0) {
    int dev = 0, nsm = 0;
    XG_CUDA(c, cudaGetDevice(&dev));
    XG_CUDA(c, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    g_nsm = nsm > 0 ? nsm : 1;
  }
  const int64_t nslice = (nrow + kSlice - 1) / kSlice;
  std::vector<int32_t> soff(nslice + 1), sw(nslice);
  int64_t tot = 0;
  for (int64_t s = 0; s < nslice; ++s) {
    uint64_t w = 0;
    for (int64_t i = s * kSlice; i < std::min(nrow, (s + 1) * kSlice); ++i)
      w = std::max<uint64_t>(w, ia[i + 1] - ia[i]);
    sw[s] = static_cast<int32_t>(w);
    soff[s] = static_cast<int32_t>(tot);
    tot += int64_t(w) * kSlice;
    if (tot >= (int64_t(1) << 31)) return fail(c, XG_ERR_ARG, "cg_setup: matrix too large");
  }
  soff[nslice] = static_cast<int32_t>(tot);
  std::vector<int32_t> col(tot, kPad), dpos(nrow);
  std::vector<int16_t> col16(fits16 ? tot : 0, kPad16);
  std::vector<double> val(tot, 0.0);
  for (int64_t i = 0; i < nrow; ++i) {
    const int64_t s = i / kSlice, lane = i % kSlice;
    for (uint64_t j = ia[i]; j < ia[i + 1]; ++j) {
      const int64_t k = int64_t(j - ia[i]);
      const int64_t e = soff[s] + k * kSlice + lane;
      col[e] = static_cast<int32_t>(ja[j - b0] - b0);
      if (fits16) col16[e] = static_cast<int16_t>(col[e] - i);
      val[e] = a[j - b0];
    }
    dpos[i] = static_cast<int32_t>(soff[s] + int64_t(diagk[i]) * kSlice + lane);
  }
  // lower / upper triangles (off-diagonal) as SELL-32, rows sorted by column;
  // posL: the full-layout index of each lower entry; tposU: the upper-layout
  // index of its transposed entry (j,i)
  std::vector<int32_t> soffL(nslice + 1), swL(nslice), soffU(nslice + 1), swU(nslice);
  int64_t totL = 0, totU = 0;
  for (int64_t s2 = 0; s2 < nslice; ++s2) {
    int64_t wl = 0, wu = 0;
    for (int64_t i = s2 * kSlice; i < std::min(nrow, (s2 + 1) * kSlice); ++i) {
      int64_t nl = 0, nu = 0;
      for (uint64_t j = ia[i]; j < ia[i + 1]; ++j) {
        const int64_t cc = int64_t(ja[j - b0] - b0);
        if (cc < i) ++nl;
        if (cc > i) ++nu;
      }
      wl = std::max(wl, nl);
      wu = std::max(wu, nu);
    }
    swL[s2] = int32_t(wl);
    swU[s2] = int32_t(wu);
    soffL[s2] = int32_t(totL);
    soffU[s2] = int32_t(totU);
    totL += wl * kSlice;
    totU += wu * kSlice;
  }
  soffL[nslice] = int32_t(totL);
  soffU[nslice] = int32_t(totU);
  std::vector<int32_t> colL(std::max<int64_t>(1, totL), kPad), posL(std::max<int64_t>(1, totL), 0),
      colU(std::max<int64_t>(1, totU), kPad), tposU(std::max<int64_t>(1, totL), 0);
  std::vector<int16_t> colL16(fits16 ? colL.size() : 0, kPad16),
      colU16(fits16 ? colU.size() : 0, kPad16);
  for (int64_t i = 0; i < nrow; ++i) {
    const int64_t s2 = i / kSlice, lane = i % kSlice;
    int64_t kl = 0, ku = 0;
    for (uint64_t j = ia[i]; j < ia[i + 1]; ++j) {
      const int64_t cc = int64_t(ja[j - b0] - b0);
      const int64_t kfull = int64_t(j - ia[i]);
      if (cc < i) {
        const int64_t e = soffL[s2] + kl * kSlice + lane;
        colL[e] = int32_t(cc);
        if (fits16) colL16[e] = int16_t(cc - i);
        posL[e] = int32_t(soff[s2] + kfull * kSlice + lane);
        ++kl;
      } else if (cc > i) {
        const int64_t e = soffU[s2] + ku * kSlice + lane;
        colU[e] = int32_t(cc);
        if (fits16) colU16[e] = int16_t(cc - i);
        ++ku;
      }
    }
  }
  for (int64_t i = 0; i < nrow; ++i) {
    const int64_t s2 = i / kSlice, lane = i % kSlice;
    int64_t kl = 0;
    for (uint64_t j = ia[i]; j < ia[i + 1]; ++j) {
      const int64_t cc = int64_t(ja[j - b0] - b0);
      if (cc >= i) continue;
      // position of column i in row cc's upper list (rows sorted by column)
      const int64_t s3 = cc / kSlice, lane3 = cc % kSlice;
      int64_t ku = 0;
      bool found = false;
      for (uint64_t jj = ia[cc]; jj < ia[cc + 1]; ++jj) {
        const int64_t c3 = int64_t(ja[jj - b0] - b0);
        if (c3 <= cc) continue;
        if (c3 == i) {
          found = true;
          break;
        }
        ++ku;
      }
      if (!found) return fail(c, XG_ERR_ARG, "cg_setup: matrix graph is not symmetric");
      tposU[soffL[s2] + kl * kSlice + lane] = int32_t(soffU[s3] + ku * kSlice + lane3);
      ++kl;
    }
  }
  if (c->cg) {
    XG_CUDA(c, cudaStreamSynchronize(c->stream));
    destroy_cg(c->cg);
    c->cg = nullptr;
  }
  auto* d = new CGDev;
  c->cg = d;
  d->n = nrow;
  d->nslice = nslice;
  d->nent = tot;
  d->use16 = fits16;
  d->maxgrid = int64_t(g_nsm) * (2048 / kBlock);
  for (int pass = 0; pass < 2; ++pass) {
    Arena& A = d->arena;
    A.plan(d->soff, nslice + 1);
    A.plan(d->swidth, nslice);
    A.plan(d->col, tot);
    A.plan(d->col16, fits16 ? tot : 1);
    A.plan(d->a0, tot);
    A.plan(d->a, tot);
    A.plan(d->a32, tot);
    A.plan(d->rs32, nrow);
    A.plan(d->diagpos, nrow);
    A.plan(d->bcmask, nrow);
    A.plan(d->bcval, nrow);
    A.plan(d->x, nrow);
    A.plan(d->b, nrow);
    A.plan(d->r, nrow);
    A.plan(d->q, nrow);
    A.plan(d->z, nrow);
    A.plan(d->d, nrow);
    A.plan(d->p[0], nrow);
    A.plan(d->p[1], nrow);
    A.plan(d->r32, nrow);
    A.plan(d->r32b, nrow);
    A.plan(d->q32, nrow);
    A.plan(d->z32, nrow);
    A.plan(d->d32, nrow);
    A.plan(d->e64, nrow);
    A.plan(d->p32[0], nrow);
    A.plan(d->p32[1], nrow);
    A.plan(d->partial, 3 * d->maxgrid);
    A.plan(d->scal, 1);
    A.plan(d->soffL, nslice + 1);
    A.plan(d->swL, nslice);
    A.plan(d->colL, colL.size());
    A.plan(d->colL16, fits16 ? colL.size() : 1);
    A.plan(d->posL, posL.size());
    A.plan(d->tposU, tposU.size());
    A.plan(d->soffU, nslice + 1);
    A.plan(d->swU, nslice);
    A.plan(d->colU, colU.size());
    A.plan(d->colU16, fits16 ? colU.size() : 1);
    A.plan(d->nvL, colL.size());
    A.plan(d->nvU, colU.size());
    A.plan(d->hvL, colL.size());
    A.plan(d->hvU, colU.size());
    A.plan(d->eL, colL.size());
    A.plan(d->eU, colU.size());
    A.plan(d->eF, tot);
    A.plan(d->srow, nrow);
    A.plan(d->v, nrow);
    A.plan(d->u, nrow);
    A.plan(d->t, nrow);
    A.plan(d->v32, nrow);
    A.plan(d->u32, nrow);
    if (pass == 0) {
      cudaError_t e = A.reserve();
      if (e != cudaSuccess) {
        destroy_cg(d);
        c->cg = nullptr;
        return fail(c, XG_ERR_CUDA, std::string("cg_setup: ") + cudaGetErrorString(e));
      }
    }
  }
  cudaStream_t s = c->stream;
  XG_CUDA(c, cudaMemcpyAsync(d->soff, soff.data(), soff.size() * 4, cudaMemcpyHostToDevice, s));
  XG_CUDA(c, cudaMemcpyAsync(d->swidth, sw.data(), sw.size() * 4, cudaMemcpyHostToDevice, s));
  XG_CUDA(c, cudaMemcpyAsync(d->col, col.data(), col.size() * 4, cudaMemcpyHostToDevice, s));
  if (fits16)
    XG_CUDA(c, cudaMemcpyAsync(d->col16, col16.data(), col16.size() * 2, cudaMemcpyHostToDevice, s));
  XG_CUDA(c, cudaMemcpyAsync(d->a0, val.data(), val.size() * 8, cudaMemcpyHostToDevice, s));
  XG_CUDA(c, cudaMemcpyAsync(d->diagpos, dpos.data(), dpos.size() * 4, cudaMemcpyHostToDevice, s));
  d->nentL = totL;
  d->nentU = totU;
  XG_CUDA(c, cudaMemcpyAsync(d->soffL, soffL.data(), soffL.size() * 4, cudaMemcpyHostToDevice, s));
  XG_CUDA(c, cudaMemcpyAsync(d->swL, swL.data(), swL.size() * 4, cudaMemcpyHostToDevice, s));
  XG_CUDA(c, cudaMemcpyAsync(d->colL, colL.data(), colL.size() * 4, cudaMemcpyHostToDevice, s));
  XG_CUDA(c, cudaMemcpyAsync(d->posL, posL.data(), posL.size() * 4, cudaMemcpyHostToDevice, s));
  XG_CUDA(c, cudaMemcpyAsync(d->tposU, tposU.data(), tposU.size() * 4, cudaMemcpyHostToDevice, s));
  XG_CUDA(c, cudaMemcpyAsync(d->soffU, soffU.data(), soffU.size() * 4, cudaMemcpyHostToDevice, s));
  XG_CUDA(c, cudaMemcpyAsync(d->swU, swU.data(), swU.size() * 4, cudaMemcpyHostToDevice, s));
  XG_CUDA(c, cudaMemcpyAsync(d->colU, colU.data(), colU.size() * 4, cudaMemcpyHostToDevice, s));
  if (fits16) {
    XG_CUDA(c, cudaMemcpyAsync(d->colL16, colL16.data(), colL16.size() * 2, cudaMemcpyHostToDevice,
                               s));
    XG_CUDA(c, cudaMemcpyAsync(d->colU16, colU16.data(), colU16.size() * 2, cudaMemcpyHostToDevice,
                               s));
  }
  XG_CUDA(c, cudaMemsetAsync(d->nvL, 0, colL.size() * 4, s));
  XG_CUDA(c, cudaMemsetAsync(d->nvU, 0, colU.size() * 4, s));
  XG_CUDA(c, cudaMemsetAsync(d->hvL, 0, colL.size() * 2, s));
  XG_CUDA(c, cudaMemsetAsync(d->hvU, 0, colU.size() * 2, s));
  XG_CUDA(c, cudaMemsetAsync(d->eU, 0, colU.size() * 4, s));
  XG_CUDA(c, cudaMemsetAsync(d->x, 0, nrow * 8, s));
  XG_CUDA(c, cudaMemsetAsync(d->b, 0, nrow * 8, s));
  XG_CUDA(c, cudaMemsetAsync(d->bcmask, 0, nrow, s));
  XG_CUDA(c, cudaMemsetAsync(d->scal, 0, sizeof(CGScalars), s));
  k_copy_values<<<blocks_for(tot, kBlock), kBlock, 0, s>>>(tot, d->a0, d->a, d->a32);
  XG_CHECK_LAUNCH(c);
  k_row_sums<<<blocks_for(nrow, kBlock), kBlock, 0, s>>>(nrow, d->soff, d->swidth, d->col, d->a,
                                                         d->rs32);
  XG_CHECK_LAUNCH(c);
  XG_CUDA(c, cudaStreamSynchronize(s));
  return XG_OK;
  XG_HOST_CATCH(c)
}

int xg_cg_mult(xg_ctx* c, const double* x, double* y) {
  int rc = use(c);
  if (rc) return rc;
  CGDev* d = c->cg;
  if (!d) return fail(c, XG_ERR_STATE, "cg_mult before cg_setup");
  if (!x || !y) return fail(c, XG_ERR_ARG, "cg_mult: null vector");
  XG_CUDA(c, cudaMemcpyAsync(d->r, x, d->n * 8, cudaMemcpyHostToDevice, c->stream));
  k_spmv<<<pgrid<k_spmv>(d->n), kBlock, 0, c->stream>>>(d->n, d->soff, d->swidth, d->col, d->a0,
                                                        d->r, d->q);
  XG_CHECK_LAUNCH(c);
  XG_CUDA(c, cudaMemcpyAsync(y, d->q, d->n * 8, cudaMemcpyDeviceToHost, c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}

int xg_cg_init(xg_ctx* c, const double* x, const double* b, const double* neubc, int64_t ndir,
               const uint64_t* dirnodes, const double* dirvals, int apply, int pc) {
  XG_HOST_TRY
  int rc = use(c);
  if (rc) return rc;
  CGDev* d = c->cg;
  if (!d) return fail(c, XG_ERR_STATE, "cg_init before cg_setup");
  if (pc != 0 && pc != 1 && pc != 2) return fail(c, XG_ERR_ARG, "cg_init: unknown preconditioner");
  if (ndir && (!dirnodes || !dirvals)) return fail(c, XG_ERR_ARG, "cg_init: null Dirichlet data");
  cudaStream_t s = c->stream;
  const int64_t n = d->n;
  if (x) XG_CUDA(c, cudaMemcpyAsync(d->x, x, n * 8, cudaMemcpyHostToDevice, s));
  if (b) XG_CUDA(c, cudaMemcpyAsync(d->b, b, n * 8, cudaMemcpyHostToDevice, s));
  d->pc = pc;
  d->apply = apply != 0;
  // the working matrix depends on the Dirichlet node set only: its scales,
  // couplings and factor survive re-initialisations with the same set (a
  // pressure solve per time step)
  uint64_t key = 1469598103934665603ull;  // FNV-1a over the mask, 0 without BCs
  if (d->apply) {
    std::vector<uint8_t> mask(n, 0);
    std::vector<double> val(n, 0.0);
    for (int64_t k = 0; k < ndir; ++k) {
      if (dirnodes[k] >= static_cast<uint64_t>(n))
        return fail(c, XG_ERR_ARG, "cg_init: Dirichlet node out of range");
      mask[dirnodes[k]] = 1;
      val[dirnodes[k]] = dirvals[k];
    }
    for (int64_t i = 0; i < n; ++i) key = (key ^ mask[i]) * 1099511628211ull;
    XG_CUDA(c, cudaMemcpyAsync(d->bcmask, mask.data(), n, cudaMemcpyHostToDevice, s));
    XG_CUDA(c, cudaMemcpyAsync(d->bcval, val.data(), n * 8, cudaMemcpyHostToDevice, s));
    double* neu = nullptr;
    if (neubc) {
      XG_CUDA(c, cudaMemcpyAsync(d->q, neubc, n * 8, cudaMemcpyHostToDevice, s));
      neu = d->q;
    }
    k_apply_bc<<<blocks_for(n, kBlock), kBlock, 0, s>>>(n, d->soff, d->swidth, d->col, d->a0,
                                                         d->a, d->a32, d->bcmask, d->bcval, neu,
                                                         d->b);
    XG_CHECK_LAUNCH(c);
    // mask and val are host vectors of this frame: complete their copies
    XG_CUDA(c, cudaStreamSynchronize(s));
  } else {
    key = 0;
    XG_CUDA(c, cudaMemsetAsync(d->bcmask, 0, n, s));
    k_copy_values<<<blocks_for(d->nent, kBlock), kBlock, 0, s>>>(d->nent, d->a0, d->a, d->a32);
    XG_CHECK_LAUNCH(c);
  }
  k_row_sums<<<blocks_for(n, kBlock), kBlock, 0, s>>>(n, d->soff, d->swidth, d->col, d->a,
                                                      d->rs32);
  XG_CHECK_LAUNCH(c);
  if (key != d->bc_key || !d->ready) {
    d->geom_set = false;
    d->factor_set = false;
  }
  d->bc_key = key;
  CGScalars h{};
  h.pc = pc;
  h.guard = d->guard;
  XG_CUDA(c, cudaMemcpyAsync(d->scal, &h, sizeof(h), cudaMemcpyHostToDevice, s));
  k_setup<<<pgrid<k_setup>(n), kBlock, 0, s>>>(n, d->soff, d->swidth, d->col, d->a, d->diagpos,
                                               d->x, d->b, d->r, d->d, d->z, d->p[0], d->d32,
                                               d->partial, d->scal);
  XG_CHECK_LAUNCH(c);
  if (pc == 2) {
    int rf = d->factor_set ? XG_OK : build_factor(c, d);
    if (rf) return rf;
    rf = factor_apply64(c, d, d->r, d->z);
    if (rf) return rf;
  }
  XG_CUDA(c, cudaStreamSynchronize(s));
  d->ready = true;
  return XG_OK;
  XG_HOST_CATCH(c)
}

int xg_cg_solve(xg_ctx* c, int64_t maxit, double tol, int64_t* it, double* normr,
                double* normb, int* converged) {
  int rc = use(c);
  if (rc) return rc;
  CGDev* d = c->cg;
  if (!d || !d->ready) return fail(c, XG_ERR_STATE, "cg_solve before cg_init");
  if (maxit <= 0 || !(tol >= 0)) return fail(c, XG_ERR_ARG, "cg_solve: bad maxit/tol");
  CGScalars h{};
  rc = cg_iterate(c, d, maxit, tol, &h);
  if (rc) return rc;
  d->last_it = h.it;
  d->last_normr = std::sqrt(h.rr);
  d->last_normb = h.normb;
  d->last_conv = h.converged;
  if (it) *it = h.it;
  if (normr) *normr = std::sqrt(h.rr);
  if (normb) *normb = h.normb;
  if (converged) *converged = h.converged;
  return XG_OK;
}

int xg_cg_solve_mixed(xg_ctx* c, int64_t maxit, double tol, double inner_tol,
                      int64_t inner_maxit, int64_t* outer, int64_t* inner, double* normr,
                      double* normb, int* converged) {
  int rc = use(c);
  if (rc) return rc;
  CGDev* d = c->cg;
  if (!d || !d->ready) return fail(c, XG_ERR_STATE, "cg_solve_mixed before cg_init");
  if (maxit <= 0 || inner_maxit <= 0 || !(tol >= 0) || !(inner_tol > 0) || !(inner_tol < 1))
    return fail(c, XG_ERR_ARG, "cg_solve_mixed: bad limits");
  cudaStream_t s = c->stream;
  CGScalars h{};
  rc = read_scal(c, d, &h);
  if (rc) return rc;
  const double nb0 = h.normb > 1.0e-14 ? h.normb : 1.0;
  XG_CUDA(c, cudaMemsetAsync(d->e64, 0, d->n * 8, s));
  // the first FP32 iteration reads p with weight beta = 0: make it finite
  XG_CUDA(c, cudaMemsetAsync(d->p32[0], 0, d->n * 4, s));
  XG_CUDA(c, cudaMemsetAsync(d->p32[1], 0, d->n * 4, s));
  rc = replace_residual(c, d, 1);
  if (rc) return rc;
  rc = read_scal(c, d, &h);
  if (rc) return rc;
  double nr = std::sqrt(h.rr);
  int64_t nout = 0;
  bool conv = nr < tol * nb0;
  int breakdown = 0;
  while (!conv && nout < maxit && h.it < inner_maxit && !breakdown) {
    h.tol = tol;
    h.delta = inner_tol;
    h.rlast = nr;
    h.maxit = inner_maxit;
    h.done = 0;
    rc = write_scal(c, d, &h);
    if (rc) return rc;
    for (;;) {
      rc = d->use16 ? mixed_batch<Cols16>(c, d, Cols16{d->col16}, Cols16{d->colU16},
                                          Cols16{d->colL16})
                    : mixed_batch<Cols32>(c, d, Cols32{d->col}, Cols32{d->colU}, Cols32{d->colL});
      if (rc) return rc;
      rc = read_scal(c, d, &h);
      if (rc) return rc;
      if (h.done) break;
    }
    breakdown = h.finished;
    k_add_correction<<<blocks_for(d->n, kBlock), kBlock, 0, s>>>(d->n, d->e64, d->x);
    XG_CHECK_LAUNCH(c);
    rc = replace_residual(c, d, 0);
    if (rc) return rc;
    rc = read_scal(c, d, &h);
    if (rc) return rc;
    nr = std::sqrt(h.rr);
    ++nout;
    conv = nr < tol * nb0;
  }
  d->last_it = h.it;
  d->last_normr = nr;
  d->last_normb = nb0;
  d->last_conv = conv;
  if (outer) *outer = nout;
  if (inner) *inner = h.it;
  if (normr) *normr = nr;
  if (normb) *normb = nb0;
  if (converged) *converged = conv ? 1 : 0;
  return XG_OK;
}

int xg_cg_set_factor(xg_ctx* c, xg_lpc* model, double scale) {
  int rc = use(c);
  if (rc) return rc;
  CGDev* d = c->cg;
  if (!d) return fail(c, XG_ERR_STATE, "cg_set_factor before cg_setup");
  d->factor_model = model;
  d->factor_c = scale;
  d->factor_set = false;
  return XG_OK;
}

int xg_cg_set_guard(xg_ctx* c, int guard) {
  int rc = use(c);
  if (rc) return rc;
  CGDev* d = c->cg;
  if (!d) return fail(c, XG_ERR_STATE, "cg_set_guard before cg_setup");
  if (guard != 0 && guard != 1) return fail(c, XG_ERR_ARG, "cg_set_guard: guard is 0 or 1");
  d->guard = guard;
  return XG_OK;
}

int xg_cg_precondition(xg_ctx* c, const double* r, double* z) {
  int rc = use(c);
  if (rc) return rc;
  CGDev* d = c->cg;
  if (!d || !d->ready) return fail(c, XG_ERR_STATE, "cg_precondition before cg_init");
  if (!r || !z) return fail(c, XG_ERR_ARG, "cg_precondition: null vector");
  cudaStream_t s = c->stream;
  XG_CUDA(c, cudaMemcpyAsync(d->q, r, d->n * 8, cudaMemcpyHostToDevice, s));
  // the passes run only while the solve is not done: save the scalars, clear
  // done, restore them afterwards
  CGScalars h{};
  rc = read_scal(c, d, &h);
  if (rc) return rc;
  CGScalars run = h;
  run.done = 0;
  rc = write_scal(c, d, &run);
  if (rc) return rc;
  if (d->pc == 2) {
    if (!d->factor_set) {
      rc = build_factor(c, d);
      if (rc) return rc;
    }
    rc = factor_apply64(c, d, d->q, d->t);
    if (rc) return rc;
  } else {
    k_jacobi_apply<<<blocks_for(d->n, kBlock), kBlock, 0, s>>>(d->n, d->q, d->d, d->t);
    XG_CHECK_LAUNCH(c);
  }
  rc = write_scal(c, d, &h);
  if (rc) return rc;
  XG_CUDA(c, cudaMemcpyAsync(z, d->t, d->n * 8, cudaMemcpyDeviceToHost, s));
  XG_CUDA(c, cudaStreamSynchronize(s));
  return XG_OK;
}

int xg_cg_solution(xg_ctx* c, double* x) {
  int rc = use(c);
  if (rc) return rc;
  CGDev* d = c->cg;
  if (!d) return fail(c, XG_ERR_STATE, "cg_solution before cg_setup");
  if (!x) return fail(c, XG_ERR_ARG, "cg_solution: null x");
  XG_CUDA(c, cudaMemcpyAsync(x, d->x, d->n * 8, cudaMemcpyDeviceToHost, c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}

}  // extern "C"
