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
// int32 columns and FP64 values, plus an FP32 copy for the mixed-precision
// inner solver.  Dirichlet elimination never rewrites the host matrix: a
// device pass builds the working values from the original ones and the
// Dirichlet mask, which is what the reference's sequential elimination
// produces (rows and columns of Dirichlet nodes zeroed, 1 on their
// diagonal), and the right-hand side correction sum_i a_ji * val_i is summed
// per row in the reference's order (decreasing node id).
//
// One PCG iteration is two kernels:
//   k_iter_a: p' = z + beta p (beta = rho/rho0), q = A p', partial (p', q)
//   k_iter_b: alpha = rho/(p,q); r -= alpha q; z = M^-1 r; x += alpha p';
//             partial (r,z), (r,r); convergence test
// Block partial sums go to a scratch array; the last block to finish (an
// atomic ticket, no spinning) adds them in block order, so every reduction is
// deterministic.  Kernels return at once when the solve is done, so the host
// launches iterations in batches and reads the done flag once per batch.

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
constexpr int kBlock = 256;
constexpr int kBatch = 16;

struct CGScalars {
  double rho, rho0, pq, alpha, rr, normb, tol;
  double pad0;
  int64_t it, maxit;
  int32_t done, finished, converged, pc;
  unsigned int ticket[4];
};
}  // namespace

struct CGDev {
  Arena arena;
  int64_t n = 0, nslice = 0, nent = 0, nblk = 0;
  int32_t *soff = nullptr, *swidth = nullptr, *col = nullptr;
  double *a0 = nullptr, *a = nullptr;  // original and working values
  float* a32 = nullptr;
  int32_t* diagpos = nullptr;          // SELL index of each row's diagonal
  uint8_t* bcmask = nullptr;
  double* bcval = nullptr;
  double *x = nullptr, *b = nullptr, *r = nullptr, *q = nullptr, *z = nullptr, *d = nullptr;
  double* p[2] = {nullptr, nullptr};
  float *r32 = nullptr, *q32 = nullptr, *z32 = nullptr, *d32 = nullptr, *e32 = nullptr;
  float* p32[2] = {nullptr, nullptr};
  double* partial = nullptr;  // 3 * nblk
  CGScalars* scal = nullptr;
  int cur = 0;
  bool apply = false;
  bool have_bc = false;
  bool ready = false;
  int pc = 1;
  int64_t last_it = 0;
  double last_normr = 0, last_normb = 0;
  int last_conv = 0;
  int64_t inner_its = 0;
  // factored approximate inverse M^-1 = -S (I+N)(I+N)^T S (pc 2): lower and
  // upper triangles of the matrix graph as SELL-32, the factor values, the
  // row scales s = 1/sqrt|a_ii| and the normalised couplings e_ij = a_ij s_i s_j
  int64_t nentL = 0, nentU = 0;
  int32_t *soffL = nullptr, *swL = nullptr, *colL = nullptr, *posL = nullptr, *tposU = nullptr;
  int32_t *soffU = nullptr, *swU = nullptr, *colU = nullptr;
  float *nvL = nullptr, *nvU = nullptr, *srow = nullptr, *eL = nullptr, *eU = nullptr;
  float* eF = nullptr;  // e_ij in the full layout (0 on the diagonal and at Dirichlet nodes)
  bool geom_set = false;
  double *u = nullptr, *t = nullptr;  // t: output of xg_cg_precondition
  float* u32 = nullptr;
  bool factor_set = false;
  xg_lpc* factor_model = nullptr;  // network emitting N, or null: N = factor_c * e
  double factor_c = 1.0;
};

void destroy_cg(CGDev* d) { delete d; }
size_t bytes_cg(const CGDev* d) { return d ? d->arena.bytes() : 0; }

namespace {

// ---------------------------------------------------------------- reductions

// Sum of one value per thread into partial[blockIdx.x]; returns true in the
// block that completes last (its threads then see every partial).
template <int K>
__device__ __forceinline__ bool block_partials(const double (&v)[K], double* partial,
                                               int64_t nblk, unsigned int* ticket) {
  __shared__ double sm[K][32];
  __shared__ bool last;
  double s[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    s[k] = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s[k] += __shfl_xor_sync(0xffffffffu, s[k], o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) sm[k][wid] = s[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    for (int k = 0; k < K; ++k) {
      double t = 0.0;
      for (int w = 0; w < nw; ++w) t += sm[k][w];
      partial[k * nblk + blockIdx.x] = t;
    }
    __threadfence();
    unsigned int prev = atomicAdd(ticket, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  return last;
}

// In the last block: deterministic sum of the partials of component k, by
// lane-strided chunks then a fixed-order tree.
__device__ double sum_partials(const double* partial, int64_t nblk, int k) {
  __shared__ double red[kBlock];
  __threadfence();
  double t = 0.0;
  for (int64_t i = threadIdx.x; i < nblk; i += blockDim.x) t += __ldcg(partial + k * nblk + i);
  red[threadIdx.x] = t;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  double r = red[0];
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------- kernels

// CSR::mult on the original (or working) values: y = A x.
__global__ void k_spmv(int64_t n, const int32_t* __restrict__ soff, const int32_t* __restrict__ sw,
                       const int32_t* __restrict__ col, const double* __restrict__ a,
                       const double* __restrict__ x, double* __restrict__ y) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int lane = int(i & 31);
  const int32_t off = soff[i >> 5], w = sw[i >> 5];
  double s = 0.0;
  for (int k = 0; k < w; ++k) {
    const int32_t e = off + k * kSlice + lane;
    const int32_t c = __ldg(col + e);
    if (c < 0) continue;
    s += __ldg(a + e) * __ldg(x + c);
  }
  y[i] = s;
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

__global__ void k_copy_values(int64_t nent, const double* __restrict__ a0, double* __restrict__ a,
                              float* __restrict__ a32) {
  int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (e >= nent) return;
  a[e] = a0[e];
  a32[e] = float(a0[e]);
}

// ConjugateGradients::setup + pc + initres (ConjugateGradients.cpp:105-319):
// r = b - A x, d = diag(A) (Jacobi) or 1 (none), z = r/d, p = r,
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
                                                   int64_t nblk, CGScalars* sc) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  double v[2] = {0.0, 0.0};
  if (i < n) {
    const int lane = int(i & 31);
    const int32_t off = soff[i >> 5], w = sw[i >> 5];
    double s = 0.0;
    for (int k = 0; k < w; ++k) {
      const int32_t e = off + k * kSlice + lane;
      const int32_t c = col[e];
      if (c < 0) continue;
      s += a[e] * x[c];
    }
    const double ri = b[i] - s;
    const double di = sc->pc == 1 ? a[diagpos[i]] : 1.0;
    r[i] = ri;
    d[i] = di;
    d32[i] = float(di);
    const double zi = ri / di;
    z[i] = zi;
    p[i] = ri;
    v[0] = b[i] * b[i];
    v[1] = ri * zi;
  }
  if (block_partials<2>(v, partial, nblk, &sc->ticket[0])) {
    double bb = sum_partials(partial, nblk, 0);
    double rz = sum_partials(partial, nblk, 1);
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

// next + qAp + q (ConjugateGradients.cpp:584-669), fused.
__global__ void __launch_bounds__(kBlock) k_iter_a(int64_t n, const int32_t* __restrict__ soff,
                                                    const int32_t* __restrict__ sw,
                                                    const int32_t* __restrict__ col,
                                                    const double* __restrict__ a,
                                                    const double* __restrict__ z,
                                                    const double* __restrict__ pold,
                                                    double* __restrict__ pnew,
                                                    double* __restrict__ q, double* partial,
                                                    int64_t nblk, CGScalars* sc) {
  if (sc->done) return;
  const double beta = sc->it == 0 ? 0.0 : sc->rho / sc->rho0;
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  double v[1] = {0.0};
  if (i < n) {
    const int lane = int(i & 31);
    const int32_t off = soff[i >> 5], w = sw[i >> 5];
    double s = 0.0;
    for (int k = 0; k < w; ++k) {
      const int32_t e = off + k * kSlice + lane;
      const int32_t c = __ldg(col + e);
      if (c < 0) continue;
      s += __ldg(a + e) * (__ldg(z + c) + beta * __ldg(pold + c));
    }
    const double pi = z[i] + beta * pold[i];
    pnew[i] = pi;
    q[i] = s;
    v[0] = pi * s;
  }
  if (block_partials<1>(v, partial, nblk, &sc->ticket[1])) {
    double pq = sum_partials(partial, nblk, 0);
    if (threadIdx.x == 0) {
      sc->rho0 = sc->rho;
      sc->pq = pq;
      if (fabs(pq) < DBL_EPSILON) {
        sc->finished = 1;
        sc->alpha = 0.0;
      } else {
        sc->alpha = sc->rho / pq;
      }
      sc->ticket[1] = 0;
    }
  }
}

// pq + rz + x (ConjugateGradients.cpp:671-823), fused.
template <bool FACTOR>
__global__ void __launch_bounds__(kBlock) k_iter_b(int64_t n, const double* __restrict__ q,
                                                    const double* __restrict__ d,
                                                    const double* __restrict__ p,
                                                    double* __restrict__ r, double* __restrict__ z,
                                                    double* __restrict__ x, double* partial,
                                                    int64_t nblk, CGScalars* sc) {
  if (sc->done) return;
  const double alpha = sc->alpha;
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  double v[2] = {0.0, 0.0};
  if (i < n) {
    const double ri = r[i] - alpha * q[i];
    r[i] = ri;
    x[i] += alpha * p[i];
    if (!FACTOR) {  // Jacobi / none; the factored inverse follows in two passes
      const double zi = ri / d[i];
      z[i] = zi;
      v[0] = ri * zi;
    }
    v[1] = ri * ri;
  }
  if (block_partials<2>(v, partial, nblk, &sc->ticket[2])) {
    double rz = sum_partials(partial, nblk, 0);
    double rr = sum_partials(partial, nblk, 1);
    if (threadIdx.x == 0) {
      if (!FACTOR) sc->rho = rz;
      sc->rr = rr;
      sc->it += 1;
      const double nb = sc->normb > 1.0e-14 ? sc->normb : 1.0;
      const double nr = sqrt(rr);
      if (sc->finished || nr < sc->tol * nb || sc->it >= sc->maxit) {
        sc->done = 1;
        sc->converged = nr > sc->tol * nb ? 0 : 1;
      }
      sc->ticket[2] = 0;
    }
  }
}

// ---- mixed precision: FP32 inner PCG on A e = r (x untouched), FP64 dots.

// r = b - A x in FP64, r32 = r, e32 = 0, z32 = r/d, p32 = z32; partials
// (r,r) and (r32,z32).
__global__ void __launch_bounds__(kBlock) k_outer_res(int64_t n, const int32_t* __restrict__ soff,
                                                       const int32_t* __restrict__ sw,
                                                       const int32_t* __restrict__ col,
                                                       const double* __restrict__ a,
                                                       const double* __restrict__ x,
                                                       const double* __restrict__ b,
                                                       const float* __restrict__ d32,
                                                       float* __restrict__ r32,
                                                       float* __restrict__ z32,
                                                       float* __restrict__ p32,
                                                       float* __restrict__ e32, double* partial,
                                                       int64_t nblk, CGScalars* sc) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  double v[2] = {0.0, 0.0};
  if (i < n) {
    const int lane = int(i & 31);
    const int32_t off = soff[i >> 5], w = sw[i >> 5];
    double s = 0.0;
    for (int k = 0; k < w; ++k) {
      const int32_t e = off + k * kSlice + lane;
      const int32_t c = col[e];
      if (c < 0) continue;
      s += a[e] * x[c];
    }
    const double ri = b[i] - s;
    const float rf = float(ri);
    const float zf = rf / d32[i];
    r32[i] = rf;
    z32[i] = zf;
    p32[i] = zf;
    e32[i] = 0.f;
    v[0] = ri * ri;
    v[1] = double(rf) * double(zf);
  }
  if (block_partials<2>(v, partial, nblk, &sc->ticket[0])) {
    double rr = sum_partials(partial, nblk, 0);
    double rz = sum_partials(partial, nblk, 1);
    if (threadIdx.x == 0) {
      sc->rr = rr;
      sc->rho = rz;
      sc->it = 0;
      sc->done = 0;
      sc->finished = 0;
      sc->ticket[0] = 0;
    }
  }
}

__global__ void __launch_bounds__(kBlock) k_in_a(int64_t n, const int32_t* __restrict__ soff,
                                                  const int32_t* __restrict__ sw,
                                                  const int32_t* __restrict__ col,
                                                  const float* __restrict__ a,
                                                  const float* __restrict__ z,
                                                  const float* __restrict__ pold,
                                                  float* __restrict__ pnew, float* __restrict__ q,
                                                  double* partial, int64_t nblk, CGScalars* sc) {
  if (sc->done) return;
  const float beta = sc->it == 0 ? 0.f : float(sc->rho / sc->rho0);
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  double v[1] = {0.0};
  if (i < n) {
    const int lane = int(i & 31);
    const int32_t off = soff[i >> 5], w = sw[i >> 5];
    float s = 0.f;
    for (int k = 0; k < w; ++k) {
      const int32_t e = off + k * kSlice + lane;
      const int32_t c = __ldg(col + e);
      if (c < 0) continue;
      s += __ldg(a + e) * (__ldg(z + c) + beta * __ldg(pold + c));
    }
    const float pi = z[i] + beta * pold[i];
    pnew[i] = pi;
    q[i] = s;
    v[0] = double(pi) * double(s);
  }
  if (block_partials<1>(v, partial, nblk, &sc->ticket[1])) {
    double pq = sum_partials(partial, nblk, 0);
    if (threadIdx.x == 0) {
      sc->rho0 = sc->rho;
      sc->pq = pq;
      if (fabs(pq) < DBL_MIN) {
        sc->finished = 1;
        sc->alpha = 0.0;
      } else {
        sc->alpha = sc->rho / pq;
      }
      sc->ticket[1] = 0;
    }
  }
}

// inner stop: ||r_inner|| < tol * ||r_outer|| (tol in sc->tol, ||r_outer||^2
// kept in sc->normb as the reference norm of this inner solve)
template <bool FACTOR>
__global__ void __launch_bounds__(kBlock) k_in_b(int64_t n, const float* __restrict__ q,
                                                  const float* __restrict__ d,
                                                  const float* __restrict__ p,
                                                  float* __restrict__ r, float* __restrict__ z,
                                                  float* __restrict__ e, double* partial,
                                                  int64_t nblk, CGScalars* sc) {
  if (sc->done) return;
  const float alpha = float(sc->alpha);
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  double v[2] = {0.0, 0.0};
  if (i < n) {
    const float ri = r[i] - alpha * q[i];
    r[i] = ri;
    e[i] += alpha * p[i];
    if (!FACTOR) {
      const float zi = ri / d[i];
      z[i] = zi;
      v[0] = double(ri) * double(zi);
    }
    v[1] = double(ri) * double(ri);
  }
  if (block_partials<2>(v, partial, nblk, &sc->ticket[2])) {
    double rz = sum_partials(partial, nblk, 0);
    double rr = sum_partials(partial, nblk, 1);
    if (threadIdx.x == 0) {
      if (!FACTOR) sc->rho = rz;
      sc->it += 1;
      const double nr = sqrt(rr);
      if (sc->finished || nr < sc->tol * sc->normb || sc->it >= sc->maxit) sc->done = 1;
      sc->ticket[2] = 0;
    }
  }
}

__global__ void k_jacobi_apply(int64_t n, const double* __restrict__ r, const double* __restrict__ d,
                               double* __restrict__ z) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i < n) z[i] = r[i] / d[i];
}

__global__ void k_add_correction(int64_t n, const float* __restrict__ e, double* __restrict__ x) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i < n) x[i] += double(e[i]);
}

__global__ void k_set_inner(CGScalars* sc, double tol, int64_t maxit) {
  sc->normb = sqrt(sc->rr);
  sc->tol = tol;
  sc->maxit = maxit;
}

// ---- factored approximate inverse (pc 2)

struct Tri {
  const int32_t* soff;
  const int32_t* sw;
  const int32_t* col;
};

// Row scales and normalised lower couplings of the working matrix:
// s_i = 1/sqrt|a_ii|, e_ij = a_ij s_i s_j (0 when i or j is a Dirichlet node).
__global__ void k_factor_geom(int64_t n, const double* __restrict__ a,
                              const int32_t* __restrict__ diagpos, const uint8_t* __restrict__ mask,
                              float* __restrict__ srow) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  srow[i] = float(1.0 / sqrt(fabs(a[diagpos[i]])));
}
__global__ void k_factor_e(int64_t n, Tri L, const int32_t* __restrict__ posL,
                           const int32_t* __restrict__ tposU, const double* __restrict__ a,
                           const float* __restrict__ srow, const uint8_t* __restrict__ mask,
                           float* __restrict__ eL, float* __restrict__ eU) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int lane = int(i & 31);
  const int32_t off = L.soff[i >> 5], w = L.sw[i >> 5];
  for (int k = 0; k < w; ++k) {
    const int32_t e = off + k * kSlice + lane;
    const int32_t j = L.col[e];
    if (j < 0) continue;
    const float v = (mask[i] || mask[j]) ? 0.f : float(a[posL[e]]) * srow[i] * srow[j];
    eL[e] = v;
    eU[tposU[e]] = v;
  }
}
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
// N_ij = c e_ij (the first-order factor, c = 1, or any uniform scaling).
__global__ void k_factor_scaled(int64_t n, Tri L, const int32_t* __restrict__ tposU,
                                const float* __restrict__ eL, const float* __restrict__ srow,
                                float c, float* __restrict__ nvL, float* __restrict__ nvU) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int lane = int(i & 31);
  const int32_t off = L.soff[i >> 5], w = L.sw[i >> 5];
  for (int k = 0; k < w; ++k) {
    const int32_t e = off + k * kSlice + lane;
    const int32_t j = L.col[e];
    if (j < 0) continue;
    const float v = c * eL[e];
    nvL[e] = v;
    nvU[tposU[e]] = v * srow[i];  // the upper copy (row j, column i) carries s_i
  }
}

// u = (I+N)^T S r: u_i = s_i r_i + sum_{j>i} N_ji s_j r_j.
template <class T>
__global__ void __launch_bounds__(kBlock) k_pc_upper(int64_t n, Tri U, const float* __restrict__ nvU,
                                                      const float* __restrict__ srow,
                                                      const T* __restrict__ r, T* __restrict__ u,
                                                      const CGScalars* __restrict__ sc) {
  if (sc->done) return;
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int lane = int(i & 31);
  const int32_t off = U.soff[i >> 5], w = U.sw[i >> 5];
  T acc = T(srow[i]) * r[i];
  for (int k = 0; k < w; ++k) {
    const int32_t e = off + k * kSlice + lane;
    const int32_t j = __ldg(U.col + e);
    if (j < 0) continue;
    acc += T(__ldg(nvU + e)) * __ldg(r + j);
  }
  u[i] = acc;
}

// z = -S (I+N) u (Dirichlet rows: z = r), partial (r,z); the last block
// stores rho = (r,z).  With SETP the search direction starts as p = z.
template <class T, bool SETP>
__global__ void __launch_bounds__(kBlock) k_pc_lower(int64_t n, Tri L, const float* __restrict__ nvL,
                                                      const float* __restrict__ srow,
                                                      const uint8_t* __restrict__ mask,
                                                      const T* __restrict__ u, const T* __restrict__ r,
                                                      T* __restrict__ z, T* __restrict__ p,
                                                      double* partial, int64_t nblk, CGScalars* sc) {
  if (sc->done) return;
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  double v[1] = {0.0};
  if (i < n) {
    const int lane = int(i & 31);
    const int32_t off = L.soff[i >> 5], w = L.sw[i >> 5];
    T acc = u[i];
    for (int k = 0; k < w; ++k) {
      const int32_t e = off + k * kSlice + lane;
      const int32_t j = __ldg(L.col + e);
      if (j < 0) continue;
      acc += T(__ldg(nvL + e)) * __ldg(u + j);
    }
    const T ri = r[i];
    const T zi = mask[i] ? ri : -T(srow[i]) * acc;
    z[i] = zi;
    if (SETP) p[i] = zi;
    v[0] = double(ri) * double(zi);
  }
  if (block_partials<1>(v, partial, nblk, &sc->ticket[3])) {
    double rz = sum_partials(partial, nblk, 0);
    if (threadIdx.x == 0) {
      sc->rho = rz;
      sc->ticket[3] = 0;
    }
  }
}

Tri tri_l(const CGDev* d) { return Tri{d->soffL, d->swL, d->colL}; }
Tri tri_u(const CGDev* d) { return Tri{d->soffU, d->swU, d->colU}; }

// Row scales and normalised couplings of the current working matrix.
int build_geom(xg_ctx* c, CGDev* d) {
  cudaStream_t s = c->stream;
  const unsigned nb = blocks_for(d->n, kBlock);
  k_factor_geom<<<nb, kBlock, 0, s>>>(d->n, d->a, d->diagpos, d->bcmask, d->srow);
  XG_CHECK_LAUNCH(c);
  k_factor_e<<<nb, kBlock, 0, s>>>(d->n, tri_l(d), d->posL, d->tposU, d->a, d->srow, d->bcmask,
                                   d->eL, d->eU);
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

// Scales, couplings and factor values of the current working matrix.
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
    k_factor_scaled<<<nb, kBlock, 0, s>>>(d->n, tri_l(d), d->tposU, d->eL, d->srow,
                                          float(d->factor_c), d->nvL, d->nvU);
    XG_CHECK_LAUNCH(c);
  }
  d->factor_set = true;
  return XG_OK;
}

int read_scal(xg_ctx* c, CGDev* d, CGScalars* h) {
  XG_CUDA(c, cudaMemcpyAsync(h, d->scal, sizeof(CGScalars), cudaMemcpyDeviceToHost, c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
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

}  // namespace xg

using namespace xg;

extern "C" {

int xg_cg_setup(xg_ctx* c, int64_t nrow, const uint64_t* ia, const uint64_t* ja, const double* a,
                int base) {
  int rc = use(c);
  if (rc) return rc;
  if (nrow <= 0 || !ia || !ja || !a || (base != 0 && base != 1))
    return fail(c, XG_ERR_ARG, "cg_setup: bad matrix");
  if (nrow >= (int64_t(1) << 31) - 64) return fail(c, XG_ERR_ARG, "cg_setup: too many rows");
  const uint64_t b0 = static_cast<uint64_t>(base);
  if (ia[0] != b0) return fail(c, XG_ERR_ARG, "cg_setup: ia[0] must equal the index base");
  std::vector<int32_t> diagk(nrow, -1);
  for (int64_t i = 0; i < nrow; ++i) {
    if (ia[i + 1] < ia[i]) return fail(c, XG_ERR_ARG, "cg_setup: ia not monotonic");
    for (uint64_t j = ia[i]; j < ia[i + 1]; ++j) {
      uint64_t cc = ja[j - b0] - b0;
      if (cc >= static_cast<uint64_t>(nrow)) return fail(c, XG_ERR_ARG, "cg_setup: column id");
      if (static_cast<int64_t>(cc) == i) diagk[i] = static_cast<int32_t>(j - ia[i]);
    }
    if (diagk[i] < 0) return fail(c, XG_ERR_ARG, "cg_setup: row without diagonal entry");
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
  std::vector<double> val(tot, 0.0);
  for (int64_t i = 0; i < nrow; ++i) {
    const int64_t s = i / kSlice, lane = i % kSlice;
    for (uint64_t j = ia[i]; j < ia[i + 1]; ++j) {
      const int64_t k = int64_t(j - ia[i]);
      const int64_t e = soff[s] + k * kSlice + lane;
      col[e] = static_cast<int32_t>(ja[j - b0] - b0);
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
  std::vector<int64_t> rowU(nrow + 1, 0);  // for locating (j,i) in row j's upper list
  for (int64_t i = 0; i < nrow; ++i) {
    const int64_t s2 = i / kSlice, lane = i % kSlice;
    int64_t kl = 0, ku = 0;
    for (uint64_t j = ia[i]; j < ia[i + 1]; ++j) {
      const int64_t cc = int64_t(ja[j - b0] - b0);
      const int64_t kfull = int64_t(j - ia[i]);
      if (cc < i) {
        const int64_t e = soffL[s2] + kl * kSlice + lane;
        colL[e] = int32_t(cc);
        posL[e] = int32_t(soff[s2] + kfull * kSlice + lane);
        ++kl;
      } else if (cc > i) {
        colU[soffU[s2] + ku * kSlice + lane] = int32_t(cc);
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
  d->nblk = (nrow + kBlock - 1) / kBlock;
  for (int pass = 0; pass < 2; ++pass) {
    Arena& A = d->arena;
    A.plan(d->soff, nslice + 1);
    A.plan(d->swidth, nslice);
    A.plan(d->col, tot);
    A.plan(d->a0, tot);
    A.plan(d->a, tot);
    A.plan(d->a32, tot);
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
    A.plan(d->q32, nrow);
    A.plan(d->z32, nrow);
    A.plan(d->d32, nrow);
    A.plan(d->e32, nrow);
    A.plan(d->p32[0], nrow);
    A.plan(d->p32[1], nrow);
    A.plan(d->partial, 3 * d->nblk);
    A.plan(d->scal, 1);
    A.plan(d->soffL, nslice + 1);
    A.plan(d->swL, nslice);
    A.plan(d->colL, colL.size());
    A.plan(d->posL, posL.size());
    A.plan(d->tposU, tposU.size());
    A.plan(d->soffU, nslice + 1);
    A.plan(d->swU, nslice);
    A.plan(d->colU, colU.size());
    A.plan(d->nvL, colL.size());
    A.plan(d->nvU, colU.size());
    A.plan(d->eL, colL.size());
    A.plan(d->eU, colU.size());
    A.plan(d->eF, tot);
    A.plan(d->srow, nrow);
    A.plan(d->u, nrow);
    A.plan(d->t, nrow);
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
  XG_CUDA(c, cudaMemsetAsync(d->nvL, 0, colL.size() * 4, s));
  XG_CUDA(c, cudaMemsetAsync(d->nvU, 0, colU.size() * 4, s));
  XG_CUDA(c, cudaMemsetAsync(d->eU, 0, colU.size() * 4, s));
  XG_CUDA(c, cudaMemsetAsync(d->x, 0, nrow * 8, s));
  XG_CUDA(c, cudaMemsetAsync(d->b, 0, nrow * 8, s));
  XG_CUDA(c, cudaMemsetAsync(d->bcmask, 0, nrow, s));
  XG_CUDA(c, cudaMemsetAsync(d->scal, 0, sizeof(CGScalars), s));
  k_copy_values<<<blocks_for(tot, kBlock), kBlock, 0, s>>>(tot, d->a0, d->a, d->a32);
  XG_CHECK_LAUNCH(c);
  XG_CUDA(c, cudaStreamSynchronize(s));
  return XG_OK;
}

int xg_cg_mult(xg_ctx* c, const double* x, double* y) {
  int rc = use(c);
  if (rc) return rc;
  CGDev* d = c->cg;
  if (!d) return fail(c, XG_ERR_STATE, "cg_mult before cg_setup");
  if (!x || !y) return fail(c, XG_ERR_ARG, "cg_mult: null vector");
  XG_CUDA(c, cudaMemcpyAsync(d->r, x, d->n * 8, cudaMemcpyHostToDevice, c->stream));
  k_spmv<<<blocks_for(d->n, kBlock), kBlock, 0, c->stream>>>(d->n, d->soff, d->swidth, d->col,
                                                              d->a0, d->r, d->q);
  XG_CHECK_LAUNCH(c);
  XG_CUDA(c, cudaMemcpyAsync(y, d->q, d->n * 8, cudaMemcpyDeviceToHost, c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}

int xg_cg_init(xg_ctx* c, const double* x, const double* b, const double* neubc, int64_t ndir,
               const uint64_t* dirnodes, const double* dirvals, int apply, int pc) {
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
  d->geom_set = false;
  d->factor_set = false;
  if (d->apply) {
    std::vector<uint8_t> mask(n, 0);
    std::vector<double> val(n, 0.0);
    for (int64_t k = 0; k < ndir; ++k) {
      if (dirnodes[k] >= static_cast<uint64_t>(n))
        return fail(c, XG_ERR_ARG, "cg_init: Dirichlet node out of range");
      mask[dirnodes[k]] = 1;
      val[dirnodes[k]] = dirvals[k];
    }
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
  } else {
    XG_CUDA(c, cudaMemsetAsync(d->bcmask, 0, n, s));
    k_copy_values<<<blocks_for(d->nent, kBlock), kBlock, 0, s>>>(d->nent, d->a0, d->a, d->a32);
    XG_CHECK_LAUNCH(c);
  }
  CGScalars h{};
  h.pc = pc;
  XG_CUDA(c, cudaMemcpyAsync(d->scal, &h, sizeof(h), cudaMemcpyHostToDevice, s));
  k_setup<<<blocks_for(n, kBlock), kBlock, 0, s>>>(n, d->soff, d->swidth, d->col, d->a, d->diagpos,
                                                    d->x, d->b, d->r, d->d, d->z, d->p[0], d->d32,
                                                    d->partial, d->nblk, d->scal);
  XG_CHECK_LAUNCH(c);
  if (pc == 2) {
    int rf = build_factor(c, d);
    if (rf) return rf;
    const unsigned nb = blocks_for(n, kBlock);
    k_pc_upper<double><<<nb, kBlock, 0, s>>>(n, tri_u(d), d->nvU, d->srow, d->r, d->u, d->scal);
    k_pc_lower<double, false><<<nb, kBlock, 0, s>>>(n, tri_l(d), d->nvL, d->srow, d->bcmask, d->u,
                                                    d->r, d->z, nullptr, d->partial, d->nblk,
                                                    d->scal);
    XG_CHECK_LAUNCH(c);
  }
  d->cur = 0;
  XG_CUDA(c, cudaStreamSynchronize(s));
  d->ready = true;
  return XG_OK;
}

namespace {
int cg_iterate(xg_ctx* c, CGDev* d, int64_t maxit, double tol, CGScalars* h) {
  cudaStream_t s = c->stream;
  // tol and maxit into the device scalars without touching the rest
  XG_CUDA(c, cudaMemcpyAsync(&d->scal->tol, &tol, sizeof(double), cudaMemcpyHostToDevice, s));
  XG_CUDA(c, cudaMemcpyAsync(&d->scal->maxit, &maxit, sizeof(int64_t), cudaMemcpyHostToDevice, s));
  const unsigned nb = static_cast<unsigned>(d->nblk);
  for (;;) {
    for (int k = 0; k < kBatch; ++k) {
      double* pold = d->p[d->cur];
      double* pnew = d->p[d->cur ^ 1];
      k_iter_a<<<nb, kBlock, 0, s>>>(d->n, d->soff, d->swidth, d->col, d->a, d->z, pold, pnew,
                                     d->q, d->partial, d->nblk, d->scal);
      if (d->pc == 2) {
        k_iter_b<true><<<nb, kBlock, 0, s>>>(d->n, d->q, d->d, pnew, d->r, d->z, d->x, d->partial,
                                             d->nblk, d->scal);
        k_pc_upper<double><<<nb, kBlock, 0, s>>>(d->n, tri_u(d), d->nvU, d->srow, d->r, d->u,
                                                 d->scal);
        k_pc_lower<double, false><<<nb, kBlock, 0, s>>>(d->n, tri_l(d), d->nvL, d->srow,
                                                        d->bcmask, d->u, d->r, d->z, nullptr,
                                                        d->partial, d->nblk, d->scal);
      } else {
        k_iter_b<false><<<nb, kBlock, 0, s>>>(d->n, d->q, d->d, pnew, d->r, d->z, d->x,
                                              d->partial, d->nblk, d->scal);
      }
      d->cur ^= 1;
    }
    XG_CHECK_LAUNCH(c);
    int rc = read_scal(c, d, h);
    if (rc) return rc;
    if (h->done) break;
  }
  // the parity of p buffers only matters while iterating; a finished solve
  // leaves p unused
  return XG_OK;
}
}  // namespace

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
  if (maxit <= 0 || inner_maxit <= 0 || !(tol >= 0) || !(inner_tol > 0))
    return fail(c, XG_ERR_ARG, "cg_solve_mixed: bad limits");
  cudaStream_t s = c->stream;
  const unsigned nb = static_cast<unsigned>(d->nblk);
  CGScalars h{};
  rc = read_scal(c, d, &h);
  if (rc) return rc;
  const double nb0 = h.normb > 1.0e-14 ? h.normb : 1.0;
  int64_t nout = 0, nin = 0;
  double nr = 0.0;
  bool conv = false;
  for (;;) {
    k_outer_res<<<nb, kBlock, 0, s>>>(d->n, d->soff, d->swidth, d->col, d->a, d->x, d->b, d->d32,
                                      d->r32, d->z32, d->p32[0], d->e32, d->partial, d->nblk,
                                      d->scal);
    XG_CHECK_LAUNCH(c);
    if (d->pc == 2) {
      k_pc_upper<float><<<nb, kBlock, 0, s>>>(d->n, tri_u(d), d->nvU, d->srow, d->r32, d->u32,
                                              d->scal);
      k_pc_lower<float, false><<<nb, kBlock, 0, s>>>(d->n, tri_l(d), d->nvL, d->srow, d->bcmask,
                                                     d->u32, d->r32, d->z32, nullptr, d->partial,
                                                     d->nblk, d->scal);
      XG_CHECK_LAUNCH(c);
    }
    rc = read_scal(c, d, &h);
    if (rc) return rc;
    nr = std::sqrt(h.rr);
    if (nr < tol * nb0) {
      conv = true;
      break;
    }
    if (nout >= maxit || nin >= maxit * inner_maxit) break;
    k_set_inner<<<1, 1, 0, s>>>(d->scal, inner_tol, inner_maxit);
    XG_CHECK_LAUNCH(c);
    int cur = 0;
    for (;;) {
      for (int k = 0; k < kBatch; ++k) {
        k_in_a<<<nb, kBlock, 0, s>>>(d->n, d->soff, d->swidth, d->col, d->a32, d->z32,
                                     d->p32[cur], d->p32[cur ^ 1], d->q32, d->partial, d->nblk,
                                     d->scal);
        if (d->pc == 2) {
          k_in_b<true><<<nb, kBlock, 0, s>>>(d->n, d->q32, d->d32, d->p32[cur ^ 1], d->r32,
                                             d->z32, d->e32, d->partial, d->nblk, d->scal);
          k_pc_upper<float><<<nb, kBlock, 0, s>>>(d->n, tri_u(d), d->nvU, d->srow, d->r32,
                                                  d->u32, d->scal);
          k_pc_lower<float, false><<<nb, kBlock, 0, s>>>(d->n, tri_l(d), d->nvL, d->srow,
                                                         d->bcmask, d->u32, d->r32, d->z32,
                                                         nullptr, d->partial, d->nblk, d->scal);
        } else {
          k_in_b<false><<<nb, kBlock, 0, s>>>(d->n, d->q32, d->d32, d->p32[cur ^ 1], d->r32,
                                              d->z32, d->e32, d->partial, d->nblk, d->scal);
        }
        cur ^= 1;
      }
      XG_CHECK_LAUNCH(c);
      rc = read_scal(c, d, &h);
      if (rc) return rc;
      if (h.done) break;
    }
    nin += h.it;
    k_add_correction<<<blocks_for(d->n, kBlock), kBlock, 0, s>>>(d->n, d->e32, d->x);
    XG_CHECK_LAUNCH(c);
    ++nout;
  }
  d->last_it = nin;
  d->inner_its = nin;
  d->last_normr = nr;
  d->last_normb = nb0;
  d->last_conv = conv;
  if (outer) *outer = nout;
  if (inner) *inner = nin;
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

int xg_cg_precondition(xg_ctx* c, const double* r, double* z) {
  int rc = use(c);
  if (rc) return rc;
  CGDev* d = c->cg;
  if (!d || !d->ready) return fail(c, XG_ERR_STATE, "cg_precondition before cg_init");
  if (!r || !z) return fail(c, XG_ERR_ARG, "cg_precondition: null vector");
  cudaStream_t s = c->stream;
  const unsigned nb = blocks_for(d->n, kBlock);
  XG_CUDA(c, cudaMemcpyAsync(d->q, r, d->n * 8, cudaMemcpyHostToDevice, s));
  // a scratch copy of the scalars with done = 0 so the passes run
  CGScalars h{};
  CGScalars* sc = d->scal + 0;
  XG_CUDA(c, cudaMemcpyAsync(&h, sc, sizeof(h), cudaMemcpyDeviceToHost, s));
  XG_CUDA(c, cudaStreamSynchronize(s));
  int32_t zero = 0;
  XG_CUDA(c, cudaMemcpyAsync(&sc->done, &zero, sizeof(int32_t), cudaMemcpyHostToDevice, s));
  if (d->pc == 2) {
    if (!d->factor_set) {
      rc = build_factor(c, d);
      if (rc) return rc;
    }
    k_pc_upper<double><<<nb, kBlock, 0, s>>>(d->n, tri_u(d), d->nvU, d->srow, d->q, d->u, sc);
    k_pc_lower<double, false><<<nb, kBlock, 0, s>>>(d->n, tri_l(d), d->nvL, d->srow, d->bcmask,
                                                    d->u, d->q, d->t, nullptr, d->partial,
                                                    d->nblk, sc);
  } else {
    k_jacobi_apply<<<nb, kBlock, 0, s>>>(d->n, d->q, d->d, d->t);
  }
  XG_CHECK_LAUNCH(c);
  XG_CUDA(c, cudaMemcpyAsync(sc, &h, sizeof(h), cudaMemcpyHostToDevice, s));
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
