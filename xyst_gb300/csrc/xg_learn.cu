// Learned preconditioner for the pressure-Poisson CG: a message-passing
// network on the matrix graph that emits the strictly lower factor N of
// M^-1 = -S (I+N)(I+N)^T S (the pc = 2 preconditioner of xg_cg.cu).
//
// There is no counterpart in the reference, whose ConjugateGradients offers
// the "none" and "jacobi" preconditioners only.  Everything here runs on the
// device: inference (at xg_cg_init with a model attached), the training loss
// and its gradient through the factor and the network, and Adam.
//
// Network (hidden width H = 64), on a system with row scales s_i = 1/sqrt|a_ii|
// and normalised couplings e_ij = a_ij s_i s_j (0 at Dirichlet nodes):
//   x_i  = [1, dirichlet_i, sum_j e_ij, degree_i / 16]
//   h0   = relu(x W0 + b0)
//   h_l  = relu([h_{l-1}, E h_{l-1}] W_l + b_l)          l = 1, 2, 3
//   [a|b] = h3 Wo
//   o_ij = w . relu(a_i + b_j + c e_ij + d) + ob          every lower edge i > j
//   N_ij = e_ij (1 + tanh o_ij)
// The dense layers run as BF16 tensor-core GEMMs with FP32 accumulation
// (precision 1) or in FP32 (precision 0); the backward pass is FP32 and
// every reduction over nodes or edges goes through fixed-order block
// partials, so a gradient is bit-reproducible.
//
// Loss: Kaporin's trace functional of the factorised approximate inverse.
// With unit-diagonal L = I + N, det(L^T A^ L) = det(A^) is fixed (A^ = I - E),
// so the Kaporin condition number of L^T A^ L falls with its trace:
//   loss = (tr(L^T A^ L) - n) / n
//        = (1/n) sum_j [-2 sum_i n_ij e_ij + sum_i n_ij^2 - sum_{i!=k} n_ij n_kj e_ik]
//   d loss / d n_ij = (2/n) (n_ij - e_ij - sum_{k != i} e_ik n_kj)
// (its minimiser on A's lower pattern is the factorised sparse approximate
// inverse with unit diagonal); training needs the matrix only, no solves.

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "xg_internal.hpp"

namespace xg {
namespace {

constexpr int H = 64;
constexpr int kSlice = 32;
constexpr int kThreads = 256;
constexpr int kRowsPerBlock = kThreads / 32;  // warp-per-row kernels
constexpr int kWgradBlocks = 296;             // 2 x 148 SMs' worth of weight-gradient partials

// flat FP32 parameter layout
constexpr int64_t oW0 = 0;
constexpr int64_t ob0 = oW0 + 4 * H;
constexpr int64_t oW1 = ob0 + H;
constexpr int64_t ob1 = oW1 + 2 * H * H;
constexpr int64_t oW2 = ob1 + H;
constexpr int64_t ob2 = oW2 + 2 * H * H;
constexpr int64_t oW3 = ob2 + H;
constexpr int64_t ob3 = oW3 + 2 * H * H;
constexpr int64_t oWo = ob3 + H;
constexpr int64_t oc = oWo + 2 * H * H;
constexpr int64_t oc2 = oc + H;
constexpr int64_t od = oc2 + H;
constexpr int64_t ow = od + H;
constexpr int64_t oob = ow + H;
constexpr int64_t kNParams = oob + 1;
constexpr int64_t kLayerW[3] = {oW1, oW2, oW3};
constexpr int64_t kLayerB[3] = {ob1, ob2, ob3};

// BF16 B-fragment images of the tensor-core layers: W1..W3 (K 128, N 64) and
// Wo (K 64, N 128); K * N / 2 32-bit words each.
constexpr int64_t kFragWords = 2 * H * H / 2;

// ---------------------------------------------------------------- helpers

__device__ __forceinline__ float relu(float v) { return v > 0.f ? v : 0.f; }

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  uint32_t u;
  memcpy(&u, &v, 4);
  return u;
}

// Fixed-order block sum of one double per thread; thread 0 gets the total.
__device__ double block_sum(double v) {
  __shared__ double red[kThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kThreads / 32; ++w) t += red[w];
  __syncthreads();
  return t;
}

// ---------------------------------------------------------------- node features

__global__ void k_features(int64_t n, const int32_t* __restrict__ soff,
                           const int32_t* __restrict__ sw, const int32_t* __restrict__ col,
                           const float* __restrict__ eF, const uint8_t* __restrict__ mask,
                           float* __restrict__ x4) {
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int lane = int(i & 31);
  const int32_t off = soff[i >> 5], w = sw[i >> 5];
  float rs = 0.f, r2 = 0.f;
  int deg = 0;
  for (int k = 0; k < w; ++k) {
    const int32_t p = off + k * kSlice + lane;
    const int32_t j = col[p];
    if (j < 0) continue;
    if (j != i) ++deg;
    const float e = eF[p];
    rs += e;
    r2 += e * e;
  }
  x4[i * 4 + 0] = mask[i] ? 1.f : 0.f;
  x4[i * 4 + 1] = rs;
  x4[i * 4 + 2] = r2;
  x4[i * 4 + 3] = float(deg) / 16.f;
}

// h0 = relu(x W0 + b0), one thread per (node, unit).
__global__ void k_input_layer(int64_t n, const float* __restrict__ x4,
                              const float* __restrict__ theta, float* __restrict__ h0) {
  int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (t >= n * H) return;
  const int64_t i = t / H;
  const int o = int(t % H);
  const float* W0 = theta + oW0;
  float v = theta[ob0 + o];
#pragma unroll
  for (int k = 0; k < 4; ++k) v += x4[i * 4 + k] * W0[k * H + o];
  h0[t] = relu(v);
}

// ---------------------------------------------------------------- E X (warp per row)

// Y = (add + E X) o [maskH > 0]   (add, maskH optional; X, Y, add, maskH n x 64)
__global__ void __launch_bounds__(kThreads) k_spmm(int64_t n, const int32_t* __restrict__ soff,
                                                   const int32_t* __restrict__ sw,
                                                   const int32_t* __restrict__ col,
                                                   const float* __restrict__ eF,
                                                   const float* __restrict__ X,
                                                   const float* __restrict__ add,
                                                   const float* __restrict__ maskH,
                                                   float* __restrict__ Y) {
  const int64_t i = blockIdx.x * int64_t(kRowsPerBlock) + (threadIdx.x >> 5);
  if (i >= n) return;
  const int lane = threadIdx.x & 31;
  const int li = int(i & 31);
  const int32_t off = soff[i >> 5], w = sw[i >> 5];
  float2 acc = add ? reinterpret_cast<const float2*>(add + i * H)[lane] : make_float2(0.f, 0.f);
  for (int k = 0; k < w; ++k) {
    const int32_t p = off + k * kSlice + li;
    const int32_t j = __ldg(col + p);
    if (j < 0) continue;
    const float e = __ldg(eF + p);
    if (e == 0.f) continue;
    const float2 xj = __ldg(reinterpret_cast<const float2*>(X + int64_t(j) * H) + lane);
    acc.x += e * xj.x;
    acc.y += e * xj.y;
  }
  if (maskH) {
    const float2 m = reinterpret_cast<const float2*>(maskH + i * H)[lane];
    if (!(m.x > 0.f)) acc.x = 0.f;
    if (!(m.y > 0.f)) acc.y = 0.f;
  }
  reinterpret_cast<float2*>(Y + i * H)[lane] = acc;
}

// ---------------------------------------------------------------- dense layers

// Y[i, :] = act([X1 | X2][i, :] W + bias) (o [maskY > 0]).  X1, X2 are n x 64
// (X2 may be null: K = 64); Y is N wide, split into Y1 (columns 0..63) and Y2
// (64..127).  W is K x N row-major, or N x K row-major with TRANS (the
// transpose of a forward weight, for the backward pass).  FP32 on CUDA cores.
template <int K, int N, bool TRANS>
__global__ void __launch_bounds__(kThreads) k_dense_f32(int64_t n, const float* __restrict__ X1,
                                                        const float* __restrict__ X2,
                                                        const float* __restrict__ W,
                                                        const float* __restrict__ bias, int act,
                                                        const float* __restrict__ maskY,
                                                        float* __restrict__ Y1,
                                                        float* __restrict__ Y2) {
  constexpr int R = 16;                 // rows per pass
  constexpr int G = kThreads / N;       // row groups
  constexpr int RPT = R / G;            // rows per thread
  __shared__ float Ws[K * N];
  __shared__ float Xs[R][K + 1];
  for (int t = threadIdx.x; t < K * N; t += kThreads) {
    const int k = t / N, o = t % N;
    Ws[t] = TRANS ? W[o * K + k] : W[t];
  }
  const int o = threadIdx.x % N, g = threadIdx.x / N;
  const float bo = bias ? bias[o] : 0.f;
  for (int64_t r0 = int64_t(blockIdx.x) * R; r0 < n; r0 += int64_t(gridDim.x) * R) {
    __syncthreads();
    for (int t = threadIdx.x; t < R * K; t += kThreads) {
      const int r = t / K, k = t % K;
      const int64_t i = r0 + r;
      float v = 0.f;
      if (i < n) v = k < H ? X1[i * H + k] : X2[i * H + (k - H)];
      Xs[r][k] = v;
    }
    __syncthreads();
    float acc[RPT];
#pragma unroll
    for (int q = 0; q < RPT; ++q) acc[q] = bo;
#pragma unroll 4
    for (int k = 0; k < K; ++k) {
      const float wk = Ws[k * N + o];
#pragma unroll
      for (int q = 0; q < RPT; ++q) acc[q] += Xs[g + q * G][k] * wk;
    }
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
      const int64_t i = r0 + g + q * G;
      if (i >= n) continue;
      float v = act ? relu(acc[q]) : acc[q];
      if (maskY && !(maskY[i * N + o] > 0.f)) v = 0.f;
      if (o < H)
        Y1[i * H + o] = v;
      else
        Y2[i * H + (o - H)] = v;
    }
  }
}

// BF16 tensor-core version of the forward layers (mma.sync m16n8k16, FP32
// accumulation): each warp owns 16-row tiles, its A fragments come straight
// from the FP32 activations (one 32-byte sector per row and k-step), the
// B fragments from a shared-memory copy of the packed weight image.
template <int K, int N>
__global__ void __launch_bounds__(kThreads) k_dense_tc(int64_t n, const float* __restrict__ X1,
                                                       const float* __restrict__ X2,
                                                       const uint32_t* __restrict__ wfrag,
                                                       const float* __restrict__ bias, int act,
                                                       float* __restrict__ Y1,
                                                       float* __restrict__ Y2) {
  constexpr int KS = K / 16, NT = N / 8;
  __shared__ uint2 Bs[KS * NT * 32];
  for (int t = threadIdx.x; t < KS * NT * 32; t += kThreads)
    Bs[t] = reinterpret_cast<const uint2*>(wfrag)[t];
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
  const int64_t ntile = (n + 15) / 16;
  const int64_t wstride = int64_t(gridDim.x) * (kThreads / 32);
  for (int64_t tile = blockIdx.x * int64_t(kThreads / 32) + (threadIdx.x >> 5); tile < ntile;
       tile += wstride) {
    const int64_t ra = tile * 16 + g, rb = ra + 8;
    float acc[NT][4];
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll
    for (int ks = 0; ks < KS; ++ks) {
      const float* X = (ks * 16 < H) ? X1 : X2;
      const int c0 = (ks * 16) % H + 2 * tq;
      float2 v00 = make_float2(0.f, 0.f), v10 = v00, v01 = v00, v11 = v00;
      if (ra < n) {
        v00 = __ldg(reinterpret_cast<const float2*>(X + ra * H + c0));
        v01 = __ldg(reinterpret_cast<const float2*>(X + ra * H + c0 + 8));
      }
      if (rb < n) {
        v10 = __ldg(reinterpret_cast<const float2*>(X + rb * H + c0));
        v11 = __ldg(reinterpret_cast<const float2*>(X + rb * H + c0 + 8));
      }
      const uint32_t a0 = pack_bf16(v00.x, v00.y), a1 = pack_bf16(v10.x, v10.y);
      const uint32_t a2 = pack_bf16(v01.x, v01.y), a3 = pack_bf16(v11.x, v11.y);
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) {
        const uint2 b = Bs[(ks * NT + nt) * 32 + lane];
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
            "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
            : "+f"(acc[nt][0]), "+f"(acc[nt][1]), "+f"(acc[nt][2]), "+f"(acc[nt][3])
            : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b.x), "r"(b.y));
      }
    }
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
      const int cc = nt * 8 + 2 * tq;
      const float b0 = bias ? bias[cc] : 0.f, b1 = bias ? bias[cc + 1] : 0.f;
      float2 ya = make_float2(acc[nt][0] + b0, acc[nt][1] + b1);
      float2 yb = make_float2(acc[nt][2] + b0, acc[nt][3] + b1);
      if (act) {
        ya.x = relu(ya.x), ya.y = relu(ya.y), yb.x = relu(yb.x), yb.y = relu(yb.y);
      }
      float* Y = cc < H ? Y1 : Y2;
      const int cy = cc % H;
      if (ra < n) *reinterpret_cast<float2*>(Y + ra * H + cy) = ya;
      if (rb < n) *reinterpret_cast<float2*>(Y + rb * H + cy) = yb;
    }
  }
}

// Packed BF16 B fragments of a K x N row-major FP32 weight: word pair
// ((ks * N/8 + nt) * 32 + lane) holds W[k0..k0+1][col] and W[k0+8..k0+9][col]
// with col = nt * 8 + lane / 4, k0 = ks * 16 + 2 (lane % 4).
__global__ void k_pack_frag(const float* __restrict__ W, int K, int N, uint32_t* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int NT = N / 8;
  if (t >= (K / 16) * NT * 32) return;
  const int lane = t & 31, blk = t >> 5;
  const int ks = blk / NT, nt = blk % NT;
  const int colw = nt * 8 + (lane >> 2), k0 = ks * 16 + 2 * (lane & 3);
  out[2 * t + 0] = pack_bf16(W[k0 * N + colw], W[(k0 + 1) * N + colw]);
  out[2 * t + 1] = pack_bf16(W[(k0 + 8) * N + colw], W[(k0 + 9) * N + colw]);
}

// ---------------------------------------------------------------- weight gradients

// Per-block partials of dW = [X1 | X2]^T dY (K x N) and, with BIAS, db = sum dY.
// X1 is n x K1 (K1 = 4 or 64), X2 n x 64 or null; dY = [dY1 | dY2], N = 64 or 128.
template <int K1, int K2, int N, bool BIAS>
__global__ void __launch_bounds__(kThreads) k_wgrad(int64_t n, const float* __restrict__ X1,
                                                    const float* __restrict__ X2,
                                                    const float* __restrict__ dY1,
                                                    const float* __restrict__ dY2,
                                                    float* __restrict__ part) {
  constexpr int K = K1 + K2;
  constexpr int R = 32;
  constexpr int NOUT = K * N + (BIAS ? N : 0);
  constexpr int PER = (NOUT + kThreads - 1) / kThreads;
  __shared__ float Xs[R][K + 1];
  __shared__ float Ys[R][N];
  float acc[PER];
#pragma unroll
  for (int q = 0; q < PER; ++q) acc[q] = 0.f;
  for (int64_t r0 = int64_t(blockIdx.x) * R; r0 < n; r0 += int64_t(gridDim.x) * R) {
    __syncthreads();
    for (int t = threadIdx.x; t < R * K; t += kThreads) {
      const int r = t / K, k = t % K;
      const int64_t i = r0 + r;
      float v = 0.f;
      if (i < n) v = k < K1 ? X1[i * K1 + k] : X2[i * H + (k - K1)];
      Xs[r][k] = v;
    }
    for (int t = threadIdx.x; t < R * N; t += kThreads) {
      const int r = t / N, o = t % N;
      const int64_t i = r0 + r;
      float v = 0.f;
      if (i < n) v = o < H ? dY1[i * H + o] : dY2[i * H + (o - H)];
      Ys[r][o] = v;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int idx = threadIdx.x + q * kThreads;
      if (idx >= NOUT) continue;
      float s = 0.f;
      if (idx < K * N) {
        const int k = idx / N, o = idx % N;
#pragma unroll 8
        for (int r = 0; r < R; ++r) s += Xs[r][k] * Ys[r][o];
      } else {
        const int o = idx - K * N;
#pragma unroll 8
        for (int r = 0; r < R; ++r) s += Ys[r][o];
      }
      acc[q] += s;
    }
  }
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int idx = threadIdx.x + q * kThreads;
    if (idx < NOUT) part[int64_t(blockIdx.x) * NOUT + idx] = acc[q];
  }
}

// grad[dst[k]] += sum over blocks of part[blk][k] (fixed order, FP64).
// dst maps output k to a parameter index: k < nw -> wofs + k, else bofs + (k - nw).
__global__ void k_reduce_parts(const float* __restrict__ part, int nblk, int nout, int nw,
                               int64_t wofs, int64_t bofs, float* __restrict__ grad) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nout) return;
  double s = 0.0;
  for (int b = 0; b < nblk; ++b) s += part[int64_t(b) * nout + k];
  const int64_t dst = k < nw ? wofs + k : bofs + (k - nw);
  grad[dst] += float(s);
}

// ---------------------------------------------------------------- edge network

struct EdgeParams {
  const float* c;
  const float* c2;
  const float* d;
  const float* w;
  const float* ob;
};

EdgeParams edge_params(const float* theta) {
  return EdgeParams{theta + oc, theta + oc2, theta + od, theta + ow, theta + oob};
}

// Edge inputs of unit pair (2 lane, 2 lane + 1): c, c2, d, w.
struct EdgeLane {
  float2 c, c2, d, w;
  __device__ EdgeLane(const EdgeParams& P, int lane)
      : c(reinterpret_cast<const float2*>(P.c)[lane]),
        c2(reinterpret_cast<const float2*>(P.c2)[lane]),
        d(reinterpret_cast<const float2*>(P.d)[lane]),
        w(reinterpret_cast<const float2*>(P.w)[lane]) {}
  __device__ float2 z(float2 ai, float2 bj, float e, float t) const {
    return make_float2(ai.x + bj.x + c.x * e + c2.x * t + d.x, ai.y + bj.y + c.y * e + c2.y * t + d.y);
  }
};

// Forward over the lower edges (warp per row i, lane = units 2 lane, 2 lane + 1).
// N_ij = (e_ij + t_ij) (1 + tanh o_ij), written to the lower layout and,
// transposed, the upper one; training also keeps tanh(o) in thL.  t_ij is read
// from the upper layout (tU).
template <bool TRAIN>
__global__ void __launch_bounds__(kThreads) k_edge_fwd(int64_t n, const int32_t* __restrict__ soffL,
                                                       const int32_t* __restrict__ swL,
                                                       const int32_t* __restrict__ colL,
                                                       const float* __restrict__ eL,
                                                       const int32_t* __restrict__ tposU,
                                                       const float* __restrict__ tU,
                                                       const float* __restrict__ A,
                                                       const float* __restrict__ B, EdgeParams P,
                                                       float* __restrict__ nL,
                                                       float* __restrict__ nU,
                                                       float* __restrict__ thL) {
  const int64_t i = blockIdx.x * int64_t(kRowsPerBlock) + (threadIdx.x >> 5);
  if (i >= n) return;
  const int lane = threadIdx.x & 31;
  const int li = int(i & 31);
  const int32_t off = soffL[i >> 5], w = swL[i >> 5];
  const float2 ai = reinterpret_cast<const float2*>(A + i * H)[lane];
  const EdgeLane E(P, lane);
  const float ob = *P.ob;
  for (int k = 0; k < w; ++k) {
    const int32_t p = off + k * kSlice + li;
    const int32_t j = __ldg(colL + p);
    if (j < 0) continue;
    const float e = __ldg(eL + p);
    const int32_t pu = tposU[p];
    const float t = tU[pu];
    float nv = 0.f, th = 0.f;
    // e = t = 0 on edges at Dirichlet nodes (N = 0 there); a zero coupling
    // elsewhere can still carry a second-order term
    if (e != 0.f || t != 0.f) {
      const float2 bj = __ldg(reinterpret_cast<const float2*>(B + int64_t(j) * H) + lane);
      const float2 z = E.z(ai, bj, e, t);
      const float o = warp_sum(E.w.x * relu(z.x) + E.w.y * relu(z.y)) + ob;
      th = tanhf(o);
      nv = (e + t) * (1.f + th);
    }
    if (lane == 0) {
      nL[p] = nv;
      nU[pu] = nv;
      if (TRAIN) thL[p] = th;
    }
  }
}

// Backward over the lower edges: d loss / d N_ij (upper layout, from
// k_cross) through tanh and the edge MLP.  da_i (sum over the row's edges) is written
// per row; do_ij goes to the upper layout for the b_j pass; the gradients of
// c, c2, d, w, ob leave as per-block partials (fixed order).
constexpr int kEdgeParts = 4 * H + 1;
__global__ void __launch_bounds__(kThreads) k_edge_bwd_lower(
    int64_t n, const int32_t* __restrict__ soffL, const int32_t* __restrict__ swL,
    const int32_t* __restrict__ colL, const float* __restrict__ eL,
    const int32_t* __restrict__ tposU, const float* __restrict__ tU,
    const float* __restrict__ thL, const float* __restrict__ A, const float* __restrict__ B,
    EdgeParams P, const float* __restrict__ dnU, float* __restrict__ da, float* __restrict__ doU,
    float* __restrict__ part) {
  constexpr int NOUT = kEdgeParts;
  __shared__ float red[kRowsPerBlock][NOUT];
  const int64_t i = blockIdx.x * int64_t(kRowsPerBlock) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float2 gw = make_float2(0.f, 0.f), gc = gw, gc2 = gw, gd = gw, dai = gw;
  float gob = 0.f;
  if (i < n) {
    const int li = int(i & 31);
    const int32_t off = soffL[i >> 5], w = swL[i >> 5];
    const float2 ai = reinterpret_cast<const float2*>(A + i * H)[lane];
    const EdgeLane E(P, lane);
    for (int k = 0; k < w; ++k) {
      const int32_t p = off + k * kSlice + li;
      const int32_t j = __ldg(colL + p);
      if (j < 0) continue;
      const float e = __ldg(eL + p);
      const int32_t pu = tposU[p];
      const float t = tU[pu];
      if (e == 0.f && t == 0.f) {
        if (lane == 0) doU[pu] = 0.f;
        continue;
      }
      const float th = thL[p];
      const float dov = dnU[pu] * (e + t) * (1.f - th * th);
      const float2 bj = __ldg(reinterpret_cast<const float2*>(B + int64_t(j) * H) + lane);
      const float2 z = E.z(ai, bj, e, t);
      const float dz0 = z.x > 0.f ? dov * E.w.x : 0.f;
      const float dz1 = z.y > 0.f ? dov * E.w.y : 0.f;
      dai.x += dz0;
      dai.y += dz1;
      gw.x += dov * relu(z.x);
      gw.y += dov * relu(z.y);
      gc.x += dz0 * e;
      gc.y += dz1 * e;
      gc2.x += dz0 * t;
      gc2.y += dz1 * t;
      gd.x += dz0;
      gd.y += dz1;
      gob += dov;
      if (lane == 0) doU[pu] = dov;
    }
    reinterpret_cast<float2*>(da + i * H)[lane] = dai;
  }
  red[wid][2 * lane] = gc.x;
  red[wid][2 * lane + 1] = gc.y;
  red[wid][H + 2 * lane] = gc2.x;
  red[wid][H + 2 * lane + 1] = gc2.y;
  red[wid][2 * H + 2 * lane] = gd.x;
  red[wid][2 * H + 2 * lane + 1] = gd.y;
  red[wid][3 * H + 2 * lane] = gw.x;
  red[wid][3 * H + 2 * lane + 1] = gw.y;
  if (lane == 0) red[wid][4 * H] = gob;
  __syncthreads();
  for (int k = threadIdx.x; k < NOUT; k += kThreads) {
    float s = 0.f;
    for (int r = 0; r < kRowsPerBlock; ++r) s += red[r][k];
    part[int64_t(blockIdx.x) * NOUT + k] = s;
  }
}

// Backward to b_j: warp per row j over its upper entries (j, i), i > j.
__global__ void __launch_bounds__(kThreads) k_edge_bwd_upper(
    int64_t n, const int32_t* __restrict__ soffU, const int32_t* __restrict__ swU,
    const int32_t* __restrict__ colU, const float* __restrict__ eU, const float* __restrict__ tU,
    const float* __restrict__ doU, const float* __restrict__ A, const float* __restrict__ B,
    EdgeParams P, float* __restrict__ db) {
  const int64_t j = blockIdx.x * int64_t(kRowsPerBlock) + (threadIdx.x >> 5);
  if (j >= n) return;
  const int lane = threadIdx.x & 31;
  const int lj = int(j & 31);
  const int32_t off = soffU[j >> 5], w = swU[j >> 5];
  const float2 bj = reinterpret_cast<const float2*>(B + j * H)[lane];
  const EdgeLane E(P, lane);
  float2 acc = make_float2(0.f, 0.f);
  for (int k = 0; k < w; ++k) {
    const int32_t p = off + k * kSlice + lj;
    const int32_t i = __ldg(colU + p);
    if (i < 0) continue;
    const float dov = doU[p];
    if (dov == 0.f) continue;
    const float e = __ldg(eU + p);
    const float2 ai = __ldg(reinterpret_cast<const float2*>(A + int64_t(i) * H) + lane);
    const float2 z = E.z(ai, bj, e, tU[p]);
    if (z.x > 0.f) acc.x += dov * E.w.x;
    if (z.y > 0.f) acc.y += dov * E.w.y;
  }
  reinterpret_cast<float2*>(db + j * H)[lane] = acc;
}

// ---------------------------------------------------------------- trace loss

// Thread per column j (the upper-layout row j lists the lower edges (i, j)):
// for each of its edges the cross term sum_{k != i} e_ik n_kj, found by
// walking row i of the full layout and searching row j's sorted upper list.
// LOSS: writes d loss / d n_ij (upper layout) and per-block partials of the
// columns' loss terms (times n); otherwise writes the cross term itself
// (with n = e: the edge feature t).
template <bool LOSS>
__global__ void __launch_bounds__(kThreads) k_cross(int64_t n, const int32_t* __restrict__ soff,
                                                      const int32_t* __restrict__ sw,
                                                      const int32_t* __restrict__ col,
                                                      const float* __restrict__ eF,
                                                      const int32_t* __restrict__ soffU,
                                                      const int32_t* __restrict__ swU,
                                                      const int32_t* __restrict__ colU,
                                                      const float* __restrict__ eU,
                                                      const float* __restrict__ nU,
                                                      float* __restrict__ dnU,
                                                      double* __restrict__ part) {
  int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  double lj = 0.0;
  if (j < n) {
    const int lane = int(j & 31);
    const int32_t offj = soffU[j >> 5], wj = swU[j >> 5];
    const float two_n = float(2.0 / double(n));
    for (int a = 0; a < wj; ++a) {
      const int32_t pa = offj + a * kSlice + lane;
      const int32_t ia = colU[pa];
      if (ia < 0) break;  // padding closes the row
      const float na = nU[pa], ea = eU[pa];
      float cross = 0.f;
      const int32_t offi = soff[ia >> 5], wi = sw[ia >> 5];
      const int li = ia & 31;
      for (int k = 0; k < wi; ++k) {
        const int32_t pk = offi + k * kSlice + li;
        const int32_t c = col[pk];
        if (c < 0 || c == ia || c <= j) continue;
        const float eik = eF[pk];
        if (eik == 0.f) continue;
        // binary search for column c in row j's upper list (PAD sorts last)
        int lo = 0, hi = wj;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          const int32_t cm = colU[offj + mid * kSlice + lane];
          if (cm >= 0 && cm < c)
            lo = mid + 1;
          else
            hi = mid;
        }
        if (lo < wj && colU[offj + lo * kSlice + lane] == c)
          cross += eik * nU[offj + lo * kSlice + lane];
      }
      if (LOSS) {
        dnU[pa] = two_n * (na - ea - cross);
        lj += double(na) * (-2.0 * double(ea) + double(na) - double(cross));
      } else {
        dnU[pa] = cross;
      }
    }
  }
  if (LOSS) {
    const double t = block_sum(lj);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
  }
}

// out[slot] = sum of nblk partials, fixed order.
__global__ void k_sum_parts(const double* __restrict__ part, int64_t nblk, double* __restrict__ out,
                            int slot) {
  double s = 0.0;
  for (int64_t b = threadIdx.x; b < nblk; b += blockDim.x) s += part[b];
  const double t = block_sum(s);
  if (threadIdx.x == 0) out[slot] = t;
}

// ---------------------------------------------------------------- Adam

__global__ void k_adam(int64_t np, float* __restrict__ theta, const float* __restrict__ grad,
                       float* __restrict__ m, float* __restrict__ v, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
  int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (k >= np) return;
  const float g = grad[k];
  const float mk = b1 * m[k] + (1.f - b1) * g;
  const float vk = b2 * v[k] + (1.f - b2) * g * g;
  m[k] = mk;
  v[k] = vk;
  theta[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
}

}  // namespace
}  // namespace xg

// ---------------------------------------------------------------- the model object

struct xg_lpc {
  xg_ctx own;  // the model's device, stream and last error
  xg_ctx* home = &own;
  int precision = 1;  // 0: FP32 dense layers, 1: BF16 tensor cores
  int64_t step = 0;
  xg::Arena params;  // theta, grad, Adam moments, BF16 fragments, partials
  float *theta = nullptr, *grad = nullptr, *m1 = nullptr, *m2 = nullptr, *wpart = nullptr;
  uint32_t* frag = nullptr;  // 4 x kFragWords: W1, W2, W3, Wo
  double* lossv = nullptr;   // [x^.b^, e.g]
  // workspace, sized for the largest graph seen
  xg::Arena work;
  int64_t cap_n = 0, cap_l = 0, cap_u = 0;
  float *x4 = nullptr, *h[4] = {}, *mh[4] = {}, *A = nullptr, *B = nullptr;
  float *da = nullptr, *db = nullptr, *du = nullptr, *du2 = nullptr, *dih = nullptr,
        *dim = nullptr;
  float *nL = nullptr, *tL = nullptr, *nU = nullptr, *doU = nullptr, *dnU = nullptr,
        *tU = nullptr;
  double* dpart = nullptr;
  float* epart = nullptr;  // edge-parameter partials, one row per block
};

namespace xg {
namespace {

int ensure_work(xg_ctx* c, xg_lpc* m, int64_t n, int64_t nl, int64_t nu) {
  if (m->work.ready() && n <= m->cap_n && nl <= m->cap_l && nu <= m->cap_u) return XG_OK;
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  m->work.release();
  const int64_t N = std::max(n, m->cap_n), L = std::max(nl, m->cap_l),
                U = std::max(nu, m->cap_u);
  const int64_t nblk = (N + kThreads - 1) / kThreads;
  const int64_t nrb = (N + kRowsPerBlock - 1) / kRowsPerBlock;
  for (int pass = 0; pass < 2; ++pass) {
    Arena& W = m->work;
    W.plan(m->x4, N * 4);
    for (int l = 0; l < 4; ++l) W.plan(m->h[l], N * H);
    for (int l = 1; l < 4; ++l) W.plan(m->mh[l], N * H);
    W.plan(m->A, N * H);
    W.plan(m->B, N * H);
    W.plan(m->da, N * H);
    W.plan(m->db, N * H);
    W.plan(m->du, N * H);
    W.plan(m->du2, N * H);
    W.plan(m->dih, N * H);
    W.plan(m->dim, N * H);
    W.plan(m->nL, std::max<int64_t>(1, L));
    W.plan(m->tL, std::max<int64_t>(1, L));
    W.plan(m->nU, std::max<int64_t>(1, U));
    W.plan(m->doU, std::max<int64_t>(1, U));
    W.plan(m->dnU, std::max<int64_t>(1, U));
    W.plan(m->tU, std::max<int64_t>(1, U));
    W.plan(m->dpart, nblk);
    W.plan(m->epart, nrb * kEdgeParts);
    if (pass == 0) {
      cudaError_t e = W.reserve();
      if (e != cudaSuccess) {
        W.release();
        m->cap_n = m->cap_l = m->cap_u = 0;
        return fail(c, XG_ERR_CUDA, std::string("lpc workspace: ") + cudaGetErrorString(e));
      }
    }
  }
  m->cap_n = N;
  m->cap_l = L;
  m->cap_u = U;
  return XG_OK;
}

int refresh_frag(xg_ctx* c, xg_lpc* m) {
  cudaStream_t s = c->stream;
  for (int l = 0; l < 3; ++l) {
    k_pack_frag<<<(kFragWords / 2 + 255) / 256, 256, 0, s>>>(m->theta + kLayerW[l], 2 * H, H,
                                                             m->frag + l * kFragWords);
  }
  k_pack_frag<<<(kFragWords / 2 + 255) / 256, 256, 0, s>>>(m->theta + oWo, H, 2 * H,
                                                           m->frag + 3 * kFragWords);
  XG_CHECK_LAUNCH(c);
  return XG_OK;
}

// Network forward on g up to a and b (m->A, m->B).
int forward_nodes(xg_ctx* c, xg_lpc* m, const LpcGraph& g) {
  cudaStream_t s = c->stream;
  const int64_t n = g.n;
  const unsigned nb = blocks_for(n, kThreads);
  const unsigned nrb = blocks_for(n, kRowsPerBlock);
  k_features<<<nb, kThreads, 0, s>>>(n, g.soff, g.sw, g.col, g.eF, g.mask, m->x4);
  k_input_layer<<<blocks_for(n * H, kThreads), kThreads, 0, s>>>(n, m->x4, m->theta, m->h[0]);
  XG_CHECK_LAUNCH(c);
  const unsigned ngemm = static_cast<unsigned>(
      std::min<int64_t>(blocks_for(n, 32), 4 * 148));
  for (int l = 1; l <= 3; ++l) {
    k_spmm<<<nrb, kThreads, 0, s>>>(n, g.soff, g.sw, g.col, g.eF, m->h[l - 1], nullptr, nullptr,
                                    m->mh[l]);
    if (m->precision == 1)
      k_dense_tc<2 * H, H><<<ngemm, kThreads, 0, s>>>(n, m->h[l - 1], m->mh[l],
                                                      m->frag + (l - 1) * kFragWords,
                                                      m->theta + kLayerB[l - 1], 1, m->h[l],
                                                      nullptr);
    else
      k_dense_f32<2 * H, H, false><<<ngemm, kThreads, 0, s>>>(
          n, m->h[l - 1], m->mh[l], m->theta + kLayerW[l - 1], m->theta + kLayerB[l - 1], 1,
          nullptr, m->h[l], nullptr);
    XG_CHECK_LAUNCH(c);
  }
  if (m->precision == 1)
    k_dense_tc<H, 2 * H><<<ngemm, kThreads, 0, s>>>(n, m->h[3], nullptr, m->frag + 3 * kFragWords,
                                                    nullptr, 0, m->A, m->B);
  else
    k_dense_f32<H, 2 * H, false><<<ngemm, kThreads, 0, s>>>(n, m->h[3], nullptr, m->theta + oWo,
                                                            nullptr, 0, nullptr, m->A, m->B);
  XG_CHECK_LAUNCH(c);
  return XG_OK;
}

// t_ij = sum_{k > j, k != i} e_ik e_kj in the upper layout (m->tU).
int edge_feature(xg_ctx* c, xg_lpc* m, const LpcGraph& g) {
  k_cross<false><<<blocks_for(g.n, kThreads), kThreads, 0, c->stream>>>(
      g.n, g.soff, g.sw, g.col, g.eF, g.soffU, g.swU, g.colU, g.eU, g.eU, m->tU, nullptr);
  XG_CHECK_LAUNCH(c);
  return XG_OK;
}

template <int K1, int K2, int N, bool BIAS>
int wgrad(xg_ctx* c, xg_lpc* m, int64_t n, const float* X1, const float* X2, const float* dY1,
          const float* dY2, int64_t wofs, int64_t bofs) {
  cudaStream_t s = c->stream;
  constexpr int NOUT = (K1 + K2) * N + (BIAS ? N : 0);
  k_wgrad<K1, K2, N, BIAS><<<kWgradBlocks, kThreads, 0, s>>>(n, X1, X2, dY1, dY2, m->wpart);
  k_reduce_parts<<<(NOUT + 255) / 256, 256, 0, s>>>(m->wpart, kWgradBlocks, NOUT,
                                                    (K1 + K2) * N, wofs, bofs, m->grad);
  XG_CHECK_LAUNCH(c);
  return XG_OK;
}

}  // namespace

int lpc_factor(xg_ctx* c, xg_lpc* m, const LpcGraph& g, float* nvL, float* nvU) {
  if (!m) return fail(c, XG_ERR_ARG, "lpc_factor: null model");
  if (m->own.device != c->device)
    return fail(c, XG_ERR_ARG, "lpc_factor: model and system on different devices");
  int rc = ensure_work(c, m, g.n, g.nentL, g.nentU);
  if (rc) return rc;
  rc = forward_nodes(c, m, g);
  if (rc) return rc;
  rc = edge_feature(c, m, g);
  if (rc) return rc;
  k_edge_fwd<false><<<blocks_for(g.n, kRowsPerBlock), kThreads, 0, c->stream>>>(
      g.n, g.soffL, g.swL, g.colL, g.eL, g.tposU, m->tU, m->A, m->B, edge_params(m->theta), nvL,
      nvU, nullptr);
  XG_CHECK_LAUNCH(c);
  return XG_OK;
}

}  // namespace xg

using namespace xg;

extern "C" {

int64_t xg_lpc_nparams(void) { return kNParams; }

int xg_lpc_create(xg_ctx* c, int precision, xg_lpc** out) {
  int rc = use(c);
  if (rc) return rc;
  if (!out) return fail(c, XG_ERR_ARG, "lpc_create: null output");
  if (precision != 0 && precision != 1) return fail(c, XG_ERR_ARG, "lpc_create: precision 0 or 1");
  auto* m = new xg_lpc;
  m->own.device = c->device;
  if (cudaStreamCreateWithFlags(&m->own.stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete m;
    return fail(c, XG_ERR_CUDA, "lpc_create: stream creation failed");
  }
  m->precision = precision;
  for (int pass = 0; pass < 2; ++pass) {
    Arena& P = m->params;
    P.plan(m->theta, kNParams);
    P.plan(m->grad, kNParams);
    P.plan(m->m1, kNParams);
    P.plan(m->m2, kNParams);
    P.plan(m->frag, 4 * kFragWords);
    P.plan(m->lossv, 4);
    P.plan(m->wpart, int64_t(kWgradBlocks) * (2 * H * 2 * H + 2 * H));
    if (pass == 0 && P.reserve() != cudaSuccess) {
      xg_lpc_destroy(m);
      return fail(c, XG_ERR_CUDA, "lpc_create: device allocation failed");
    }
  }
  cudaStream_t s = m->own.stream;
  cudaError_t e = cudaMemsetAsync(m->theta, 0, kNParams * 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->grad, 0, kNParams * 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->m1, 0, kNParams * 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->m2, 0, kNParams * 4, s);
  if (e == cudaSuccess && refresh_frag(&m->own, m) != XG_OK) e = cudaErrorUnknown;
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    xg_lpc_destroy(m);
    return fail(c, XG_ERR_CUDA, "lpc_create: initialisation failed");
  }
  *out = m;
  return XG_OK;
}

int xg_lpc_destroy(xg_lpc* m) {
  if (!m) return XG_OK;
  cudaSetDevice(m->own.device);
  if (m->own.stream) {
    cudaStreamSynchronize(m->own.stream);
    cudaStreamDestroy(m->own.stream);
  }
  delete m;
  return XG_OK;
}

const char* xg_lpc_last_error(xg_lpc* m) { return m ? m->own.err.c_str() : "null model"; }

int xg_lpc_set_params(xg_lpc* m, const float* theta) {
  if (!m || !theta) return XG_ERR_ARG;
  xg_ctx* c = m->home;
  int rc = use(c);
  if (rc) return rc;
  XG_CUDA(c, cudaMemcpyAsync(m->theta, theta, kNParams * 4, cudaMemcpyHostToDevice, c->stream));
  XG_CUDA(c, cudaMemsetAsync(m->m1, 0, kNParams * 4, c->stream));
  XG_CUDA(c, cudaMemsetAsync(m->m2, 0, kNParams * 4, c->stream));
  m->step = 0;
  rc = refresh_frag(c, m);
  if (rc) return rc;
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}

int xg_lpc_get_params(xg_lpc* m, float* theta) {
  if (!m || !theta) return XG_ERR_ARG;
  xg_ctx* c = m->home;
  int rc = use(c);
  if (rc) return rc;
  XG_CUDA(c, cudaMemcpyAsync(theta, m->theta, kNParams * 4, cudaMemcpyDeviceToHost, c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}

int xg_lpc_zero_grads(xg_lpc* m) {
  if (!m) return XG_ERR_ARG;
  xg_ctx* c = m->home;
  int rc = use(c);
  if (rc) return rc;
  XG_CUDA(c, cudaMemsetAsync(m->grad, 0, kNParams * 4, c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}

int xg_lpc_get_grads(xg_lpc* m, float* grad) {
  if (!m || !grad) return XG_ERR_ARG;
  xg_ctx* c = m->home;
  int rc = use(c);
  if (rc) return rc;
  XG_CUDA(c, cudaMemcpyAsync(grad, m->grad, kNParams * 4, cudaMemcpyDeviceToHost, c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}

int xg_lpc_grad(xg_lpc* m, xg_ctx* c, double* loss) {
  int rc = use(c);
  if (rc) return rc;
  if (!m) return fail(c, XG_ERR_ARG, "lpc_grad: null model");
  if (m->own.device != c->device)
    return fail(c, XG_ERR_ARG, "lpc_grad: model and system on different devices");
  LpcGraph g;
  rc = cg_graph(c, &g);
  if (rc) return rc;
  // the model's own stream work (parameter uploads) is complete: every model
  // call synchronises before it returns
  rc = ensure_work(c, m, g.n, g.nentL, g.nentU);
  if (rc) return rc;
  cudaStream_t s = c->stream;
  const int64_t n = g.n;
  const unsigned nb = blocks_for(n, kThreads);
  const unsigned nrb = blocks_for(n, kRowsPerBlock);
  const EdgeParams P = edge_params(m->theta);
  rc = forward_nodes(c, m, g);
  if (rc) return rc;
  rc = edge_feature(c, m, g);
  if (rc) return rc;
  k_edge_fwd<true><<<nrb, kThreads, 0, s>>>(n, g.soffL, g.swL, g.colL, g.eL, g.tposU, m->tU,
                                            m->A, m->B, P, m->nL, m->nU, m->tL);
  XG_CHECK_LAUNCH(c);
  // trace loss and d loss / d N
  k_cross<true><<<nb, kThreads, 0, s>>>(n, g.soff, g.sw, g.col, g.eF, g.soffU, g.swU, g.colU,
                                        g.eU, m->nU, m->dnU, m->dpart);
  k_sum_parts<<<1, kThreads, 0, s>>>(m->dpart, nb, m->lossv, 0);
  XG_CHECK_LAUNCH(c);
  // edge backward
  k_edge_bwd_lower<<<nrb, kThreads, 0, s>>>(n, g.soffL, g.swL, g.colL, g.eL, g.tposU, m->tU,
                                            m->tL, m->A, m->B, P, m->dnU, m->da, m->doU,
                                            m->epart);
  k_reduce_parts<<<1, 512, 0, s>>>(m->epart, int(nrb), kEdgeParts, kEdgeParts, oc, 0, m->grad);
  k_edge_bwd_upper<<<nrb, kThreads, 0, s>>>(n, g.soffU, g.swU, g.colU, g.eU, m->tU, m->doU, m->A,
                                            m->B, P, m->db);
  XG_CHECK_LAUNCH(c);
  // output layer: dWo = h3^T [da | db]; du3 = ([da | db] Wo^T) o [h3 > 0]
  const unsigned ngemm = static_cast<unsigned>(std::min<int64_t>(blocks_for(n, 32), 4 * 148));
  rc = wgrad<H, 0, 2 * H, false>(c, m, n, m->h[3], nullptr, m->da, m->db, oWo, 0);
  if (rc) return rc;
  k_dense_f32<2 * H, H, true><<<ngemm, kThreads, 0, s>>>(n, m->da, m->db, m->theta + oWo, nullptr,
                                                         0, m->h[3], m->du, nullptr);
  XG_CHECK_LAUNCH(c);
  float* du = m->du;
  float* dnext = m->du2;
  for (int l = 3; l >= 1; --l) {
    rc = wgrad<H, H, H, true>(c, m, n, m->h[l - 1], m->mh[l], du, nullptr, kLayerW[l - 1],
                              kLayerB[l - 1]);
    if (rc) return rc;
    // [dih | dim] = du W_l^T
    k_dense_f32<H, 2 * H, true><<<ngemm, kThreads, 0, s>>>(n, du, nullptr,
                                                           m->theta + kLayerW[l - 1], nullptr, 0,
                                                           nullptr, m->dih, m->dim);
    // du_{l-1} = (dih + E dim) o [h_{l-1} > 0]   (E symmetric)
    k_spmm<<<nrb, kThreads, 0, s>>>(n, g.soff, g.sw, g.col, g.eF, m->dim, m->dih, m->h[l - 1],
                                    dnext);
    XG_CHECK_LAUNCH(c);
    std::swap(du, dnext);
  }
  rc = wgrad<4, 0, H, true>(c, m, n, m->x4, nullptr, du, nullptr, oW0, ob0);
  if (rc) return rc;
  double lv = 0.0;
  XG_CUDA(c, cudaMemcpyAsync(&lv, m->lossv, sizeof(lv), cudaMemcpyDeviceToHost, s));
  XG_CUDA(c, cudaStreamSynchronize(s));
  if (loss) *loss = lv / double(n);
  return XG_OK;
}

int xg_lpc_adam(xg_lpc* m, double lr, double beta1, double beta2, double eps) {
  if (!m) return XG_ERR_ARG;
  xg_ctx* c = m->home;
  int rc = use(c);
  if (rc) return rc;
  m->step += 1;
  const double c1 = 1.0 - std::pow(beta1, double(m->step));
  const double c2 = 1.0 - std::pow(beta2, double(m->step));
  k_adam<<<blocks_for(kNParams, 256), 256, 0, c->stream>>>(kNParams, m->theta, m->grad, m->m1,
                                                          m->m2, float(lr), float(beta1),
                                                          float(beta2), float(eps), float(c1),
                                                          float(c2));
  XG_CHECK_LAUNCH(c);
  rc = refresh_frag(c, m);
  if (rc) return rc;
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}

}  // extern "C"
