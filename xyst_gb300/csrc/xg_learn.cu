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
// The dense layers -- forward, the backward data products dY W^T and the
// weight gradients X^T dY -- run as BF16 GEMMs with FP32 accumulation on the
// 5th-generation tensor cores (tcgen05.mma, accumulators in TMEM; precision
// 1), or in FP32 on the CUDA cores (precision 0, the reference the tensor-core
// path is tested against).  Every reduction over nodes or edges goes
// through fixed-order block partials, so a gradient is bit-reproducible.
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


// ---------------------------------------------------------------- helpers

__device__ __forceinline__ float relu(float v) { return v > 0.f ? v : 0.f; }

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
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

// ---------------------------------------------------------------- tcgen05 (5th-gen tensor cores)
//
// BF16 GEMMs on sm_103a tensor cores: operands in shared memory, the FP32
// accumulator in tensor memory (TMEM).  One thread of the CTA issues
// tcgen05.mma; its completion arrives on an mbarrier (tcgen05.commit); the
// epilogue reads the accumulator back with tcgen05.ld.  Operand layout: the
// canonical K-major layout without swizzle -- 8 x 8 BF16 "core matrices"
// (8 rows of 16 contiguous bytes, 128 bytes each), adjacent core matrices
// along K kLbo bytes apart and along M (or N) sbo = K * 16 bytes apart.
// The element (row r, k) of an R x K operand therefore sits at byte
//   (r / 8) * (K * 16) + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2.
// Every wait on the mbarrier is bounded: after kUmmaSpin polls the CTA
// records an error status, frees its TMEM and returns.

constexpr int kUmmaThreads = 128;  // one thread per accumulator row (TMEM lane)
constexpr int kUmmaM = 128;        // rows per MMA tile
constexpr uint32_t kLbo = 128;     // bytes between core matrices along K
constexpr int kUmmaSpin = 1 << 20;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (r, k) in an R x K K-major core-matrix operand
__device__ __forceinline__ uint32_t umma_off(int r, int k, int K) {
  return uint32_t((r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor (no swizzle): start address, LBO and SBO
// in 16-byte units, descriptor version 1.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= uint64_t((saddr >> 4) & 0x3FFF);
  d |= uint64_t((lbo >> 4) & 0x3FFF) << 16;
  d |= uint64_t((sbo >> 4) & 0x3FFF) << 32;
  d |= uint64_t(1) << 46;  // version
  return d;                // base offset 0, layout type 0 (no swizzle)
}

// Instruction descriptor of kind::f16: BF16 A and B (K-major), FP32 D, M x N.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N) {
  return (1u << 4)       // D format FP32
         | (1u << 7)     // A format BF16
         | (1u << 10)    // B format BF16
         | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint64_t* mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(mbar))
      : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Bounded wait for the mbarrier phase with the given parity; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity) {
  const uint32_t a = smem_u32(mbar);
  for (int it = 0; it < kUmmaSpin; ++it) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy shared-memory writes made visible to the tensor cores
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 32 consecutive FP32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float v[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint16_t bf16_bits(float f) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(f));
}

// Y = act([X1 | X2] Bt^T + bias) (o [maskY > 0]) on the tensor cores, for
// rows 0..n-1: X1, X2 n x 64 FP32 (X2 null: KIN = 64); Bt NOUT x KIN
// (FROM_W: built from a KIN x NOUT row-major weight W, Bt[o][k] = W[k][o] --
// the forward layer; otherwise Bt = W, NOUT x KIN row-major -- dX = dY W^T
// of the backward pass); Y split into Y1 (columns 0..63) and Y2 (64..127).
// Operands are rounded to BF16, products accumulated in FP32.  Each CTA
// takes 128-row tiles in turn; one TMEM accumulator of NOUT columns.
template <int KIN, int NOUT, bool FROM_W>
__global__ void __launch_bounds__(kUmmaThreads, 1)
    k_dense_umma(int64_t n, const float* __restrict__ X1, const float* __restrict__ X2,
                 const float* __restrict__ W, const float* __restrict__ bias, int act,
                 const float* __restrict__ maskY, float* __restrict__ Y1, float* __restrict__ Y2,
                 int32_t* __restrict__ err) {
  static_assert(KIN % 16 == 0 && NOUT % 32 == 0 && NOUT >= 32 && NOUT <= 256, "UMMA shape");
  extern __shared__ __align__(1024) uint8_t umma_smem[];
  uint8_t* sA = umma_smem;                     // kUmmaM x KIN BF16
  uint8_t* sB = umma_smem + kUmmaM * KIN * 2;  // NOUT x KIN BF16
  __shared__ uint64_t mbar;
  __shared__ uint32_t taddr_s;
  const int tid = threadIdx.x, warp = tid >> 5;
  // the weight operand, once per CTA
  for (int t = tid; t < NOUT * KIN; t += kUmmaThreads) {
    const int o = t / KIN, k = t % KIN;
    const float v = FROM_W ? W[k * NOUT + o] : W[o * KIN + k];
    *reinterpret_cast<uint16_t*>(sB + umma_off(o, k, KIN)) = bf16_bits(v);
  }
  if (tid == 0) mbar_init(&mbar, 1);
  if (warp == 0) tmem_alloc(&taddr_s, NOUT);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = taddr_s;
  constexpr uint32_t idesc = umma_idesc_bf16(kUmmaM, NOUT);
  const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
  const int64_t ntile = (n + kUmmaM - 1) / kUmmaM;
  uint32_t phase = 0;
  bool ok = true;
  for (int64_t tile = blockIdx.x; tile < ntile && ok; tile += gridDim.x) {
    // A tile: row tid of the tile, KIN values rounded to BF16, 16 bytes at a time
    const int64_t i = tile * kUmmaM + tid;
#pragma unroll
    for (int k0 = 0; k0 < KIN; k0 += 8) {
      const float* X = k0 < H ? X1 : X2;
      const int c = k0 % H;
      float v[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      if (i < n) {
        const float4 lo = __ldg(reinterpret_cast<const float4*>(X + i * H + c));
        const float4 hi = __ldg(reinterpret_cast<const float4*>(X + i * H + c + 4));
        v[0] = lo.x, v[1] = lo.y, v[2] = lo.z, v[3] = lo.w;
        v[4] = hi.x, v[5] = hi.y, v[6] = hi.z, v[7] = hi.w;
      }
      uint4 pk;
      pk.x = uint32_t(bf16_bits(v[0])) | (uint32_t(bf16_bits(v[1])) << 16);
      pk.y = uint32_t(bf16_bits(v[2])) | (uint32_t(bf16_bits(v[3])) << 16);
      pk.z = uint32_t(bf16_bits(v[4])) | (uint32_t(bf16_bits(v[5])) << 16);
      pk.w = uint32_t(bf16_bits(v[6])) | (uint32_t(bf16_bits(v[7])) << 16);
      *reinterpret_cast<uint4*>(sA + umma_off(tid, k0, KIN)) = pk;
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {
#pragma unroll
      for (int ks = 0; ks < KIN / 16; ++ks)
        umma_bf16(tmem, umma_desc(a0 + ks * 2 * kLbo, kLbo, KIN * 16),
                  umma_desc(b0 + ks * 2 * kLbo, kLbo, KIN * 16), idesc, ks > 0 ? 1u : 0u);
      umma_commit(&mbar);
    }
    ok = mbar_wait(&mbar, phase);
    phase ^= 1;
    ok = __syncthreads_and(ok) != 0;  // block-uniform before the warp-collective TMEM reads
    tc_fence_after();
    if (ok) {
      // accumulator row tid (TMEM lane 32 warp + lane): NOUT columns
#pragma unroll
      for (int c0 = 0; c0 < NOUT; c0 += 32) {
        float v[32];
        tmem_ld32(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0), v);
        if (i < n) {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int o = c0 + j;
            float y = v[j] + (bias ? bias[o] : 0.f);
            if (act) y = relu(y);
            if (maskY && !(maskY[i * NOUT + o] > 0.f)) y = 0.f;
            v[j] = y;
          }
          float* Y = c0 < H ? Y1 : Y2;
          float* dst = Y + i * H + (c0 % H);
#pragma unroll
          for (int j = 0; j < 32; j += 4)
            *reinterpret_cast<float4*>(dst + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
        }
      }
    }
    // every lane's reads of this accumulator and of the A tile are done
    // before the next tile's MMAs overwrite them
    tc_fence_before();
    ok = __syncthreads_and(ok) != 0;
    tc_fence_after();
  }
  if (!ok) {
    // a timed-out wait: give the MMAs in flight one more bounded wait before
    // the accumulator is freed
    mbar_wait(&mbar, phase ^ 1);
    if (tid == 0) atomicCAS(err, 0, 1);
  }
  __syncthreads();
  if (warp == 0) tmem_free(tmem, NOUT);
}

// Per-CTA partials of dW = X^T dY (KIN x NOUT, KIN = 64 or 128 from X1 | X2)
// on the tensor cores and, with BIAS, db = sum dY (FP32 on the CUDA cores):
// the CTA accumulates its 128-row tiles in TMEM (rows as the reduction
// dimension: the A operand is X^T -- KIN rows padded to 128, the rows of
// the tile along K -- and the B operand dY^T) and writes its partial to
// part[blockIdx.x] (KIN*NOUT weights, then NOUT biases), summed over CTAs
// in a fixed order afterwards.
template <int KIN, int NOUT, bool BIAS>
__global__ void __launch_bounds__(kUmmaThreads, 1)
    k_wgrad_umma(int64_t n, const float* __restrict__ X1, const float* __restrict__ X2,
                 const float* __restrict__ dY1, const float* __restrict__ dY2,
                 float* __restrict__ part, int32_t* __restrict__ err) {
  static_assert((KIN == 64 || KIN == 128) && NOUT % 32 == 0 && NOUT <= 256, "UMMA shape");
  constexpr int KR = kUmmaM;  // reduction rows per tile (the MMA's K)
  extern __shared__ __align__(1024) uint8_t umma_smem[];
  uint8_t* sA = umma_smem;                    // (X^T) 128 x 128 BF16, rows >= KIN zero
  uint8_t* sB = umma_smem + kUmmaM * KR * 2;  // (dY^T) NOUT x 128 BF16
  __shared__ uint64_t mbar;
  __shared__ uint32_t taddr_s;
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int t = tid; t < (kUmmaM - KIN) * KR; t += kUmmaThreads) {
    const int r = KIN + t / KR, k = t % KR;
    *reinterpret_cast<uint16_t*>(sA + umma_off(r, k, KR)) = 0;
  }
  if (tid == 0) mbar_init(&mbar, 1);
  if (warp == 0) tmem_alloc(&taddr_s, NOUT);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = taddr_s;
  constexpr uint32_t idesc = umma_idesc_bf16(kUmmaM, NOUT);
  const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
  const int64_t ntile = (n + KR - 1) / KR;
  uint32_t phase = 0, acc = 0;
  bool ok = true;
  float dbias = 0.f;  // thread tid < NOUT: column tid of dY summed over this CTA's rows
  for (int64_t tile = blockIdx.x; tile < ntile && ok; tile += gridDim.x) {
    // row tid of the tile: its KIN inputs as column tid of A, its NOUT
    // output gradients as column tid of B
    const int64_t i = tile * KR + tid;
    for (int k = 0; k < KIN; ++k) {
      const float v = i < n ? (k < H ? X1[i * H + k] : X2[i * H + (k - H)]) : 0.f;
      *reinterpret_cast<uint16_t*>(sA + umma_off(k, tid, KR)) = bf16_bits(v);
    }
    for (int o = 0; o < NOUT; ++o) {
      const float v = i < n ? (o < H ? dY1[i * H + o] : dY2[i * H + (o - H)]) : 0.f;
      *reinterpret_cast<uint16_t*>(sB + umma_off(o, tid, KR)) = bf16_bits(v);
    }
    if (BIAS && tid < NOUT) {
      for (int r = 0; r < KR; ++r) {
        const int64_t ir = tile * KR + r;
        if (ir < n) dbias += tid < H ? dY1[ir * H + tid] : dY2[ir * H + (tid - H)];
      }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {
#pragma unroll
      for (int ks = 0; ks < KR / 16; ++ks)
        umma_bf16(tmem, umma_desc(a0 + ks * 2 * kLbo, kLbo, KR * 16),
                  umma_desc(b0 + ks * 2 * kLbo, kLbo, KR * 16), idesc, (acc | ks) ? 1u : 0u);
      umma_commit(&mbar);
    }
    acc = 1;
    // the operand tiles are rewritten only after these MMAs have read them
    ok = mbar_wait(&mbar, phase);
    phase ^= 1;
    tc_fence_after();
    ok = __syncthreads_and(ok) != 0;
  }
  constexpr int NW = KIN * NOUT;
  float* out = part + int64_t(blockIdx.x) * (NW + (BIAS ? NOUT : 0));
  if (ok) {
    // accumulator row tid = input unit tid (< KIN), NOUT columns; a CTA with
    // no tile writes zeros
    if (tid < KIN) {  // warp-uniform: KIN is a multiple of 32
#pragma unroll
      for (int c0 = 0; c0 < NOUT; c0 += 32) {
        float v[32];
        tmem_ld32(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0), v);
#pragma unroll
        for (int j = 0; j < 32; ++j) out[tid * NOUT + c0 + j] = acc ? v[j] : 0.f;
      }
    }
    if (BIAS && tid < NOUT) out[NW + tid] = dbias;
  } else {
    // a timed-out wait: one more bounded wait for the MMAs in flight
    mbar_wait(&mbar, phase ^ 1);
    if (tid == 0) atomicCAS(err, 0, 1);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_free(tmem, NOUT);
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
  double* lossv = nullptr;   // [x^.b^, e.g]
  int32_t* uerr = nullptr;   // nonzero: a tensor-core GEMM's mbarrier wait timed out
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

// The tensor-core GEMMs: dense layer (forward or backward data) and weight
// gradient partials, on one CTA per SM at most (each holds up to 128 TMEM
// columns and 64 KB of operand tiles).
int umma_grid(int64_t n) {
  static int nsm = [] {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      v = 1;
    return v < 1 ? 1 : v;
  }();
  return static_cast<int>(std::max<int64_t>(1, std::min<int64_t>((n + kUmmaM - 1) / kUmmaM, nsm)));
}

template <int KIN, int NOUT, bool FROM_W>
int dense_umma(xg_ctx* c, xg_lpc* m, int64_t n, const float* X1, const float* X2, const float* W,
               const float* bias, int act, const float* maskY, float* Y1, float* Y2) {
  constexpr int smem = (kUmmaM * KIN + NOUT * KIN) * 2;
  static const cudaError_t attr = cudaFuncSetAttribute(
      k_dense_umma<KIN, NOUT, FROM_W>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  XG_CUDA(c, attr);
  k_dense_umma<KIN, NOUT, FROM_W><<<umma_grid(n), kUmmaThreads, smem, c->stream>>>(
      n, X1, X2, W, bias, act, maskY, Y1, Y2, m->uerr);
  XG_CHECK_LAUNCH(c);
  return XG_OK;
}

template <int KIN, int NOUT, bool BIAS>
int wgrad_umma(xg_ctx* c, xg_lpc* m, int64_t n, const float* X1, const float* X2,
               const float* dY1, const float* dY2, int64_t wofs, int64_t bofs) {
  constexpr int smem = (kUmmaM * kUmmaM + NOUT * kUmmaM) * 2;
  constexpr int NW = KIN * NOUT, NOUTP = NW + (BIAS ? NOUT : 0);
  static const cudaError_t attr = cudaFuncSetAttribute(
      k_wgrad_umma<KIN, NOUT, BIAS>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  XG_CUDA(c, attr);
  const int grid = umma_grid(n);
  k_wgrad_umma<KIN, NOUT, BIAS><<<grid, kUmmaThreads, smem, c->stream>>>(n, X1, X2, dY1, dY2,
                                                                          m->wpart, m->uerr);
  k_reduce_parts<<<(NOUTP + 255) / 256, 256, 0, c->stream>>>(m->wpart, grid, NOUTP, NW, wofs,
                                                             bofs, m->grad);
  XG_CHECK_LAUNCH(c);
  return XG_OK;
}

// The tensor-core GEMMs' error word (after a synchronise), reset when set.
int umma_status(xg_ctx* c, xg_lpc* m) {
  int32_t e = 0;
  XG_CUDA(c, cudaMemcpyAsync(&e, m->uerr, sizeof(e), cudaMemcpyDeviceToHost, c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (!e) return XG_OK;
  XG_CUDA(c, cudaMemsetAsync(m->uerr, 0, sizeof(e), c->stream));
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return fail(c, XG_ERR_DEVICE, "tensor-core GEMM: an mbarrier wait timed out");
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
    XG_CHECK_LAUNCH(c);
    int rc = XG_OK;
    if (m->precision == 1)
      rc = dense_umma<2 * H, H, true>(c, m, n, m->h[l - 1], m->mh[l], m->theta + kLayerW[l - 1],
                                      m->theta + kLayerB[l - 1], 1, nullptr, m->h[l], nullptr);
    else
      k_dense_f32<2 * H, H, false><<<ngemm, kThreads, 0, s>>>(
          n, m->h[l - 1], m->mh[l], m->theta + kLayerW[l - 1], m->theta + kLayerB[l - 1], 1,
          nullptr, m->h[l], nullptr);
    if (rc) return rc;
    XG_CHECK_LAUNCH(c);
  }
  if (m->precision == 1) {
    int rc = dense_umma<H, 2 * H, true>(c, m, n, m->h[3], nullptr, m->theta + oWo, nullptr, 0,
                                        nullptr, m->A, m->B);
    if (rc) return rc;
  } else {
    k_dense_f32<H, 2 * H, false><<<ngemm, kThreads, 0, s>>>(n, m->h[3], nullptr, m->theta + oWo,
                                                            nullptr, 0, nullptr, m->A, m->B);
  }
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
  return m->precision == 1 ? umma_status(c, m) : XG_OK;
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
    P.plan(m->lossv, 4);
    P.plan(m->uerr, 1);
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
  if (e == cudaSuccess) e = cudaMemsetAsync(m->uerr, 0, sizeof(int32_t), s);
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
  const bool tc = m->precision == 1;
  rc = tc ? wgrad_umma<H, 2 * H, false>(c, m, n, m->h[3], nullptr, m->da, m->db, oWo, 0)
          : wgrad<H, 0, 2 * H, false>(c, m, n, m->h[3], nullptr, m->da, m->db, oWo, 0);
  if (rc) return rc;
  if (tc) {
    rc = dense_umma<2 * H, H, false>(c, m, n, m->da, m->db, m->theta + oWo, nullptr, 0, m->h[3],
                                     m->du, nullptr);
    if (rc) return rc;
  } else {
    k_dense_f32<2 * H, H, true><<<ngemm, kThreads, 0, s>>>(n, m->da, m->db, m->theta + oWo,
                                                           nullptr, 0, m->h[3], m->du, nullptr);
  }
  XG_CHECK_LAUNCH(c);
  float* du = m->du;
  float* dnext = m->du2;
  for (int l = 3; l >= 1; --l) {
    rc = tc ? wgrad_umma<2 * H, H, true>(c, m, n, m->h[l - 1], m->mh[l], du, nullptr,
                                         kLayerW[l - 1], kLayerB[l - 1])
            : wgrad<H, H, H, true>(c, m, n, m->h[l - 1], m->mh[l], du, nullptr, kLayerW[l - 1],
                                   kLayerB[l - 1]);
    if (rc) return rc;
    // [dih | dim] = du W_l^T
    if (tc) {
      rc = dense_umma<H, 2 * H, false>(c, m, n, du, nullptr, m->theta + kLayerW[l - 1], nullptr,
                                       0, nullptr, m->dih, m->dim);
      if (rc) return rc;
    } else {
      k_dense_f32<H, 2 * H, true><<<ngemm, kThreads, 0, s>>>(n, du, nullptr,
                                                             m->theta + kLayerW[l - 1], nullptr,
                                                             0, nullptr, m->dih, m->dim);
    }
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
  if (tc) {
    rc = umma_status(c, m);
    if (rc) return rc;
  }
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
  XG_CUDA(c, cudaStreamSynchronize(c->stream));
  return XG_OK;
}

}  // extern "C"
