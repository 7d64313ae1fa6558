// Allocation-free CFL time step for callers that cannot allocate device
// memory.
//
// Some callers own every byte of device memory through their own pool (for
// example a runtime that reserves the GPU's memory at start-up and hands out
// pieces of it), or run in a place where a cudaMalloc is not allowed.  They
// already hold the RieCG state and nodal volumes on the device and only need
// the CFL time step of RieCG::dt.  xg_riecg_dt_noalloc computes it with the
// same per-node formula as xg_riecg_dt, but its block minima live in a
// file-scope __device__ array instead of a context's allocation, so the call
// allocates nothing.
//
// The array holds kNoallocMaxBlocks block minima plus one result slot
// (512 KiB + 256 B); every GPU that loads the library holds it until the
// process exits.  It bounds npoin to kNoallocMaxBlocks * 256 nodes.  All calls
// on a device share it and it keeps the last call's contents: every call
// overwrites exactly the slots it reads, so nothing needs clearing between
// calls, but calls that overlap on the GPU (e.g. issued on different streams
// without ordering) race on it.

#include <cfloat>
#include <cmath>
#include <cstring>
#include <mutex>

#include "xg_internal.hpp"

namespace {

constexpr int kNoallocBlock = 256;
constexpr int64_t kNoallocMaxBlocks = 65536;
constexpr int kNoallocMaxDevices = 64;

// [0, kNoallocMaxBlocks): block minima (bits of positive doubles);
// [kNoallocMaxBlocks]: the reduced minimum.
static __device__ __align__(256) unsigned long long g_dt_scratch[kNoallocMaxBlocks + 32];

unsigned long long* g_scratch_ptr[kNoallocMaxDevices] = {};
std::once_flag g_scratch_once[kNoallocMaxDevices];
cudaError_t g_scratch_err[kNoallocMaxDevices] = {};

__device__ __forceinline__ double node_dt(const double u[5], double vol, double g) {
  double r = u[0];
  double uu = u[1] / r, vv = u[2] / r, ww = u[3] / r;
  double pr = (u[4] - 0.5 * r * (uu * uu + vv * vv + ww * ww)) * (g - 1.0);
  double c = sqrt(g * fmax(pr, 0.0) / r);
  double L = cbrt(vol);
  double vel = sqrt(uu * uu + vv * vv + ww * ww);
  return L / fmax(vel + c, 1.0e-8);
}

__device__ __forceinline__ unsigned long long warp_min(unsigned long long b) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long other = __shfl_xor_sync(0xffffffffu, b, o);
    b = other < b ? other : b;
  }
  return b;
}

// Per-block minimum of the per-node CFL dt of node-major U (npoin x 5).
__global__ void __launch_bounds__(kNoallocBlock) k_dt_blocks(int64_t n,
                                                              const double* __restrict__ U,
                                                              const double* __restrict__ vol,
                                                              double gamma,
                                                              unsigned long long* scratch) {
  __shared__ unsigned long long red[kNoallocBlock / 32];
  int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  double dtp = DBL_MAX;
  if (p < n) {
    double u[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) u[c] = U[p * 5 + c];
    dtp = node_dt(u, vol[p], gamma);
  }
  unsigned long long b = warp_min(__double_as_longlong(dtp));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = b;
  __syncthreads();
  if (threadIdx.x < 32) {
    unsigned long long x =
        threadIdx.x < kNoallocBlock / 32 ? red[threadIdx.x] : __double_as_longlong(DBL_MAX);
    x = warp_min(x);
    if (threadIdx.x == 0) scratch[blockIdx.x] = x;
  }
}

// One block: minimum of the nblk block minima into scratch[kNoallocMaxBlocks].
__global__ void __launch_bounds__(kNoallocBlock) k_dt_final(int64_t nblk,
                                                             unsigned long long* scratch) {
  __shared__ unsigned long long red[kNoallocBlock / 32];
  unsigned long long b = __double_as_longlong(DBL_MAX);
  for (int64_t i = threadIdx.x; i < nblk; i += blockDim.x) {
    unsigned long long v = scratch[i];
    b = v < b ? v : b;
  }
  b = warp_min(b);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = b;
  __syncthreads();
  if (threadIdx.x < 32) {
    unsigned long long x =
        threadIdx.x < kNoallocBlock / 32 ? red[threadIdx.x] : __double_as_longlong(DBL_MAX);
    x = warp_min(x);
    if (threadIdx.x == 0) scratch[kNoallocMaxBlocks] = x;
  }
}

}  // namespace

extern "C" {

// See include/xg.h.
int xg_riecg_dt_noalloc(const double* U, const double* vol, int64_t npoin, double gamma,
                        double cfl, double const_dt, void* stream, double* dt) {
  if (!dt) return XG_ERR_ARG;
  if (std::fabs(const_dt) > DBL_EPSILON) {
    *dt = const_dt;
    return XG_OK;
  }
  if (!U || !vol || npoin <= 0) return XG_ERR_ARG;
  const int64_t nblk = (npoin + kNoallocBlock - 1) / kNoallocBlock;
  if (nblk > kNoallocMaxBlocks) return XG_ERR_ARG;  // npoin > 16,777,216
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return XG_ERR_CUDA;
  if (dev < 0 || dev >= kNoallocMaxDevices) return XG_ERR_ARG;
  // Once per device, with that device current: the device address of the
  // scratch array (the host-side name is only a stand-in for it).
  std::call_once(g_scratch_once[dev], [dev]() {
    void* ptr = nullptr;
    g_scratch_err[dev] = cudaGetSymbolAddress(&ptr, g_dt_scratch);
    if (g_scratch_err[dev] == cudaSuccess) g_scratch_ptr[dev] = static_cast<unsigned long long*>(ptr);
  });
  if (g_scratch_err[dev] != cudaSuccess || !g_scratch_ptr[dev]) return XG_ERR_CUDA;
  unsigned long long* scratch = g_scratch_ptr[dev];
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_dt_blocks<<<static_cast<unsigned>(nblk), kNoallocBlock, 0, s>>>(npoin, U, vol, gamma, scratch);
  if (cudaGetLastError() != cudaSuccess) return XG_ERR_CUDA;
  k_dt_final<<<1, kNoallocBlock, 0, s>>>(nblk, scratch);
  if (cudaGetLastError() != cudaSuccess) return XG_ERR_CUDA;
  unsigned long long bits = 0;
  if (cudaMemcpyAsync(&bits, scratch + kNoallocMaxBlocks, sizeof(bits), cudaMemcpyDeviceToHost,
                      s) != cudaSuccess)
    return XG_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return XG_ERR_CUDA;
  double m;
  static_assert(sizeof(m) == sizeof(bits), "64-bit double expected");
  std::memcpy(&m, &bits, sizeof(m));
  *dt = m * cfl;
  return XG_OK;
}

}  // extern "C"
