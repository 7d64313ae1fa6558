// Internal definitions shared by the libxg translation units: the context,
// a device arena, error plumbing and the per-solver device state types.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <exception>
#include <new>
#include <string>
#include <vector>

#include "../../include/xg.h"

namespace xg {

// Bump allocator over one cudaMalloc block per solver: every device array of
// a solver lives in one allocation, 256-byte aligned, released together.
class Arena {
 public:
  Arena() = default;
  Arena(const Arena&) = delete;
  Arena& operator=(const Arena&) = delete;
  ~Arena() { release(); }

  // First pass: record sizes (ptr == nullptr); second pass after reserve().
  template <class T>
  void plan(T*& p, size_t count) {
    size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
    if (base_) {
      p = reinterpret_cast<T*>(base_ + off_);
      off_ += bytes;
    } else {
      p = nullptr;
      need_ += bytes;
    }
  }
  cudaError_t reserve() {
    if (need_ == 0) need_ = 256;
    cudaError_t e = cudaMalloc(&base_, need_);
    off_ = 0;
    return e;
  }
  void release() {
    if (base_) cudaFree(base_);
    base_ = nullptr;
    need_ = off_ = 0;
  }
  size_t bytes() const { return need_; }
  bool ready() const { return base_ != nullptr; }

 private:
  char* base_ = nullptr;
  size_t need_ = 0;
  size_t off_ = 0;
};

struct RieCGDev;  // xg_riecg.cu
struct CGDev;     // xg_cg.cu
struct KozCGDev;  // xg_kozcg.cu
struct ChoCGDev;  // xg_chocg.cu

// Matrix graph of a CG system as the learned preconditioner sees it: the full
// rows, the strictly lower and strictly upper triangles (SELL-32 each, slice
// offsets / widths / columns, PAD < 0), the normalised couplings
// e_ij = a_ij s_i s_j in each layout, the row scales s_i = 1/sqrt|a_ii|, the
// Dirichlet mask and tposU (upper-layout index of the transpose of each
// lower entry).
struct LpcGraph {
  int64_t n = 0, nslice = 0, nentL = 0, nentU = 0;
  const int32_t *soff = nullptr, *sw = nullptr, *col = nullptr;
  const int32_t *soffL = nullptr, *swL = nullptr, *colL = nullptr;
  const int32_t *soffU = nullptr, *swU = nullptr, *colU = nullptr;
  const int32_t* tposU = nullptr;
  const float *eF = nullptr, *eL = nullptr, *eU = nullptr, *srow = nullptr;
  const uint8_t* mask = nullptr;
};

// The context's CG system (xg_cg.cu), geometry computed on first use.
int cg_graph(xg_ctx* c, LpcGraph* g);

// Learned factor (xg_learn.cu): runs the network on g and writes the factor
// values N_ij in the lower layout (nvL) and, transposed, the upper one (nvU).
int lpc_factor(xg_ctx* c, xg_lpc* m, const LpcGraph& g, float* nvL, float* nvU);

// Device-side pressure solves for ChoCG on the context's CG system: the
// Dirichlet mask and the values of the first solves (host arrays, one per
// row), a zero initial guess, ConjugateGradients::init with apply and a
// device right-hand side (values zero when zero_values, the stored ones
// otherwise), the device solution and the row count.
int cg_set_dirichlet(xg_ctx* c, const uint8_t* mask, const double* val);
int cg_zero_solution(xg_ctx* c);
int cg_init_device(xg_ctx* c, const double* b_dev, int zero_values, int pc);
int cg_to_sell(xg_ctx* c, const uint64_t* ia, const double* csr, double* dev_out);
int64_t cg_nent(xg_ctx* c);
double* cg_values_device(xg_ctx* c);
const double* cg_solution_device(xg_ctx* c);
int64_t cg_rows(xg_ctx* c);

void destroy_riecg(RieCGDev*);
void destroy_cg(CGDev*);
void destroy_kozcg(KozCGDev*);
void destroy_chocg(ChoCGDev*);
size_t bytes_chocg(const ChoCGDev*);
size_t bytes_riecg(const RieCGDev*);
size_t bytes_cg(const CGDev*);
size_t bytes_kozcg(const KozCGDev*);

}  // namespace xg

struct xg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  xg::RieCGDev* riecg = nullptr;
  xg::CGDev* cg = nullptr;
  xg::KozCGDev* kozcg = nullptr;
  xg::ChoCGDev* chocg = nullptr;
};

namespace xg {

inline int fail(xg_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

#define XG_CUDA(ctx, call)                                                        \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess)                                                        \
      return ::xg::fail((ctx), XG_ERR_CUDA,                                       \
                        std::string(#call) + ": " + cudaGetErrorString(e_));      \
  } while (0)

#define XG_CHECK_LAUNCH(ctx) XG_CUDA(ctx, cudaGetLastError())

// Host-side set-up bodies run inside XG_HOST_TRY ... XG_HOST_CATCH(ctx): an
// exception (std::bad_alloc on a large mesh, std::system_error when threads
// are refused) becomes XG_ERR_HOST instead of crossing the C ABI.
#define XG_HOST_TRY try {
#define XG_HOST_CATCH(ctx)                                                         \
  }                                                                                \
  catch (const std::bad_alloc&) {                                                  \
    return ::xg::fail((ctx), XG_ERR_HOST, "out of host memory");                   \
  }                                                                                \
  catch (const std::exception& ex_) {                                              \
    return ::xg::fail((ctx), XG_ERR_HOST, std::string("host: ") + ex_.what());     \
  }                                                                                \
  catch (...) {                                                                    \
    return ::xg::fail((ctx), XG_ERR_HOST, "host-side exception");                  \
  }

// Grid size for n items at b threads per block, as a multiple of what one
// wave needs is left to the hardware scheduler: every node kernel is a flat
// one-thread-per-item launch.
inline unsigned blocks_for(int64_t n, int b) {
  return static_cast<unsigned>((n + b - 1) / b);
}

// Make the context's device current for the calling thread.
inline int use(xg_ctx* c) {
  if (!c) return XG_ERR_ARG;
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return fail(c, XG_ERR_CUDA, cudaGetErrorString(e));
  return XG_OK;
}

}  // namespace xg
