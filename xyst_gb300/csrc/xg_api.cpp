// Context lifetime and error reporting of the libxg C ABI.

#include <new>

#include "xg_internal.hpp"

extern "C" {

int xg_create(int device, xg_ctx** out) {
  if (!out) return XG_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess) return XG_ERR_CUDA;
  if (device < 0 || device >= ndev) return XG_ERR_ARG;
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return XG_ERR_CUDA;
  auto* c = new (std::nothrow) xg_ctx;
  if (!c) return XG_ERR_ARG;
  c->device = device;
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return XG_ERR_CUDA;
  }
  *out = c;
  return XG_OK;
}

int xg_destroy(xg_ctx* c) {
  if (!c) return XG_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  xg::destroy_riecg(c->riecg);
  xg::destroy_cg(c->cg);
  xg::destroy_kozcg(c->kozcg);
  xg::destroy_chocg(c->chocg);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return XG_OK;
}

const char* xg_last_error(const xg_ctx* c) { return c ? c->err.c_str() : "null context"; }

int xg_device_bytes(const xg_ctx* c, int64_t* bytes) {
  if (!c || !bytes) return XG_ERR_ARG;
  *bytes = static_cast<int64_t>(xg::bytes_riecg(c->riecg) + xg::bytes_cg(c->cg) +
                                xg::bytes_kozcg(c->kozcg) + xg::bytes_chocg(c->chocg));
  return XG_OK;
}

}  // extern "C"
