// CSR matrix and preconditioned conjugate gradients (filled in below).
#include "xg_internal.hpp"

namespace xg {
struct CGDev {
  Arena arena;
};
void destroy_cg(CGDev* d) { delete d; }
size_t bytes_cg(const CGDev* d) { return d ? d->arena.bytes() : 0; }
}  // namespace xg
