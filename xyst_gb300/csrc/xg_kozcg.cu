// KozCG element kernels (filled in below).
#include "xg_internal.hpp"

namespace xg {
struct KozCGDev {
  Arena arena;
};
void destroy_kozcg(KozCGDev* d) { delete d; }
size_t bytes_kozcg(const KozCGDev* d) { return d ? d->arena.bytes() : 0; }
}  // namespace xg
