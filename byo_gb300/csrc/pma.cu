// pma.cu -- packed-memory-array container (placeholder until the device PMA
// lands; every entry point reports BYO_ENOTSUP).
#include "internal.h"

namespace byo {
struct Pma {};
int pma_build(byo_graph *g, const uint64_t *, uint64_t) {
  return set_error(g->ctx, BYO_ENOTSUP, "pma container not available");
}
int pma_update(byo_graph *g, const uint64_t *, uint64_t, int, int, uint64_t *) {
  return set_error(g->ctx, BYO_ENOTSUP, "pma container not available");
}
int pma_export_keys(byo_graph *g, uint64_t *) {
  return set_error(g->ctx, BYO_ENOTSUP, "pma container not available");
}
void pma_destroy(Pma *p) { delete p; }
}  // namespace byo
