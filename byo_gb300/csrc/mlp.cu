// mlp.cu -- learned direction policy (placeholder: no trained network yet,
// callers fall back to the GBBS m/20 rule).
#include "internal.h"

namespace byo {
struct Mlp {};
int policy_choose(byo_ctx *ctx, const float *, int, int *) {
  return set_error(ctx, BYO_ENOTSUP, "no trained policy");
}
}  // namespace byo
