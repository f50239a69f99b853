// Learned propagator scheduler.
#include "pir_engine.h"

namespace pirgpu {
struct SchedState {};
void destroy_sched_state(pirgpu_ctx *ctx) {
  delete ctx->sched;
  ctx->sched = nullptr;
}
int fixpoint_learned(pirgpu_ctx *ctx, const pir_opts &, pir_stats *) {
  return set_err(ctx, PIR_EINVAL, "learned schedule: not built");
}
}  // namespace pirgpu
