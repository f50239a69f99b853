// Batched fixpoints (search nodes, uneven instances).
#include "pir_engine.h"

namespace pirgpu {
struct BatchState {};
void destroy_batch_state(pirgpu_ctx *ctx) {
  delete ctx->batch;
  ctx->batch = nullptr;
}
}  // namespace pirgpu

extern "C" int pir_fixpoint_nodes(pirgpu_ctx *ctx, int32_t, const int32_t *, const int32_t *, const int32_t *,
                                  const int32_t *, const pir_opts *, int32_t *, int32_t *, int32_t *, int32_t *,
                                  pir_stats *) {
  return pirgpu::set_err(ctx, PIR_EINVAL, "pir_fixpoint_nodes: not built");
}

extern "C" int pir_fixpoint_instances(pirgpu_ctx *ctx, int32_t, const int64_t *, const int64_t *, const int32_t *,
                                      const int32_t *, const int32_t *, const int32_t *, int32_t *, int32_t *,
                                      const pir_opts *, int32_t *, int32_t *, float *, pir_stats *) {
  return pirgpu::set_err(ctx, PIR_EINVAL, "pir_fixpoint_instances: not built");
}
