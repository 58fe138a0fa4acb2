// sg_kernels_mixed.cu - MIXED-mode kernels (placeholder until the mixed path lands).
#include "sg_engine.h"

int sg_mixed_init(sg_ctx *) { return sg_fail(SG_ERR_UNSUPPORTED, "MIXED mode is not built yet"); }
void sg_mixed_free(sg_ctx *) {}
int sg_mixed_enqueue_integrate(sg_ctx *, int) { return SG_ERR_UNSUPPORTED; }
int sg_mixed_enqueue_forces(sg_ctx *) { return SG_ERR_UNSUPPORTED; }
int sg_mixed_enqueue_reduce(sg_ctx *, int) { return SG_ERR_UNSUPPORTED; }
