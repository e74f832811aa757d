// tl_ir.cu -- FP32 inner CG inside FP64 iterative refinement.
#include "tl_solvers.h"

void tl_release_ir(tl_ctx *ctx) { (void)ctx; }

int tl_ir_solve(tl_ctx *ctx, double, double, const tl_params *, tl_result *) {
  tl_set_error(ctx, "FP32 refinement not built yet");
  return TL_ERR_ARG;
}

int tl_ir_bench_kernel(tl_ctx *ctx, int, int, double *) {
  tl_set_error(ctx, "FP32 kernels not built yet");
  return TL_ERR_ARG;
}
