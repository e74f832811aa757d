// tl_solvers.cu -- the Chebyshev, PPCG and Jacobi solver plugins.
#include "tl_solvers.h"

int tl_record_solver_body(tl_ctx *ctx, int which, cudaGraphConditionalHandle h) {
  (void)h;
  tl_set_error(ctx, "no loop body %d", which);
  return TL_ERR_ARG;
}

int tl_cheby_solve(tl_ctx *ctx, double, double, const tl_params *, tl_result *) {
  tl_set_error(ctx, "Chebyshev solver not built yet");
  return TL_ERR_ARG;
}
int tl_ppcg_solve(tl_ctx *ctx, double, double, const tl_params *, tl_result *) {
  tl_set_error(ctx, "PPCG solver not built yet");
  return TL_ERR_ARG;
}
int tl_jacobi_solve(tl_ctx *ctx, double, double, const tl_params *, tl_result *) {
  tl_set_error(ctx, "Jacobi solver not built yet");
  return TL_ERR_ARG;
}
