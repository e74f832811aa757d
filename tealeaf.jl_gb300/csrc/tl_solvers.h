// tl_solvers.h -- host-side context of the library (not part of the C ABI).
#pragma once

#include "tl_internal.cuh"

// Cached iteration-loop graphs.
enum {
  TL_GRAPH_CG_REF = 0,       // reference-mode CG step + halo of u, p
  TL_GRAPH_CG_REF_NOHALO,    // reference-mode CG step without the halo (Cheby/PPCG presteps)
  TL_GRAPH_CG_EXACT,         // tealeaf fused CG, reference operation order
  TL_GRAPH_CG_FAST,          // tealeaf fused CG, FMA
  TL_GRAPH_CHEBY_EXACT,      // Chebyshev steps, the first of the pair reading ub
  TL_GRAPH_CHEBY_FAST,
  TL_GRAPH_PPCG_EXACT,       // two PPCG outer steps with their inner sweeps
  TL_GRAPH_PPCG_FAST,
  TL_GRAPH_JACOBI,           // two Jacobi sweeps with their every-50th residual checks
  TL_GRAPH_JACOBI_FAST,      // the same with the fused sweep
  TL_NGRAPH
};

struct tl_ir_state;    // FP32 refinement buffers (tl_ir.cu)
struct tl_warm_state;  // warm-start network and its buffers (tl_warm.cu)

struct tl_ctx {
  tl_config cfg{};
  tl::Geom g{};
  int lead = 0;
  long long field_stride = 0;
  int device = 0, sm_count = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  tl::Walk walk_exact{};            // fixed layout of the bit-reproducible kernels
  tl::Walk walk_w64{}, walk_ur64{};  // autotuned layouts of the fused FP64 CG kernels
  int max_blocks = 0;                // capacity of the reduction partials
  int host_loop = 0;                 // iteration loops launched from the host (TEALEAF_GB300_LOOP=host)
  double *buf = nullptr;
  void *small = nullptr;
  size_t buf_bytes = 0, small_bytes = 0;
  tl::Fields F{};
  double *field_ptr[TL_NFIELDS] = {};
  tl::DevScalars *host_sc = nullptr;
  int toexchange[TL_NEX] = {};
  int initialised = 0;
  double last_solve_ms = 0.0;
  long long launches = 0;     // kernels launched by the current solve
  cudaEvent_t tev0 = nullptr, tev1 = nullptr;  // user timer
  cudaGraphExec_t graph[TL_NGRAPH] = {};
  int ppcg_graph_inner = -1;  // inner sweeps recorded in the PPCG graphs
  tl_ir_state *ir = nullptr;
  tl_warm_state *warm = nullptr;  // learned warm start (tl_warm.cu)
  char msg[512] = {};
};

void tl_set_error(tl_ctx *ctx, const char *fmt, ...);
int tl_cuda_fail(tl_ctx *ctx, cudaError_t e, const char *what, int line);
double *tl_exchange_ptr(tl_ctx *ctx, int ex);
int tl_marked(tl_ctx *ctx, double **ptrs);
int tl_halo_check(tl_ctx *ctx, int depth);
tl::Walk tl_walk_balanced(int nx, int ny, int cols_per_warp, int warps, int blocks);
// Times candidate walks of one kernel (`launch` runs it once with a walk) and
// returns the fastest; occ4/occ8 are the kernel's resident blocks per SM at 4
// and 8 warps per block.
tl::Walk tl_autotune(tl_ctx *ctx, int cols_per_warp, int occ4, int occ8, void (*launch)(tl_ctx *, const tl::Walk &));
int tl_occupancy_cg(int kernel, int threads);  // 0: fused W, 1: fused UR (FP64)
void tl_launch_w64_for_tuning(tl_ctx *ctx, const tl::Walk &wk);
void tl_launch_ur64_for_tuning(tl_ctx *ctx, const tl::Walk &wk);
void tl_release_graphs(tl_ctx *ctx);
void tl_release_ir(tl_ctx *ctx);
void tl_release_ir_graphs(tl_ctx *ctx);

// shared solver pieces (tl_solve.cu)
int tl_set_loop_params(tl_ctx *ctx, const tl_params *prm, int switch_rule, int stale_rro);
int tl_read_scalars(tl_ctx *ctx);
const tl::Walk &tl_walk_for(tl_ctx *ctx, int exact);
int tl_cg_init(tl_ctx *ctx, double rx, double ry, int coefficient, int exact);
int tl_get_graph(tl_ctx *ctx, int which, cudaGraphExec_t *out);
int tl_run_graph(tl_ctx *ctx, int which, double *ms);
int tl_cg_solve(tl_ctx *ctx, double rx, double ry, const tl_params *prm, tl_result *res);

// the other solver plugins (tl_solvers.cu) and the FP32 refinement (tl_ir.cu)
int tl_record_solver_body(tl_ctx *ctx, int which, cudaGraphConditionalHandle h);
int tl_cheby_solve(tl_ctx *ctx, double rx, double ry, const tl_params *prm, tl_result *res);
int tl_ppcg_solve(tl_ctx *ctx, double rx, double ry, const tl_params *prm, tl_result *res);
int tl_jacobi_solve(tl_ctx *ctx, double rx, double ry, const tl_params *prm, tl_result *res);
int tl_ir_solve(tl_ctx *ctx, double rx, double ry, const tl_params *prm, tl_result *res);
int tl_ensure_ir(tl_ctx *ctx, int tune = 1);  // allocates and tunes the FP32 refinement buffers
// Chebyshev after its first step, in FP32 inside FP64 refinement (tl_ir.cu)
int tl_cheby32_run(tl_ctx *ctx, const tl_params *prm, int *refinements, double *rel_out);
int tl_ir_presteps(tl_ctx *ctx, double rx, double ry, const tl_params *prm, int *refinements, double *rr_out,
                   double *rel_out, int *switched);
int tl_ppcg32_run(tl_ctx *ctx, const tl_params *prm, double rr, int *refinements, double *rel_out);
int tl_ir_bench_kernel(tl_ctx *ctx, int kernel, int reps, double *ms_per_launch);
tl::Walk *tl_ir_walk(tl_ctx *ctx, int kernel);  // the FP32 kernels' layouts (kernel 2, 3)

// warm start (tl_warm.cu): after init + copyu!, maybe replace the plain start
// by the projected prediction; always records u^n for the next step.
int tl_warm_try(tl_ctx *ctx, double rx, double ry, int warmstart, tl_result *res);
void tl_release_warm(tl_ctx *ctx);

#define CK(x)                                                     \
  do {                                                            \
    cudaError_t e_ = (x);                                         \
    if (e_ != cudaSuccess) return tl_cuda_fail(ctx, e_, #x, __LINE__); \
  } while (0)
#define CKL() CK(cudaGetLastError())
