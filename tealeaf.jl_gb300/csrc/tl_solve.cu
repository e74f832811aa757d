// tl_solve.cu -- solve!(chunk, set, rx, ry) for the CG plugin
// (src/solvers/CG.jl:7-29) and the shared pieces of the other solvers:
// tea_leaf_init, loop parameters, and the while-node iteration graphs.
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "tl_solvers.h"
#include "tl_walk.cuh"

using namespace tl;

namespace {

struct LoopParams {
  double eps, epslim;
  int maxiters, presteps, errorswitch, stale_rro, crit, switch_rule;
};

__global__ void k_set_params(DevScalars *sc, LoopParams p) {
  sc->eps = p.eps;
  sc->epslim = p.epslim;
  sc->maxiters = p.maxiters;
  sc->presteps = p.presteps;
  sc->errorswitch = p.errorswitch;
  sc->stale_rro = p.stale_rro;
  sc->crit = p.crit;
  sc->switch_rule = p.switch_rule;
}

}  // namespace

int tl_set_loop_params(tl_ctx *ctx, const tl_params *prm, int switch_rule, int stale_rro) {
  LoopParams p;
  p.eps = prm->eps;
  p.epslim = prm->epslim;
  p.maxiters = prm->maxiters;
  p.presteps = prm->presteps;
  p.errorswitch = prm->errorswitch;
  p.stale_rro = stale_rro;
  p.crit = prm->criterion;
  p.switch_rule = switch_rule;
  k_set_params<<<1, 1, 0, ctx->stream>>>(ctx->F.sc, p);
  CKL();
  return TL_OK;
}

int tl_read_scalars(tl_ctx *ctx) {
  CK(cudaMemcpyAsync(ctx->host_sc, ctx->F.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return TL_OK;
}

const Walk &tl_walk_for(tl_ctx *ctx, int exact) {
  return (ctx->cfg.mode == TL_MODE_REFERENCE || exact) ? ctx->walk_exact : ctx->walk_ur64;
}

// CG.init! (CG.jl:47-79).  Also stores the fused kernels' diagonal.
int tl_cg_init(tl_ctx *ctx, double rx, double ry, int coefficient, int exact) {
  if (coefficient != TL_CONDUCTIVITY && coefficient != TL_RECIP_CONDUCTIVITY) {
    tl_set_error(ctx, "Coefficient %d is not valid (src/solvers/CG.jl:49)", coefficient);
    return TL_ERR_COEF;
  }
  launch_init_pre(ctx->stream, ctx->F, ctx->g, coefficient, ctx->cfg.mode);
  CKL();
  launch_init_coef(ctx->stream, ctx->F, ctx->g, rx, ry, 0, coefficient);
  CKL();
  if (ctx->cfg.mode == TL_MODE_TEALEAF && !exact) {
    launch_init_diag(ctx->stream, ctx->F, ctx->g);
    CKL();
  }
  launch_init_resid(ctx->stream, ctx->F, ctx->g, ctx->walk_exact, ctx->cfg.mode);
  CKL();
  return TL_OK;
}

// ---------------------------------------------------------------------------
// iteration graphs
// ---------------------------------------------------------------------------

// Records the body of one while-node loop on the context stream.
static int record_body(tl_ctx *ctx, int which, cudaGraphConditionalHandle h) {
  const Fields &F = ctx->F;
  const Geom &g = ctx->g;
  cudaStream_t st = ctx->stream;
  switch (which) {
    case TL_GRAPH_CG_REF:
    case TL_GRAPH_CG_REF_NOHALO: {
      const Walk &wk = ctx->walk_exact;
      launch_ref_w(st, F, g, wk);
      launch_ref_ur(st, F, g, wk, h, 1);
      launch_ref_p(st, F, g, wk);
      if (which == TL_GRAPH_CG_REF) {
        double *ptrs[2] = {F.p, F.u};  // haloupdate!(chunk, set, 1) with u, p marked (CG.jl:23)
        launch_halo(st, ptrs, 2, g, 1, TL_MODE_REFERENCE);
      }
      break;
    }
    case TL_GRAPH_CG_EXACT:
    case TL_GRAPH_CG_FAST: {
      const int exact = which == TL_GRAPH_CG_EXACT;
      const Walk &ww = exact ? ctx->walk_exact : ctx->walk_w64;
      const Walk &wu = exact ? ctx->walk_exact : ctx->walk_ur64;
      launch_tl_w(st, F, g, ww, F.p, F.pb, exact, 0);
      launch_tl_ur(st, F, g, wu, F.pb, exact, 0, h, 0);
      launch_tl_w(st, F, g, ww, F.pb, F.p, exact, 1);
      launch_tl_ur(st, F, g, wu, F.p, exact, 1, h, 1);
      break;
    }
    default:
      return tl_record_solver_body(ctx, which, h);
  }
  return cudaGetLastError() == cudaSuccess ? TL_OK : TL_ERR_CUDA;
}

int tl_get_graph(tl_ctx *ctx, int which, cudaGraphExec_t *out) {
  if (ctx->graph[which]) {
    *out = ctx->graph[which];
    return TL_OK;
  }
  cudaGraph_t graph = nullptr;
  CK(cudaGraphCreate(&graph, 0));
  cudaGraphConditionalHandle h;
  cudaError_t e = cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    return tl_cuda_fail(ctx, e, "cudaGraphConditionalHandleCreate", __LINE__);
  }
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    return tl_cuda_fail(ctx, e, "cudaGraphAddNode(while)", __LINE__);
  }
  cudaGraph_t body = np.conditional.phGraph_out[0];
  e = cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    return tl_cuda_fail(ctx, e, "cudaStreamBeginCaptureToGraph", __LINE__);
  }
  int rc = record_body(ctx, which, h);
  cudaGraph_t captured = nullptr;
  e = cudaStreamEndCapture(ctx->stream, &captured);
  if (rc || e != cudaSuccess) {
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return tl_cuda_fail(ctx, e, "cudaStreamEndCapture", __LINE__);
    tl_set_error(ctx, "recording loop body %d failed: %s", which, cudaGetErrorString(cudaGetLastError()));
    return TL_ERR_CUDA;
  }
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return tl_cuda_fail(ctx, e, "cudaGraphInstantiate", __LINE__);
  ctx->graph[which] = exec;
  *out = exec;
  return TL_OK;
}

void tl_release_graphs(tl_ctx *ctx) {
  for (int k = 0; k < TL_NGRAPH; ++k)
    if (ctx->graph[k]) {
      cudaGraphExecDestroy(ctx->graph[k]);
      ctx->graph[k] = nullptr;
    }
}

// The same loop launched from the host: batches of eight two-iteration
// bodies whose kernels all skip once the device has set `done`, with the flag
// read back after each batch.  Profilers cannot see kernels inside graphs
// that hold conditional nodes; this mode (TEALEAF_GB300_LOOP=host) runs the
// identical kernels where they can.
static int run_host_loop_cg(tl_ctx *ctx, int exact) {
  const Fields &F = ctx->F;
  const Geom &g = ctx->g;
  const Walk &ww = exact ? ctx->walk_exact : ctx->walk_w64;
  const Walk &wu = exact ? ctx->walk_exact : ctx->walk_ur64;
  for (;;) {
    for (int b = 0; b < 8; ++b) {
      launch_tl_w(ctx->stream, F, g, ww, F.p, F.pb, exact, 1);
      launch_tl_ur(ctx->stream, F, g, wu, F.pb, exact, 1, 0, 0);
      launch_tl_w(ctx->stream, F, g, ww, F.pb, F.p, exact, 1);
      launch_tl_ur(ctx->stream, F, g, wu, F.p, exact, 1, 0, 0);
    }
    CKL();
    int rc = tl_read_scalars(ctx);
    if (rc) return rc;
    if (ctx->host_sc->done) return TL_OK;
  }
}

// Runs one loop graph, timing it with events on the context stream.
int tl_run_graph(tl_ctx *ctx, int which, double *ms) {
  const bool host = ctx->host_loop && (which == TL_GRAPH_CG_EXACT || which == TL_GRAPH_CG_FAST);
  cudaGraphExec_t exec = nullptr;
  if (!host) {
    int rc = tl_get_graph(ctx, which, &exec);
    if (rc) return rc;
  }
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  if (host) {
    int rc = run_host_loop_cg(ctx, which == TL_GRAPH_CG_EXACT);
    if (rc) return rc;
  } else {
    CK(cudaGraphLaunch(exec, ctx->stream));
  }
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaEventSynchronize(ctx->ev1));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1));
  if (ms) *ms += t;
  return TL_OK;
}

// ---------------------------------------------------------------------------
// walk layouts and the autotuner
// ---------------------------------------------------------------------------

// Rows per tile chosen so that the tiles spread evenly over `blocks`
// persistent blocks: minimise the rows the busiest block walks (one extra
// neighbour row re-read per tile), preferring longer tiles on ties.
Walk tl_walk_balanced(int nx, int ny, int cols_per_warp, int warps, int blocks) {
  Walk w;
  w.warps = warps;
  const int TW = cols_per_warp * warps;
  w.ntx = (nx + TW - 1) / TW;
  long long best_cost = -1;
  int best_rows = 1;
  const int rmax = ny < 1024 ? ny : 1024;
  for (int rows = 4 < ny ? 4 : ny; rows <= rmax; ++rows) {
    const long long nty = (ny + rows - 1) / rows, tiles = (long long)w.ntx * nty;
    const long long per = (tiles + blocks - 1) / blocks;
    const long long cost = per * (rows + 1);
    if (best_cost < 0 || cost < best_cost || (cost == best_cost && rows > best_rows)) {
      best_cost = cost;
      best_rows = rows;
    }
  }
  w.rows = best_rows;
  w.tiles = w.ntx * ((ny + best_rows - 1) / best_rows);
  w.blocks = w.tiles < blocks ? w.tiles : blocks;
  if (w.blocks < 1) w.blocks = 1;
  return w;
}

// A walk with fixed rows per tile: tiles in row-major order, so that the
// blocks running at one time sweep neighbouring tiles of the same rows.
static Walk walk_fixed(int nx, int ny, int cols_per_warp, int warps, int rows, int blocks) {
  Walk w;
  w.warps = warps;
  w.rows = rows;
  const int TW = cols_per_warp * warps;
  w.ntx = (nx + TW - 1) / TW;
  w.tiles = w.ntx * ((ny + rows - 1) / rows);
  w.blocks = w.tiles < blocks ? w.tiles : blocks;
  if (w.blocks < 1) w.blocks = 1;
  return w;
}

// Candidates: 4 or 8 warps per block; 2..8 resident blocks per SM (within the
// kernel's occupancy); tiles of 8, 16 or 32 rows, or the balanced length.
// Short tiles keep the blocks that run together inside the same DRAM rows;
// the balanced length gives one long tile per block.  Each candidate runs
// twice untimed and three times under CUDA events on the context stream.
Walk tl_autotune(tl_ctx *ctx, int cols_per_warp, int occ4, int occ8, void (*launch)(tl_ctx *, const tl::Walk &)) {
  const Geom &g = ctx->g;
  // without tuning (TEALEAF_GB300_TUNE=0): 8 warps, 8-row tiles, 3 blocks per SM
  Walk best = walk_fixed(g.nx, g.ny, cols_per_warp, 8, 8, 3 * ctx->sm_count);
  const char *tune = getenv("TEALEAF_GB300_TUNE");
  if (!launch || (tune && !strcmp(tune, "0"))) return best;  // no launcher: the fixed layout
  float best_ms = -1.f;
  for (int warps = 4; warps <= 8; warps += 4) {
    const int occ = warps == 4 ? occ4 : occ8;
    for (int bps = 2; bps <= occ && bps <= 8; ++bps) {
      const int B = bps * ctx->sm_count;
      if (B > ctx->max_blocks) break;
      const Walk cands[4] = {walk_fixed(g.nx, g.ny, cols_per_warp, warps, 8, B),
                             walk_fixed(g.nx, g.ny, cols_per_warp, warps, 16, B),
                             walk_fixed(g.nx, g.ny, cols_per_warp, warps, 32, B),
                             tl_walk_balanced(g.nx, g.ny, cols_per_warp, warps, B)};
      bool grid_full = false;
      for (const Walk &w : cands) {
        if (w.blocks < B) grid_full = true;  // fewer tiles than blocks: more blocks per SM cannot help
        launch(ctx, w);
        launch(ctx, w);
        if (cudaEventRecord(ctx->tev0, ctx->stream) != cudaSuccess) return best;
        for (int k = 0; k < 3; ++k) launch(ctx, w);
        if (cudaEventRecord(ctx->tev1, ctx->stream) != cudaSuccess) return best;
        if (cudaEventSynchronize(ctx->tev1) != cudaSuccess) return best;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->tev0, ctx->tev1);
        if (best_ms < 0.f || ms < best_ms) {
          best_ms = ms;
          best = w;
        }
      }
      if (grid_full) break;
    }
  }
  cudaGetLastError();
  return best;
}

void tl_launch_w64_for_tuning(tl_ctx *ctx, const Walk &wk) {
  launch_tl_w(ctx->stream, ctx->F, ctx->g, wk, ctx->F.p, ctx->F.pb, 0, 0);
}

void tl_launch_ur64_for_tuning(tl_ctx *ctx, const Walk &wk) {
  launch_tl_ur(ctx->stream, ctx->F, ctx->g, wk, ctx->F.pb, 0, 0, 0, 0);
}

// ---------------------------------------------------------------------------
// CG solve!
// ---------------------------------------------------------------------------

// Relative criterion: the loop stops on sqrt(rr / u0.u0) < eps for the
// recursive residual; the true residual u0 - A u is then measured and, if it
// has drifted above eps, CG restarts from it (r = p = u0 - A u) within the
// remaining iteration budget.
static int true_residual(tl_ctx *ctx, int write, double *rr) {
  launch_true_resid(ctx->stream, ctx->F, ctx->g, ctx->walk_exact, ctx->cfg.mode, write);
  ctx->launches += 1;
  CKL();
  int rc = tl_read_scalars(ctx);
  if (rc) return rc;
  *rr = ctx->host_sc->red[0];
  return TL_OK;
}

int tl_cg_solve(tl_ctx *ctx, double rx, double ry, const tl_params *prm, tl_result *res) {
  const int ref = ctx->cfg.mode == TL_MODE_REFERENCE;
  const int exact = ref || prm->exact;
  int rc = tl_cg_init(ctx, rx, ry, prm->coefficient, exact);
  if (rc) return rc;
  ctx->launches += exact ? 3 : 4;
  if ((rc = tl_set_loop_params(ctx, prm, 0, 0))) return rc;
  const int up[2] = {TL_EX_U, TL_EX_P};
  if ((rc = tl_halo_update(ctx, 1, up, 2, 1))) return rc;   // CG.jl:11
  if ((rc = tl_copy_u(ctx))) return rc;                     // CG.jl:12
  ctx->launches += 3;
  if (prm->warmstart && (rc = tl_warm_try(ctx, rx, ry, prm->warmstart, res))) return rc;
  ctx->last_solve_ms = 0.0;
  if (prm->criterion == TL_CRIT_RELATIVE) {
    // the relative test also holds before the first iteration (an exact
    // start, where CG's alpha would be 0/0)
    if ((rc = tl_read_scalars(ctx))) return rc;
    const DevScalars &s0 = *ctx->host_sc;
    const double rel0 = s0.bb > 0 ? sqrt(s0.rro / s0.bb) : sqrt(s0.rro);
    if (rel0 < prm->eps) {
      res->iters = res->cg_iters = 0;
      res->error = s0.rro;
      res->converged = 1;
      res->rel_residual = rel0;
      res->launches = (int)ctx->launches;
      return TL_OK;
    }
  }
  const int which = ref ? TL_GRAPH_CG_REF : (exact ? TL_GRAPH_CG_EXACT : TL_GRAPH_CG_FAST);
  double rel = -1.0;
  int ran = 0;
  for (int restart = 0; restart < 8 && prm->maxiters >= 1; ++restart) {
    const int before = ctx->host_sc->iter;
    if ((rc = tl_run_graph(ctx, which, &ctx->last_solve_ms))) return rc;
    if ((rc = tl_read_scalars(ctx))) return rc;
    const int trips = ctx->host_sc->iter - (restart ? before : 0);
    ctx->launches += ref ? 4LL * trips : 4LL * ((trips + 1) / 2);
    ran = 1;
    if (!ref) {
      // the last iteration's p! and haloupdate! of u, p
      const double *pcur = (ctx->host_sc->iter & 1) ? ctx->F.pb : ctx->F.p;
      launch_tl_p(ctx->stream, ctx->F, ctx->g, tl_walk_for(ctx, exact), pcur, ctx->F.p, exact);
      CKL();
      if ((rc = tl_halo_update(ctx, 1, nullptr, -1, 1))) return rc;
      ctx->launches += 2;
    }
    if (prm->criterion != TL_CRIT_RELATIVE) break;
    double tr;
    if ((rc = true_residual(ctx, 0, &tr))) return rc;
    const double bb = ctx->host_sc->bb;
    rel = bb > 0 ? sqrt(tr / bb) : sqrt(tr);
    if (rel < prm->eps || ref || ctx->host_sc->iter >= prm->maxiters) break;
    if ((rc = true_residual(ctx, 1, &tr))) return rc;  // restart from the true residual
  }
  if ((rc = tl_read_scalars(ctx))) return rc;
  const DevScalars &sc = *ctx->host_sc;
  res->iters = sc.iter;
  res->cg_iters = sc.iter;
  res->error = ran ? sc.error : ERROR_START;
  res->converged = ran && (prm->criterion == TL_CRIT_RELATIVE ? (rel >= 0 && rel < prm->eps) : sc.converged);
  res->rel_residual = rel;
  res->launches = (int)ctx->launches;
  return TL_OK;
}

extern "C" int tl_solve(tl_ctx *ctx, double rx, double ry, const tl_params *prm, tl_result *res) {
  if (!ctx || !prm || !res) return TL_ERR_ARG;
  memset(res, 0, sizeof *res);
  res->r0_plain = -1.0;
  res->r0_pred = -1.0;
  if (!ctx->initialised) {
    tl_set_error(ctx, "solve before initialise/set_states");
    return TL_ERR_STATE;
  }
  if (prm->maxiters > ctx->cfg.maxiters) {
    tl_set_error(ctx, "maxiters %d exceeds the context's coefficient tables (%d)", prm->maxiters, ctx->cfg.maxiters);
    return TL_ERR_ARG;
  }
  ctx->launches = 0;
  switch (prm->solver) {
    case TL_SOLVER_CG:
      if (prm->precision == TL_PREC_FP32_IR) return tl_ir_solve(ctx, rx, ry, prm, res);
      return tl_cg_solve(ctx, rx, ry, prm, res);
    case TL_SOLVER_CHEBY: return tl_cheby_solve(ctx, rx, ry, prm, res);
    case TL_SOLVER_PPCG: return tl_ppcg_solve(ctx, rx, ry, prm, res);
    case TL_SOLVER_JACOBI: return tl_jacobi_solve(ctx, rx, ry, prm, res);
    default:
      tl_set_error(ctx, "unknown solver %d", prm->solver);
      return TL_ERR_ARG;
  }
}
