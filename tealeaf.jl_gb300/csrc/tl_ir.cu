// tl_ir.cu -- CG with FP32 inner sweeps inside FP64 refinement.
//
// The inner iteration is CG on FP32 vectors (p, r and the correction x) with
// the stencil faces formed from FP32 inverse weights; each dot sums a lane's
// products over eight rows in FP32 and accumulates those partial sums in
// FP64 (one FP64 add per 32 cells: the FP64 pipe of this part issues 1/64 as
// fast as FP32).  Whenever the FP32 residual has dropped by a factor
// delta since the last refinement, or claims convergence, the loop returns to
// a refinement step done entirely in FP64:
//     u += x;  x = 0;  r = u0 - A u (true residual);  test ||r|| / ||u0||.
// The FP32 residual is then replaced by the true one and the search
// direction is kept (the reliable-update form of iterative refinement), so
// the Krylov space built so far is not thrown away.
//
// FP32 arrays: pitched like the FP64 fields, 32 floats per pitch unit, first
// interior cell of each row 128-byte aligned; each lane owns 4 consecutive
// cells (one float4).  The FP32 stencil uses the difference form
// w = p + kx1 (p - pE) + kx0 (p - pW) + ky1 (p - pN) + ky0 (p - pS), which
// keeps the identity term exact where the large coupling terms cancel, with
// kx = rx/2 (iw_W + iw) and ky = ry/2 (iw_S + iw) from the inverse weights.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>

#include "tl_ir_ops.cuh"

using namespace tl;


namespace {

int grid_for(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152LL * 32) b = 152LL * 32;
  return (int)(b < 1 ? 1 : b);
}

template <int AHEAD>
void launch_ir_dir_t(tl_ctx *ctx, const float *psrc, float *pdst, int guard, const Walk &wk) {
  OpIrDir<AHEAD> op;
  op.F = ctx->F;
  op.g = g32_of(ctx);
  op.q = ptrs_of(ctx);
  op.psrc = psrc;
  op.pdst = pdst;
  op.guard = guard;
  k_walk32<OpIrDir<AHEAD>><<<wk.blocks, 32 * wk.warps, 0, ctx->stream>>>(op, wk, ctx->g.ny);
}

void launch_ir_dir(tl_ctx *ctx, const float *psrc, float *pdst, int guard) {
  if (ctx->ir->dir_ahead == 1) launch_ir_dir_t<1>(ctx, psrc, pdst, guard, ctx->ir->walk_dir);
  else launch_ir_dir_t<2>(ctx, psrc, pdst, guard, ctx->ir->walk_dir);
}

template <int AHEAD, int KIND>
void launch_sweep_t(tl_ctx *ctx, const Walk &wk, const float *src, float *a, float *b, float *out, int pp, int guard,
                    cudaGraphConditionalHandle cond, int set_cond) {
  OpIrSweep<AHEAD, KIND> op;
  op.F = ctx->F;
  op.g = g32_of(ctx);
  op.s = src;
  op.iw = ctx->ir->iw;
  op.a = a;
  op.b = b;
  op.out = out;
  op.pp = pp;
  op.guard = guard;
  op.cond = cond;
  op.set_cond = set_cond;
  k_walk32<OpIrSweep<AHEAD, KIND>><<<wk.blocks, 32 * wk.warps, 0, ctx->stream>>>(op, wk, ctx->g.ny);
}

template <int KIND>
void launch_sweep_kind(tl_ctx *ctx, const float *src, float *a, float *b, float *out, int pp, int guard,
                       cudaGraphConditionalHandle cond, int set_cond) {
  const int slot = KIND == SWEEP_PPCG_LAST ? SWEEP_PPCG_INNER : KIND;
  const Walk &wk = ctx->ir->walk_sweep[slot];
  if (ctx->ir->sweep_ahead[slot] == 1) launch_sweep_t<1, KIND>(ctx, wk, src, a, b, out, pp, guard, cond, set_cond);
  else launch_sweep_t<2, KIND>(ctx, wk, src, a, b, out, pp, guard, cond, set_cond);
}

// The FP32 CG update step on p' (x += alpha p', r -= alpha w, r.r).
void launch_ir_update(tl_ctx *ctx, const float *p, int guard, cudaGraphConditionalHandle cond, int set_cond) {
  launch_sweep_kind<SWEEP_CG>(ctx, p, ctx->ir->x, ctx->ir->r, nullptr, 0, guard, cond, set_cond);
}

template <class Op>
int occupancy_of(int threads) {
  int n = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_walk32<Op>, threads, 0);
  return e == cudaSuccess ? n : 1;
}

void tune_dir2(tl_ctx *ctx, const Walk &wk) { launch_ir_dir_t<2>(ctx, ctx->ir->p, ctx->ir->pb, 0, wk); }
void tune_dir1(tl_ctx *ctx, const Walk &wk) { launch_ir_dir_t<1>(ctx, ctx->ir->p, ctx->ir->pb, 0, wk); }

// Tuning launches of one sweep form on the (zeroed) FP32 buffers.
template <int AHEAD, int KIND>
void tune_sweep(tl_ctx *ctx, const Walk &wk) {
  tl_ir_state *ir = ctx->ir;
  if (KIND == SWEEP_CG) launch_sweep_t<AHEAD, KIND>(ctx, wk, ir->pb, ir->x, ir->r, nullptr, 0, 0, 0, 0);
  else if (KIND == SWEEP_PPCG_UPDATE) launch_sweep_t<AHEAD, KIND>(ctx, wk, ir->pb, ir->x, ir->r, ir->sd, 0, 0, 0, 0);
  else if (KIND == SWEEP_CHEBY) launch_sweep_t<AHEAD, KIND>(ctx, wk, ir->sd, ir->r, ir->p, ir->sdb, 0, 0, 0, 0);
  else launch_sweep_t<AHEAD, KIND>(ctx, wk, ir->sd, ir->r, ir->x, ir->sdb, 1, 0, 0, 0);
}

// Average time of `reps` launches of one tuned form (after two warm-up launches).
float time_form(tl_ctx *ctx, void (*launch)(tl_ctx *, const Walk &), const Walk &wk, int reps) {
  launch(ctx, wk);
  launch(ctx, wk);
  float ms = -1.f;
  if (cudaEventRecord(ctx->tev0, ctx->stream) != cudaSuccess) return ms;
  for (int k = 0; k < reps; ++k) launch(ctx, wk);
  if (cudaEventRecord(ctx->tev1, ctx->stream) != cudaSuccess || cudaEventSynchronize(ctx->tev1) != cudaSuccess)
    return ms;
  cudaEventElapsedTime(&ms, ctx->tev0, ctx->tev1);
  return ms / reps;
}

// Both forms of one sweep kind tuned; the faster kept (without tuning: the
// fixed layout and the form that loads rows as reached).
template <int KIND>
void tune_kind(tl_ctx *ctx, bool tuning) {
  using O2 = OpIrSweep<2, KIND>;
  using O1 = OpIrSweep<1, KIND>;
  const Walk w2 = tl_autotune(ctx, 128, occupancy_of<O2>(128), occupancy_of<O2>(256), tuning ? tune_sweep<2, KIND> : nullptr);
  const Walk w1 = tl_autotune(ctx, 128, occupancy_of<O1>(128), occupancy_of<O1>(256), tuning ? tune_sweep<1, KIND> : nullptr);
  const float t2 = tuning ? time_form(ctx, tune_sweep<2, KIND>, w2, 5) : 1.f;
  const float t1 = tuning ? time_form(ctx, tune_sweep<1, KIND>, w1, 5) : 0.f;
  const int ahead = (t1 >= 0.f && t2 >= 0.f && t2 < t1) ? 2 : 1;
  ctx->ir->sweep_ahead[KIND] = ahead;
  ctx->ir->walk_sweep[KIND] = ahead == 1 ? w1 : w2;
}

constexpr int NBUF = 7;  // FP32 arrays: p, pb, r, x, sd, sdb, iw

// The FP32 buffers of a context, allocated on first use; `tune` autotunes
// the single-deck kernels' layouts (the batched solve has its own walk and
// skips it).
int ensure_ir(tl_ctx *ctx, bool tune = true) {
  if (ctx->ir) return TL_OK;
  tl_ir_state *ir = new (std::nothrow) tl_ir_state();
  if (!ir) return TL_ERR_NOMEM;
  ctx->ir = ir;
  const Geom &g = ctx->g;
  ir->pitch = (g.X + 31) / 32 * 32;
  ir->lead = (32 - g.hd % 32) % 32;
  ir->stride = (ir->lead + ir->pitch * (long long)g.Y + 64 + 63) / 64 * 64;
  CK(cudaMalloc(&ir->buf, sizeof(float) * ir->stride * NBUF));
  CK(cudaMemsetAsync(ir->buf, 0, sizeof(float) * ir->stride * NBUF, ctx->stream));
  float *f[NBUF];
  for (int k = 0; k < NBUF; ++k) f[k] = ir->buf + ir->stride * k + ir->lead;
  ir->p = f[0]; ir->pb = f[1]; ir->r = f[2]; ir->x = f[3]; ir->sd = f[4]; ir->sdb = f[5]; ir->iw = f[6];
  // tune on the zeroed buffers, then zero them again: the trial launches
  // leave NaN behind (alpha = 0/0)
  // OpIrDir and each sweep kind: both forms tuned, the faster kept (without
  // tuning, TEALEAF_GB300_TUNE=0: the fixed layout, the direction step with
  // rows two ahead and the sweeps with rows as reached)
  const char *env = getenv("TEALEAF_GB300_TUNE");
  const bool tuning = tune && !(env && !strcmp(env, "0"));
  const Walk d2 = tl_autotune(ctx, 128, occupancy_of<OpIrDir<2>>(128), occupancy_of<OpIrDir<2>>(256),
                              tuning ? tune_dir2 : nullptr);
  const Walk d1 = tl_autotune(ctx, 128, occupancy_of<OpIrDir<1>>(128), occupancy_of<OpIrDir<1>>(256),
                              tuning ? tune_dir1 : nullptr);
  const float s2 = tuning ? time_form(ctx, tune_dir2, d2, 5) : 0.f;
  const float s1 = tuning ? time_form(ctx, tune_dir1, d1, 5) : 1.f;
  ir->dir_ahead = (s1 >= 0.f && s2 >= 0.f && s1 < s2) ? 1 : 2;
  ir->walk_dir = ir->dir_ahead == 1 ? d1 : d2;
  tune_kind<SWEEP_CG>(ctx, tuning);
  tune_kind<SWEEP_PPCG_UPDATE>(ctx, tuning);
  tune_kind<SWEEP_CHEBY>(ctx, tuning);
  tune_kind<SWEEP_PPCG_INNER>(ctx, tuning);
  cudaGetLastError();
  CK(cudaMemsetAsync(ir->buf, 0, sizeof(float) * ir->stride * NBUF, ctx->stream));
  return TL_OK;
}

int ir_graph(tl_ctx *ctx, int which, cudaGraphExec_t *out) {
  tl_ir_state *ir = ctx->ir;
  if (ir->graph[which]) {
    *out = ir->graph[which];
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
  float *a = which ? ir->pb : ir->p, *b = which ? ir->p : ir->pb;
  launch_ir_dir(ctx, a, b, 0);
  launch_ir_update(ctx, b, 0, h, 0);
  launch_ir_dir(ctx, b, a, 1);
  launch_ir_update(ctx, a, 1, h, 1);
  cudaError_t le = cudaGetLastError();
  cudaGraph_t captured = nullptr;
  e = cudaStreamEndCapture(ctx->stream, &captured);
  if (e != cudaSuccess || le != cudaSuccess) {
    cudaGraphDestroy(graph);
    return tl_cuda_fail(ctx, e != cudaSuccess ? e : le, "capture of the FP32 loop", __LINE__);
  }
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return tl_cuda_fail(ctx, e, "cudaGraphInstantiate", __LINE__);
  ir->graph[which] = exec;
  *out = exec;
  return TL_OK;
}

}  // namespace

int tl_ensure_ir(tl_ctx *ctx, int tune) { return ensure_ir(ctx, tune != 0); }

void tl_release_ir_graphs(tl_ctx *ctx) {
  if (!ctx->ir) return;
  for (auto &gx : ctx->ir->graph)
    if (gx) {
      cudaGraphExecDestroy(gx);
      gx = nullptr;
    }
  for (auto &gx : ctx->ir->ppcg_graph)
    if (gx) {
      cudaGraphExecDestroy(gx);
      gx = nullptr;
    }
}

void tl_release_ir(tl_ctx *ctx) {
  if (!ctx->ir) return;
  tl_release_ir_graphs(ctx);
  if (ctx->ir->buf) cudaFree(ctx->ir->buf);
  delete ctx->ir;
  ctx->ir = nullptr;
}

// The refinement step: u += e, e = 0 (e: the FP32 correction, x by
// default), the halo of u, the true residual r = u0 - A u in FP64 and its
// FP32 copy.  Returns the true r.r in *rr.
static int refine(tl_ctx *ctx, double *rr, float *e = nullptr) {
  const G32 g32 = g32_of(ctx);
  k_ir_fold<<<grid_for((long long)ctx->g.nx * ctx->g.ny), 256, 0, ctx->stream>>>(ctx->F, ctx->g, g32,
                                                                                e ? e : ctx->ir->x);
  CKL();
  double *u = ctx->F.u;
  launch_halo(ctx->stream, &u, 1, ctx->g, 1, TL_MODE_TEALEAF);
  CKL();
  OpIrResid op;
  op.F = ctx->F;
  op.g = ctx->g;
  op.g32 = g32;
  op.r32 = ctx->ir->r;
  launch_walk<1>(ctx->stream, op, ctx->walk_exact, ctx->g.ny);
  CKL();
  ctx->launches += 3;
  int rc = tl_read_scalars(ctx);
  if (rc) return rc;
  *rr = ctx->host_sc->red[0];
  return TL_OK;
}

// The inner loop with its refinements, from the state tl_cg_init and copyu
// left (u, r = p = u0 - A u, r.r in rro).  Runs until the relative true
// residual is below eps, the iteration budget is spent or, as CG presteps of
// Chebyshev (switch rule 1), the switch test held; the FP32 search direction
// is exported into p.  Returns the last true r.r and its relative value.
static int ir_loop(tl_ctx *ctx, const tl_params &p, double rx, double ry, double *rr_out, double *rel_out,
                   int *refinements) {
  const G32 g32 = g32_of(ctx);
  tl_ir_state *ir = ctx->ir;
  k_ir_convert<<<grid_for((long long)ctx->g.X * ctx->g.Y), 256, 0, ctx->stream>>>(ctx->F, ctx->g, g32, ir->r, ir->p,
                                                                                  ir->x);
  k_ir_convert_iw<<<grid_for((long long)ctx->g.X * ctx->g.Y), 256, 0, ctx->stream>>>(ctx->F, ctx->g, g32, ir->iw,
                                                                                     p.coefficient, rx, ry);
  CKL();
  ctx->launches += 9;
  int rc = tl_read_scalars(ctx);
  if (rc) return rc;
  const double bb = ctx->host_sc->bb;
  double rr = ctx->host_sc->rro;
  double rel = bb > 0 ? sqrt(rr / bb) : sqrt(rr);
  int which = 0, nref = 0, switched = 0;
  ctx->last_solve_ms = 0.0;
  while (rel >= p.eps && ctx->host_sc->iter < p.maxiters && !switched) {
    k_ir_start<<<1, 1, 0, ctx->stream>>>(ctx->F.sc, rr, IR_DELTA * IR_DELTA);
    CKL();
    cudaGraphExec_t exec = nullptr;
    if (!ctx->host_loop && (rc = ir_graph(ctx, which, &exec))) return rc;
    const int before = ctx->host_sc->iter;
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    if (ctx->host_loop) {
      // the same kernels launched from the host (see run_host_loop_cg)
      float *a = which ? ir->pb : ir->p, *b = which ? ir->p : ir->pb;
      for (;;) {
        for (int k = 0; k < 8; ++k) {
          launch_ir_dir(ctx, a, b, 1);
          launch_ir_update(ctx, b, 1, 0, 0);
          launch_ir_dir(ctx, b, a, 1);
          launch_ir_update(ctx, a, 1, 0, 0);
        }
        CKL();
        if ((rc = tl_read_scalars(ctx))) return rc;
        if (ctx->host_sc->done) break;
      }
    } else {
      CK(cudaGraphLaunch(exec, ctx->stream));
    }
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    CK(cudaEventSynchronize(ctx->ev1));
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1));
    ctx->last_solve_ms += t;
    if ((rc = tl_read_scalars(ctx))) return rc;
    const int trips = ctx->host_sc->iter - before;
    switched = ctx->host_sc->prestep_switch;
    ctx->launches += 1 + 4LL * ((trips + 1) / 2);
    if (trips & 1) which ^= 1;  // the last step wrote p into the other buffer
    if ((rc = refine(ctx, &rr))) return rc;
    ++nref;
    rel = bb > 0 ? sqrt(rr / bb) : sqrt(rr);
  }
  float *pcur = which ? ir->pb : ir->p;
  ir->pwhich = which;
  k_ir_export_p<<<grid_for((long long)ctx->g.nx * ctx->g.ny), 256, 0, ctx->stream>>>(ctx->F, ctx->g, g32, pcur);
  CKL();
  const int up[2] = {TL_EX_U, TL_EX_P};
  if ((rc = tl_halo_update(ctx, 1, up, 2, 1))) return rc;
  ctx->launches += 2;
  if ((rc = tl_read_scalars(ctx))) return rc;
  *rr_out = rr;
  *rel_out = rel;
  *refinements = nref;
  return TL_OK;
}

int tl_ir_solve(tl_ctx *ctx, double rx, double ry, const tl_params *prm, tl_result *res) {
  if (ctx->cfg.mode != TL_MODE_TEALEAF) {
    tl_set_error(ctx, "FP32 refinement needs the tealeaf (5-point) semantics");
    return TL_ERR_ARG;
  }
  int rc = ensure_ir(ctx);
  if (rc) return rc;
  tl_params p = *prm;
  p.criterion = TL_CRIT_RELATIVE;
  if ((rc = tl_cg_init(ctx, rx, ry, p.coefficient, 1))) return rc;
  if ((rc = tl_set_loop_params(ctx, &p, 0, 0))) return rc;
  const int up[2] = {TL_EX_U, TL_EX_P};
  if ((rc = tl_halo_update(ctx, 1, up, 2, 1))) return rc;
  if ((rc = tl_copy_u(ctx))) return rc;
  if (prm->warmstart && (rc = tl_warm_try(ctx, rx, ry, prm->warmstart, res))) return rc;
  double rr = 0.0, rel = 0.0;
  int refinements = 0;
  if ((rc = ir_loop(ctx, p, rx, ry, &rr, &rel, &refinements))) return rc;
  res->iters = ctx->host_sc->iter;
  res->cg_iters = ctx->host_sc->iter;
  res->error = rr;
  res->rel_residual = rel;
  res->converged = rel < p.eps;
  res->refinements = refinements;
  res->launches = (int)ctx->launches;
  return TL_OK;
}

// The CG presteps of Chebyshev (Cheby.jl:15-35, tealeaf mode) as FP32 inner
// sweeps inside FP64 refinement.  The FP32 epilogues record alpha and beta in
// the coefficient tables for the eigenvalue estimate and apply the switch
// test (Cheby.jl:25-29) to the inner r.r; when it holds, the correction is
// folded into u and the true residual measured before the Chebyshev phase
// takes over.  On return u (with its halo) is the iterate, the host scalars
// hold the loop's end state, *switched says whether the Chebyshev (or PPCG)
// phase takes over (the switch test held and the true residual is not yet
// below eps), *rr_out is the true r.r and *rel_out its relative value.  The
// same presteps serve PPCG (PPCG.jl:27-31 is the same test).
int tl_ir_presteps(tl_ctx *ctx, double rx, double ry, const tl_params *prm, int *refinements, double *rr_out,
                   double *rel_out, int *switched) {
  int rc = ensure_ir(ctx);
  if (rc) return rc;
  tl_params p = *prm;
  p.criterion = TL_CRIT_RELATIVE;
  // exact 0: the stored diagonal, which the FP64 Chebyshev steps after the
  // switch read
  if ((rc = tl_cg_init(ctx, rx, ry, p.coefficient, 0))) return rc;
  if ((rc = tl_set_loop_params(ctx, &p, 1, 0))) return rc;
  const int up[2] = {TL_EX_U, TL_EX_P};
  if ((rc = tl_halo_update(ctx, 1, up, 2, 1))) return rc;
  if ((rc = tl_copy_u(ctx))) return rc;
  if ((rc = ir_loop(ctx, p, rx, ry, rr_out, rel_out, refinements))) return rc;
  *switched = ctx->host_sc->prestep_switch && *rel_out >= p.eps;
  return TL_OK;
}

tl::Walk *tl_ir_walk(tl_ctx *ctx, int kernel) {
  if (ensure_ir(ctx)) return nullptr;
  switch (kernel) {
    case 8: return &ctx->ir->walk_dir;
    case 9: return &ctx->ir->walk_sweep[SWEEP_CG];
    default: return nullptr;
  }
}

// ---------------------------------------------------------------------------
// Chebyshev steps in FP32 inside FP64 refinement
// ---------------------------------------------------------------------------

namespace tl {
namespace {

// The start of the FP32 Chebyshev phase: p32 = (float) p (the first
// Chebyshev step's p) and both correction buffers zeroed.
__global__ void k_cheby32_convert(Fields F, Geom g, G32 g32, float *p, float *e0, float *e1) {
  const long long n = (long long)g.X * g.Y;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int I = (int)(k % g.X), J = (int)(k / g.X);
    const size_t c = (size_t)I + (size_t)J * g.pitch, c32 = (size_t)I + (size_t)J * g32.pitch;
    const bool interior = I >= g.hd && I < g.X - g.hd && J >= g.hd && J < g.Y - g.hd;
    p[c32] = interior ? (float)F.p[c] : 0.f;
    e0[c32] = 0.f;
    e1[c32] = 0.f;
  }
}

// One FP32 Chebyshev step on the correction (the sweep of kind SWEEP_CHEBY):
// r = r0 - A e, p = alpha_k p + beta_k r, e' = e + p, r.r.
void launch_cheby32(tl_ctx *ctx, const float *esrc, float *edst, int guard) {
  launch_sweep_kind<SWEEP_CHEBY>(ctx, esrc, ctx->ir->r, ctx->ir->p, edst, 0, guard, 0, 0);
}

}  // namespace
}  // namespace tl

// The Chebyshev iteration after its switch, in FP32 inside FP64 refinement
// (tealeaf mode).  On entry the FP64 Chebyshev phase has run its first step
// (the iterate is in ub after an odd count).  The FP32 steps solve for the
// correction of the current refinement with the same coefficient sequence;
// each refinement folds the correction into u, measures the true residual in
// FP64 and restarts the correction from it, so the recurrence continues
// unchanged.  Stops on the relative true residual ||u0 - A u|| / ||u0|| < eps
// or the iteration budget.
int tl_cheby32_run(tl_ctx *ctx, const tl_params *prm, int *refinements, double *rel_out) {
  int rc = ensure_ir(ctx);
  if (rc) return rc;
  tl_ir_state *ir = ctx->ir;
  const G32 g32 = g32_of(ctx);
  if ((rc = tl_read_scalars(ctx))) return rc;
  if (ctx->host_sc->cheby_iters & 1) {
    launch_copy_interior(ctx->stream, ctx->F.u, ctx->F.ub, ctx->g);
    CKL();
  }
  k_cheby32_convert<<<grid_for((long long)ctx->g.X * ctx->g.Y), 256, 0, ctx->stream>>>(ctx->F, ctx->g, g32, ir->p,
                                                                                       ir->x, ir->pb);
  CKL();
  double rr;
  if ((rc = refine(ctx, &rr))) return rc;  // x = 0: the halo of u and the true residual
  const double bb = ctx->host_sc->bb;
  double rel = bb > 0 ? sqrt(rr / bb) : sqrt(rr);
  int nref = 0;
  float *ea = ir->x, *eb = ir->pb;  // the correction starts each inner loop in ea, zeroed
  ctx->last_solve_ms = 0.0;
  while (rel >= prm->eps && ctx->host_sc->iter < prm->maxiters) {
    k_ir_start<<<1, 1, 0, ctx->stream>>>(ctx->F.sc, rr, IR_DELTA * IR_DELTA);
    CKL();
    const int it0 = ctx->host_sc->cheby_iters;
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    for (;;) {
      for (int s = 0; s < 16; ++s) launch_cheby32(ctx, (s & 1) ? eb : ea, (s & 1) ? ea : eb, 1);
      CKL();
      if ((rc = tl_read_scalars(ctx))) return rc;
      if (ctx->host_sc->done) break;
    }
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    CK(cudaEventSynchronize(ctx->ev1));
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1));
    ctx->last_solve_ms += t;
    const int steps = ctx->host_sc->cheby_iters - it0;
    ctx->launches += 1 + steps;
    float *ecur = (steps & 1) ? eb : ea;
    if ((rc = refine(ctx, &rr, ecur))) return rc;
    ++nref;
    rel = bb > 0 ? sqrt(rr / bb) : sqrt(rr);
    eb = ecur == ir->x ? ir->pb : ir->x;
    ea = ecur;
  }
  k_ir_export_p<<<grid_for((long long)ctx->g.nx * ctx->g.ny), 256, 0, ctx->stream>>>(ctx->F, ctx->g, g32, ir->p);
  CKL();
  *refinements = nref;
  *rel_out = rel;
  return TL_OK;
}

// ---------------------------------------------------------------------------
// PPCG in FP32 inside FP64 refinement
// ---------------------------------------------------------------------------

namespace tl {
namespace {

// PPCG's update after the direction step (PPCG.jl:64-72 with the
// tealeaf-mode start of the inner sweeps): x += alpha p', r -= alpha A p',
// sd = r / theta.
void launch_ppcg32_ur(tl_ctx *ctx, const float *p, int guard) {
  tl_ir_state *ir = ctx->ir;
  launch_sweep_kind<SWEEP_PPCG_UPDATE>(ctx, p, ir->x, ir->r, ir->sd, 0, guard, 0, 0);
}

// One PPCG inner sweep in FP32 (PPCG.jl:74-88, the halo of sd reflected in
// the index math): r -= A sd, x += sd, sd' = alpha_pp sd + beta_pp r.  The
// last sweep of an outer step also sums r.r and closes the step (beta, the
// iteration count, the refinement test).
void launch_ppcg32_inner(tl_ctx *ctx, int pp, int last, int guard, cudaGraphConditionalHandle cond, int set_cond) {
  tl_ir_state *ir = ctx->ir;
  const float *src = (pp & 1) ? ir->sd : ir->sdb;
  float *dst = (pp & 1) ? ir->sdb : ir->sd;
  if (last) launch_sweep_kind<SWEEP_PPCG_LAST>(ctx, src, ir->r, ir->x, dst, pp, guard, cond, set_cond);
  else launch_sweep_kind<SWEEP_PPCG_INNER>(ctx, src, ir->r, ir->x, dst, pp, guard, 0, 0);
}

// One PPCG outer step in FP32: W (p' = beta p + r, w = A p', alpha), the
// update, and n inner sweeps, the last of which closes the step.  `which`
// selects the buffer that holds p; the step writes p' into the other one.
void ppcg32_outer(tl_ctx *ctx, int which, int n, int guard, cudaGraphConditionalHandle cond, int set_cond) {
  tl_ir_state *ir = ctx->ir;
  float *a = which ? ir->pb : ir->p, *b = which ? ir->p : ir->pb;
  launch_ir_dir(ctx, a, b, guard);
  launch_ppcg32_ur(ctx, b, 1);
  for (int pp = 1; pp <= n; ++pp) launch_ppcg32_inner(ctx, pp, pp == n, 1, cond, pp == n && set_cond);
}

int ppcg32_graph(tl_ctx *ctx, int which, int n, cudaGraphExec_t *out) {
  tl_ir_state *ir = ctx->ir;
  if (ir->ppcg_inner != n) {  // the recorded sweeps depend on the inner step count
    for (auto &gx : ir->ppcg_graph)
      if (gx) {
        cudaGraphExecDestroy(gx);
        gx = nullptr;
      }
    ir->ppcg_inner = n;
  }
  if (ir->ppcg_graph[which]) {
    *out = ir->ppcg_graph[which];
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
  // two outer steps per trip, p returning to its buffer
  ppcg32_outer(ctx, which, n, 0, h, 0);
  ppcg32_outer(ctx, which ^ 1, n, 1, h, 1);
  cudaError_t le = cudaGetLastError();
  cudaGraph_t captured = nullptr;
  e = cudaStreamEndCapture(ctx->stream, &captured);
  if (e != cudaSuccess || le != cudaSuccess) {
    cudaGraphDestroy(graph);
    return tl_cuda_fail(ctx, e != cudaSuccess ? e : le, "capture of the FP32 PPCG loop", __LINE__);
  }
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return tl_cuda_fail(ctx, e, "cudaGraphInstantiate", __LINE__);
  ir->ppcg_graph[which] = exec;
  *out = exec;
  return TL_OK;
}

}  // namespace
}  // namespace tl

// The PPCG iteration after its switch, in FP32 inside FP64 refinement
// (tealeaf mode).  On entry the FP32-refined CG presteps have ended at the
// switch (tl_ir_presteps): u holds the iterate, r its true residual in FP64
// and FP32, the search direction is in the FP32 buffer the presteps left it
// in, and the device scalars hold theta, beta and the inner coefficients.
// The outer steps continue the search direction; each refinement folds the
// correction into u, measures the true residual in FP64 and replaces the
// FP32 residual with it.  Stops on the relative true residual
// ||u0 - A u|| / ||u0|| < eps or the iteration budget.
int tl_ppcg32_run(tl_ctx *ctx, const tl_params *prm, double rr, int *refinements, double *rel_out) {
  int rc = ensure_ir(ctx);
  if (rc) return rc;
  tl_ir_state *ir = ctx->ir;
  const G32 g32 = g32_of(ctx);
  const int n = prm->ppcginnersteps;
  if ((rc = tl_read_scalars(ctx))) return rc;
  const double bb = ctx->host_sc->bb;
  double rel = bb > 0 ? sqrt(rr / bb) : sqrt(rr);
  int which = ir->pwhich, nref = 0;
  ctx->last_solve_ms = 0.0;
  while (rel >= prm->eps && ctx->host_sc->iter < prm->maxiters) {
    k_ir_start<<<1, 1, 0, ctx->stream>>>(ctx->F.sc, rr, IR_DELTA * IR_DELTA);
    CKL();
    cudaGraphExec_t exec = nullptr;
    if (!ctx->host_loop && (rc = ppcg32_graph(ctx, which, n, &exec))) return rc;
    const int before = ctx->host_sc->iter;
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    if (ctx->host_loop) {
      for (;;) {
        for (int k = 0; k < 4; ++k) {
          ppcg32_outer(ctx, which, n, 1, 0, 0);
          ppcg32_outer(ctx, which ^ 1, n, 1, 0, 0);
        }
        CKL();
        if ((rc = tl_read_scalars(ctx))) return rc;
        if (ctx->host_sc->done) break;
      }
    } else {
      CK(cudaGraphLaunch(exec, ctx->stream));
    }
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    CK(cudaEventSynchronize(ctx->ev1));
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1));
    ctx->last_solve_ms += t;
    if ((rc = tl_read_scalars(ctx))) return rc;
    const int steps = ctx->host_sc->iter - before;
    ctx->launches += 1 + (2LL + n) * steps;
    if (steps & 1) which ^= 1;  // the last outer step wrote p into the other buffer
    if ((rc = refine(ctx, &rr))) return rc;
    ++nref;
    rel = bb > 0 ? sqrt(rr / bb) : sqrt(rr);
  }
  ir->pwhich = which;
  k_ir_export_p<<<grid_for((long long)ctx->g.nx * ctx->g.ny), 256, 0, ctx->stream>>>(ctx->F, ctx->g, g32,
                                                                                      which ? ir->pb : ir->p);
  CKL();
  *refinements = nref;
  *rel_out = rel;
  return TL_OK;
}

// Back-to-back launches of one FP32 kernel on the current FP32 fields (ids as
// in tl_bench_kernel): 6 the Chebyshev step, 7 a PPCG inner sweep, 8 OpIrDir,
// 9 the CG update step.
int tl_ir_bench_kernel(tl_ctx *ctx, int kernel, int reps, double *ms_per_launch) {
  int rc = ensure_ir(ctx);
  if (rc) return rc;
  if (kernel < 6 || kernel > 9) return TL_ERR_ARG;
  tl_ir_state *ir = ctx->ir;
  CK(cudaEventRecord(ctx->tev0, ctx->stream));
  for (int k = 0; k < reps; ++k) {
    if (kernel == 8) launch_ir_dir(ctx, (k & 1) ? ir->pb : ir->p, (k & 1) ? ir->p : ir->pb, 0);
    else if (kernel == 9) launch_ir_update(ctx, ir->pb, 0, 0, 0);
    else if (kernel == 6) launch_cheby32(ctx, (k & 1) ? ir->pb : ir->x, (k & 1) ? ir->x : ir->pb, 0);
    else launch_ppcg32_inner(ctx, 1 + (k & 1), 0, 0, 0, 0);
  }
  CKL();
  CK(cudaEventRecord(ctx->tev1, ctx->stream));
  CK(cudaEventSynchronize(ctx->tev1));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, ctx->tev0, ctx->tev1));
  *ms_per_launch = t / reps;
  return TL_OK;
}
