// tl_ir.cu -- CG with FP32 inner sweeps inside FP64 refinement.
//
// The inner iteration is CG on FP32 vectors (p, r, w and the correction x)
// with FP32 Kx/Ky; each dot sums a lane's four products in FP32 and
// accumulates those partial sums in FP64 (one FP64 add per four cells: the
// FP64 pipe of this part issues 1/64 as fast as FP32).  Whenever the FP32 residual has dropped by a factor
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
// keeps the identity term exact where the large coupling terms cancel.
#include <cmath>
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

void launch_ir_w(tl_ctx *ctx, const float *psrc, float *pdst, int guard, const Walk *walk = nullptr) {
  OpIrW op;
  op.F = ctx->F;
  op.g = g32_of(ctx);
  op.q = ptrs_of(ctx);
  op.psrc = psrc;
  op.pdst = pdst;
  op.guard = guard;
  const Walk &wk = walk ? *walk : ctx->ir->walk_w;
  k_walk32<OpIrW><<<wk.blocks, 32 * wk.warps, 0, ctx->stream>>>(op, wk, ctx->g.ny);
}

void launch_ir_ur(tl_ctx *ctx, const float *p, int guard, cudaGraphConditionalHandle cond, int set_cond,
                  const Walk *walk = nullptr) {
  OpIrUR op;
  op.F = ctx->F;
  op.g = g32_of(ctx);
  op.q = ptrs_of(ctx);
  op.p = p;
  op.guard = guard;
  op.cond = cond;
  op.set_cond = set_cond;
  const Walk &wk = walk ? *walk : ctx->ir->walk_ur;
  k_walk32<OpIrUR><<<wk.blocks, 32 * wk.warps, 0, ctx->stream>>>(op, wk, ctx->g.ny);
}

int occupancy32(int kernel, int threads) {
  int n = 0;
  cudaError_t e = kernel == 0 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_walk32<OpIrW>, threads, 0)
                              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_walk32<OpIrUR>, threads, 0);
  return e == cudaSuccess ? n : 1;
}

void tune_w32(tl_ctx *ctx, const Walk &wk) { launch_ir_w(ctx, ctx->ir->p, ctx->ir->pb, 0, &wk); }
void tune_ur32(tl_ctx *ctx, const Walk &wk) { launch_ir_ur(ctx, ctx->ir->pb, 0, 0, 0, &wk); }

int ensure_ir(tl_ctx *ctx) {
  if (ctx->ir) return TL_OK;
  tl_ir_state *ir = new (std::nothrow) tl_ir_state();
  if (!ir) return TL_ERR_NOMEM;
  ctx->ir = ir;
  const Geom &g = ctx->g;
  ir->pitch = (g.X + 31) / 32 * 32;
  ir->lead = (32 - g.hd % 32) % 32;
  ir->stride = (ir->lead + ir->pitch * (long long)g.Y + 64 + 63) / 64 * 64;
  CK(cudaMalloc(&ir->buf, sizeof(float) * ir->stride * 7));
  CK(cudaMemsetAsync(ir->buf, 0, sizeof(float) * ir->stride * 7, ctx->stream));
  float *f[7];
  for (int k = 0; k < 7; ++k) f[k] = ir->buf + ir->stride * k + ir->lead;
  ir->kx = f[0]; ir->ky = f[1]; ir->p = f[2]; ir->pb = f[3]; ir->r = f[4]; ir->w = f[5]; ir->x = f[6];
  // tune on the zeroed buffers, then zero them again: the trial launches
  // leave NaN behind (alpha = 0/0)
  ir->walk_w = tl_autotune(ctx, 128, occupancy32(0, 128), occupancy32(0, 256), tune_w32);
  ir->walk_ur = tl_autotune(ctx, 128, occupancy32(1, 128), occupancy32(1, 256), tune_ur32);
  CK(cudaMemsetAsync(ir->buf, 0, sizeof(float) * ir->stride * 7, ctx->stream));
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
  launch_ir_w(ctx, a, b, 0);
  launch_ir_ur(ctx, b, 0, h, 0);
  launch_ir_w(ctx, b, a, 1);
  launch_ir_ur(ctx, a, 1, h, 1);
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

int tl_ensure_ir(tl_ctx *ctx) { return ensure_ir(ctx); }

void tl_release_ir_graphs(tl_ctx *ctx) {
  if (!ctx->ir) return;
  for (auto &gx : ctx->ir->graph)
    if (gx) {
      cudaGraphExecDestroy(gx);
      gx = nullptr;
    }
}

void tl_release_ir(tl_ctx *ctx) {
  if (!ctx->ir) return;
  for (auto &gx : ctx->ir->graph)
    if (gx) cudaGraphExecDestroy(gx);
  if (ctx->ir->buf) cudaFree(ctx->ir->buf);
  delete ctx->ir;
  ctx->ir = nullptr;
}

// The refinement step.  Returns the true r.r in *rr.
static int refine(tl_ctx *ctx, double *rr) {
  const G32 g32 = g32_of(ctx);
  k_ir_fold<<<grid_for((long long)ctx->g.nx * ctx->g.ny), 256, 0, ctx->stream>>>(ctx->F, ctx->g, g32, ctx->ir->x);
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
  const G32 g32 = g32_of(ctx);
  tl_ir_state *ir = ctx->ir;
  k_ir_convert<<<grid_for((long long)ctx->g.X * ctx->g.Y), 256, 0, ctx->stream>>>(ctx->F, ctx->g, g32, ir->kx, ir->ky,
                                                                                  ir->r, ir->p, ir->x);
  CKL();
  ctx->launches += 8;
  if ((rc = tl_read_scalars(ctx))) return rc;
  const double bb = ctx->host_sc->bb;
  double rr = ctx->host_sc->rro;
  double rel = bb > 0 ? sqrt(rr / bb) : sqrt(rr);
  int which = 0, refinements = 0;
  ctx->last_solve_ms = 0.0;
  while (rel >= p.eps && ctx->host_sc->iter < p.maxiters) {
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
          launch_ir_w(ctx, a, b, 1);
          launch_ir_ur(ctx, b, 1, 0, 0);
          launch_ir_w(ctx, b, a, 1);
          launch_ir_ur(ctx, a, 1, 0, 0);
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
    ctx->launches += 1 + 4LL * ((trips + 1) / 2);
    if (trips & 1) which ^= 1;  // the last step wrote p into the other buffer
    if ((rc = refine(ctx, &rr))) return rc;
    ++refinements;
    rel = bb > 0 ? sqrt(rr / bb) : sqrt(rr);
  }
  float *pcur = which ? ir->pb : ir->p;
  k_ir_export_p<<<grid_for((long long)ctx->g.nx * ctx->g.ny), 256, 0, ctx->stream>>>(ctx->F, ctx->g, g32, pcur);
  CKL();
  if ((rc = tl_halo_update(ctx, 1, up, 2, 1))) return rc;
  ctx->launches += 2;
  if ((rc = tl_read_scalars(ctx))) return rc;
  res->iters = ctx->host_sc->iter;
  res->cg_iters = ctx->host_sc->iter;
  res->error = rr;
  res->rel_residual = rel;
  res->converged = rel < p.eps;
  res->refinements = refinements;
  res->launches = (int)ctx->launches;
  if (prm->warmstart) tl_warm_after(ctx, res, prm->warmstart);
  return TL_OK;
}

int tl_ir_bench_kernel(tl_ctx *ctx, int kernel, int reps, double *ms_per_launch) {
  int rc = ensure_ir(ctx);
  if (rc) return rc;
  if (kernel != 2 && kernel != 3) return TL_ERR_ARG;
  tl_ir_state *ir = ctx->ir;
  CK(cudaEventRecord(ctx->tev0, ctx->stream));
  for (int k = 0; k < reps; ++k) {
    if (kernel == 2) launch_ir_w(ctx, (k & 1) ? ir->pb : ir->p, (k & 1) ? ir->p : ir->pb, 0);
    else launch_ir_ur(ctx, ir->pb, 0, 0, 0);
  }
  CKL();
  CK(cudaEventRecord(ctx->tev1, ctx->stream));
  CK(cudaEventSynchronize(ctx->tev1));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, ctx->tev0, ctx->tev1));
  *ms_per_launch = t / reps;
  return TL_OK;
}

tl::Walk *tl_ir_walk(tl_ctx *ctx, int kernel) {
  if (ensure_ir(ctx)) return nullptr;
  return kernel == 2 ? &ctx->ir->walk_w : &ctx->ir->walk_ur;
}
