// tl_api.cu -- the C ABI (include/tealeaf_gb300.h): context, copies, and the
// host orchestration of each reference entry point.  Iteration loops run as
// CUDA graphs whose while-node is driven by the convergence test on the
// device; the host only reads the scalars back once a solve has ended.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "tl_internal.cuh"
#include "tl_solvers.h"

using namespace tl;

namespace {

constexpr int EXACT_WARPS = 4;
constexpr int EXACT_ROWS = 8;

long long round_up(long long v, long long m) { return (v + m - 1) / m * m; }

Walk make_walk(int nx, int ny, int warps, int rows, int max_blocks) {
  Walk w;
  w.warps = warps;
  w.rows = rows;
  const int TW = 64 * warps;
  w.ntx = (nx + TW - 1) / TW;
  const int nty = (ny + rows - 1) / rows;
  w.tiles = w.ntx * nty;
  w.blocks = w.tiles < max_blocks ? w.tiles : max_blocks;
  if (w.blocks < 1) w.blocks = 1;
  return w;
}

}  // namespace

void tl_set_error(tl_ctx *ctx, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(ctx->msg, sizeof ctx->msg, fmt, ap);
  va_end(ap);
}

int tl_cuda_fail(tl_ctx *ctx, cudaError_t e, const char *what, int line) {
  tl_set_error(ctx, "CUDA error in %s (tl_api line %d): %s", what, line, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? TL_ERR_NOMEM : TL_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// creation
// ---------------------------------------------------------------------------

extern "C" int tl_create(tl_ctx **out, const tl_config *cfg) {
  if (!out || !cfg) return TL_ERR_ARG;
  *out = nullptr;
  tl_ctx *ctx = new (std::nothrow) tl_ctx();
  if (!ctx) return TL_ERR_NOMEM;
  *out = ctx;
  if (cfg->xcells < 1 || cfg->ycells < 1 || cfg->halodepth < 1 || cfg->maxiters < 1 ||
      (cfg->mode != TL_MODE_REFERENCE && cfg->mode != TL_MODE_TEALEAF)) {
    tl_set_error(ctx, "invalid configuration (cells %d x %d, halo depth %d, maxiters %d, mode %d)", cfg->xcells,
                 cfg->ycells, cfg->halodepth, cfg->maxiters, cfg->mode);
    return TL_ERR_ARG;
  }
  const int X = cfg->xcells + 2 * cfg->halodepth, Y = cfg->ycells + 2 * cfg->halodepth;
  if (cfg->mode == TL_MODE_REFERENCE && X != Y) {
    tl_set_error(ctx, "DimensionMismatch: celly broadcasts vertexy against vertexx (src/chunk.jl:44) on a "
                      "non-square deck");
    return TL_ERR_REFERENCE_THROWS;
  }
  ctx->cfg = *cfg;
  Geom &g = ctx->g;
  g.nx = cfg->xcells;
  g.ny = cfg->ycells;
  g.hd = cfg->halodepth;
  g.X = X;
  g.Y = Y;
  g.pitch = round_up(X, 16);
  ctx->lead = (16 - (cfg->halodepth % 16)) % 16;
  CK(cudaGetDevice(&ctx->device));
  CK(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, ctx->device));
  CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  CK(cudaEventCreate(&ctx->ev0));
  CK(cudaEventCreate(&ctx->ev1));
  CK(cudaEventCreate(&ctx->tev0));
  CK(cudaEventCreate(&ctx->tev1));

  ctx->walk_exact = make_walk(g.nx, g.ny, EXACT_WARPS, EXACT_ROWS, 2 * ctx->sm_count);
  ctx->max_blocks = 8 * ctx->sm_count;  // the autotuner tries at most 8 resident blocks per SM
  const int max_blocks = ctx->max_blocks;
  const char *loop = getenv("TEALEAF_GB300_LOOP");
  ctx->host_loop = loop && !strcmp(loop, "host");

  // fields: TL_NFIELDS reference fields + pb, ub, sdb, diag
  const int nbuf = TL_NFIELDS + 4;
  const long long per = round_up(ctx->lead + g.pitch * (long long)Y, 32);
  ctx->field_stride = per;
  CK(cudaMalloc(&ctx->buf, sizeof(double) * per * nbuf));
  CK(cudaMemsetAsync(ctx->buf, 0, sizeof(double) * per * nbuf, ctx->stream));
  ctx->buf_bytes = sizeof(double) * per * nbuf;
  double *f[nbuf];
  for (int k = 0; k < nbuf; ++k) f[k] = ctx->buf + per * k + ctx->lead;
  Fields &F = ctx->F;
  F.density0 = f[TL_DENSITY0]; F.density = f[TL_DENSITY]; F.energy0 = f[TL_ENERGY0]; F.energy = f[TL_ENERGY];
  F.u = f[TL_U]; F.u0 = f[TL_U0]; F.p = f[TL_P]; F.r = f[TL_R]; F.mi = f[TL_MI]; F.w = f[TL_W];
  F.kx = f[TL_KX]; F.ky = f[TL_KY]; F.sd = f[TL_SD]; F.volume = f[TL_VOLUME];
  F.pb = f[TL_NFIELDS]; F.ub = f[TL_NFIELDS + 1]; F.sdb = f[TL_NFIELDS + 2]; F.diag = f[TL_NFIELDS + 3];
  for (int k = 0; k < TL_NFIELDS; ++k) ctx->field_ptr[k] = f[k];

  const size_t tab = (size_t)cfg->maxiters + 2;
  CK(cudaMalloc(&ctx->small, sizeof(double) * (4 * tab + (size_t)MAX_RED * max_blocks) + sizeof(DevScalars) + 256));
  char *s = reinterpret_cast<char *>(ctx->small);
  F.cgalpha = reinterpret_cast<double *>(s);
  F.cgbeta = F.cgalpha + tab;
  F.chebyalpha = F.cgbeta + tab;
  F.chebybeta = F.chebyalpha + tab;
  F.partials = F.chebybeta + tab;
  F.sc = reinterpret_cast<DevScalars *>(F.partials + (size_t)MAX_RED * max_blocks);
  F.counter = reinterpret_cast<unsigned *>(reinterpret_cast<char *>(F.sc) + sizeof(DevScalars));
  ctx->small_bytes = sizeof(double) * (4 * tab + (size_t)MAX_RED * max_blocks) + sizeof(DevScalars) + 256;
  CK(cudaMemsetAsync(ctx->small, 0, ctx->small_bytes, ctx->stream));
  CK(cudaMallocHost(&ctx->host_sc, sizeof(DevScalars)));

  if (cfg->mode == TL_MODE_TEALEAF) {
    // Tune the fused kernels on the zeroed fields, then zero everything the
    // trial launches touched (they leave NaN behind: alpha = 0/0).
    ctx->walk_w64 = tl_autotune(ctx, 64, tl_occupancy_cg(0, 128), tl_occupancy_cg(0, 256), tl_launch_w64_for_tuning);
    ctx->walk_ur64 = tl_autotune(ctx, 64, tl_occupancy_cg(1, 128), tl_occupancy_cg(1, 256), tl_launch_ur64_for_tuning);
    CK(cudaMemsetAsync(ctx->buf, 0, ctx->buf_bytes, ctx->stream));
    CK(cudaMemsetAsync(ctx->small, 0, ctx->small_bytes, ctx->stream));
  } else {
    ctx->walk_w64 = ctx->walk_ur64 = ctx->walk_exact;
  }
  launch_fill(ctx->stream, F.volume, g, cfg->dx * cfg->dy);  // chunk.jl:79
  CKL();
  CK(cudaStreamSynchronize(ctx->stream));
  return TL_OK;
}

extern "C" int tl_destroy(tl_ctx *ctx) {
  if (!ctx) return TL_OK;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  tl_release_graphs(ctx);
  if (ctx->buf) cudaFree(ctx->buf);
  if (ctx->small) cudaFree(ctx->small);
  if (ctx->host_sc) cudaFreeHost(ctx->host_sc);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->tev0) cudaEventDestroy(ctx->tev0);
  if (ctx->tev1) cudaEventDestroy(ctx->tev1);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  tl_release_ir(ctx);
  tl_release_warm(ctx);
  delete ctx;
  return TL_OK;
}

extern "C" const char *tl_last_error(const tl_ctx *ctx) { return ctx ? ctx->msg : "null context"; }

// ---------------------------------------------------------------------------
// copies
// ---------------------------------------------------------------------------

static int check_field(tl_ctx *ctx, int field, int ld) {
  if (field < 0 || field >= TL_NFIELDS) {
    tl_set_error(ctx, "field %d out of range", field);
    return TL_ERR_ARG;
  }
  if (ld < ctx->g.X) {
    tl_set_error(ctx, "leading dimension %d is smaller than X = %d", ld, ctx->g.X);
    return TL_ERR_ARG;
  }
  return TL_OK;
}

// Pinned (page-locked, mapped) host memory is read and written by a kernel
// over the host link; any other host memory goes through cudaMemcpy2DAsync.
// On this part the kernel path runs at the link's rate, as the copy engines
// do, and keeps that rate where the copy engines' slows down under sustained
// load.
static const void *mapped_ptr(const void *host) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

__global__ void k_copy_pitched(double *__restrict__ dst, long long dpitch, const double *__restrict__ src,
                               long long spitch, int X, int Y) {
  const long long n = (long long)X * Y;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const long long i = k % X, j = k / X;
    dst[i + j * dpitch] = src[i + j * spitch];
  }
}

static int copy_field(tl_ctx *ctx, double *dst, long long dpitch, const double *src, long long spitch,
                      cudaMemcpyKind kind, const void *host) {
  const Geom &g = ctx->g;
  const void *mapped = mapped_ptr(host);
  if (mapped) {
    const double *s = kind == cudaMemcpyHostToDevice ? static_cast<const double *>(mapped) : src;
    double *d = kind == cudaMemcpyHostToDevice ? dst : static_cast<double *>(const_cast<void *>(mapped));
    k_copy_pitched<<<8 * ctx->sm_count, 256, 0, ctx->stream>>>(d, dpitch, s, spitch, g.X, g.Y);
    CKL();
  } else {
    CK(cudaMemcpy2DAsync(dst, sizeof(double) * dpitch, src, sizeof(double) * spitch, sizeof(double) * g.X, g.Y,
                         kind, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return TL_OK;
}

extern "C" int tl_upload(tl_ctx *ctx, int field, const double *host, int ld) {
  if (!ctx || !host) return TL_ERR_ARG;
  int rc = check_field(ctx, field, ld);
  if (rc) return rc;
  return copy_field(ctx, ctx->field_ptr[field], ctx->g.pitch, host, ld, cudaMemcpyHostToDevice, host);
}

extern "C" int tl_download(tl_ctx *ctx, int field, double *host, int ld) {
  if (!ctx || !host) return TL_ERR_ARG;
  int rc = check_field(ctx, field, ld);
  if (rc) return rc;
  return copy_field(ctx, host, ld, ctx->field_ptr[field], ctx->g.pitch, cudaMemcpyDeviceToHost, host);
}

// ---------------------------------------------------------------------------
// state, halo, init helpers
// ---------------------------------------------------------------------------

extern "C" int tl_set_states(tl_ctx *ctx, const tl_state *states, int nstates) {
  if (!ctx || !states || nstates < 1 || nstates > MAX_STATES) {
    if (ctx) tl_set_error(ctx, "state count %d outside 1..%d", nstates, MAX_STATES);
    return TL_ERR_ARG;
  }
  StateTable t;
  memset(&t, 0, sizeof t);
  for (int k = 0; k < nstates; ++k) t.s[k] = states[k];
  t.n = nstates;
  launch_set_states(ctx->stream, ctx->F, ctx->g, t, ctx->cfg.xmin, ctx->cfg.ymin, ctx->cfg.dx, ctx->cfg.dy,
                    ctx->cfg.mode);
  CKL();
  ctx->initialised = 1;
  return TL_OK;
}

double *tl_exchange_ptr(tl_ctx *ctx, int ex) {
  switch (ex) {
    case TL_EX_DENSITY: return ctx->F.density;
    case TL_EX_P: return ctx->F.p;
    case TL_EX_ENERGY0: return ctx->F.energy0;
    case TL_EX_ENERGY: return ctx->F.energy;
    case TL_EX_U: return ctx->F.u;
    default: return ctx->F.sd;
  }
}

int tl_halo_check(tl_ctx *ctx, int depth) {
  const Geom &g = ctx->g;
  if (depth < 1) {
    tl_set_error(ctx, "halo depth %d < 1", depth);
    return TL_ERR_ARG;
  }
  if (ctx->cfg.mode == TL_MODE_REFERENCE) {
    if (g.hd - depth - 1 < 0) {
      tl_set_error(ctx, "BoundsError: halo index %d (1-based) in updateface! (src/kernels.jl:196)", g.hd - depth);
      return TL_ERR_REFERENCE_THROWS;
    }
  } else if (depth > g.hd) {
    tl_set_error(ctx, "halo depth %d exceeds halo_depth %d", depth, g.hd);
    return TL_ERR_ARG;
  }
  if (depth > g.nx || depth > g.ny) {
    tl_set_error(ctx, "halo depth %d exceeds the interior", depth);
    return TL_ERR_ARG;
  }
  return TL_OK;
}

// Fields currently marked for exchange, in EXCHANGE_FIELDS order.
int tl_marked(tl_ctx *ctx, double **ptrs) {
  int n = 0;
  for (int k = 0; k < TL_NEX; ++k)
    if (ctx->toexchange[k]) ptrs[n++] = tl_exchange_ptr(ctx, k);
  return n;
}

extern "C" int tl_halo_update(tl_ctx *ctx, int depth, const int *fields, int nfields, int reset) {
  if (!ctx) return TL_ERR_ARG;
  int rc = tl_halo_check(ctx, depth);
  if (rc) return rc;
  double *ptrs[TL_NEX];
  int n = 0;
  if (nfields >= 0) {
    for (int k = 0; k < nfields; ++k)
      if (!fields || fields[k] < 0 || fields[k] >= TL_NEX) {
        tl_set_error(ctx, "exchange field out of range");
        return TL_ERR_ARG;
      }
    if (reset)
      for (int k = 0; k < TL_NEX; ++k) ctx->toexchange[k] = 0;
    for (int k = 0; k < nfields; ++k) {
      ctx->toexchange[fields[k]] = 1;
      ptrs[n++] = tl_exchange_ptr(ctx, fields[k]);
    }
  } else {
    n = tl_marked(ctx, ptrs);
  }
  launch_halo(ctx->stream, ptrs, n, ctx->g, depth, ctx->cfg.mode);
  CKL();
  return TL_OK;
}

extern "C" int tl_initialise(tl_ctx *ctx, const tl_state *states, int nstates) {
  int rc = tl_set_states(ctx, states, nstates);
  if (rc) return rc;
  const int ex[3] = {TL_EX_DENSITY, TL_EX_ENERGY0, TL_EX_ENERGY};
  if ((rc = tl_halo_update(ctx, 1, ex, 3, 1))) return rc;
  launch_copy_full(ctx->stream, ctx->F.energy, ctx->F.energy0, ctx->g);  // TeaLeaf.jl:41
  CKL();
  CK(cudaStreamSynchronize(ctx->stream));
  return TL_OK;
}

extern "C" int tl_copy_u(tl_ctx *ctx) {
  if (!ctx) return TL_ERR_ARG;
  launch_copyu(ctx->stream, ctx->F, ctx->g, ctx->walk_exact, 1);
  CKL();
  return TL_OK;
}

extern "C" int tl_residual(tl_ctx *ctx) {
  if (!ctx) return TL_ERR_ARG;
  launch_residual(ctx->stream, ctx->F, ctx->g, ctx->cfg.mode);
  CKL();
  return TL_OK;
}

extern "C" int tl_finalise(tl_ctx *ctx) {
  if (!ctx) return TL_ERR_ARG;
  launch_finalise(ctx->stream, ctx->F, ctx->g);
  CKL();
  return TL_OK;
}

extern "C" int tl_solve_finished(tl_ctx *ctx, int checkresult) {  // kernels.jl:166-170
  if (!ctx) return TL_ERR_ARG;
  int rc;
  if (checkresult && (rc = tl_residual(ctx))) return rc;
  if ((rc = tl_finalise(ctx))) return rc;
  const int ex = TL_EX_ENERGY;
  if ((rc = tl_halo_update(ctx, 1, &ex, 1, 0))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  return TL_OK;
}

extern "C" int tl_field_summary(tl_ctx *ctx, double out[4]) {
  if (!ctx || !out) return TL_ERR_ARG;
  launch_summary(ctx->stream, ctx->F, ctx->g, ctx->walk_exact);
  CKL();
  CK(cudaMemcpyAsync(ctx->host_sc, ctx->F.sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (int k = 0; k < 4; ++k) out[k] = ctx->host_sc->red[k];
  return TL_OK;
}

extern "C" int tl_get_cg_coefficients(tl_ctx *ctx, double *alpha, double *beta, int n) {
  if (!ctx || n < 0 || n > ctx->cfg.maxiters) return TL_ERR_ARG;
  if (n == 0) return TL_OK;
  CK(cudaStreamSynchronize(ctx->stream));
  if (alpha) CK(cudaMemcpy(alpha, ctx->F.cgalpha + 1, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (beta) CK(cudaMemcpy(beta, ctx->F.cgbeta + 1, sizeof(double) * n, cudaMemcpyDeviceToHost));
  return TL_OK;
}

extern "C" int tl_reduction_layout(tl_ctx *ctx, int *warps, int *rows, int *blocks) {
  if (!ctx) return TL_ERR_ARG;
  if (warps) *warps = ctx->walk_exact.warps;
  if (rows) *rows = ctx->walk_exact.rows;
  if (blocks) *blocks = ctx->walk_exact.blocks;
  return TL_OK;
}

extern "C" int tl_synchronize(tl_ctx *ctx) {
  if (!ctx) return TL_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  return TL_OK;
}

extern "C" int tl_last_solve_ms(tl_ctx *ctx, double *ms) {
  if (!ctx || !ms) return TL_ERR_ARG;
  *ms = ctx->last_solve_ms;
  return TL_OK;
}

extern "C" int tl_timer_start(tl_ctx *ctx) {
  if (!ctx) return TL_ERR_ARG;
  CK(cudaEventRecord(ctx->tev0, ctx->stream));
  return TL_OK;
}

extern "C" int tl_timer_stop(tl_ctx *ctx, double *ms) {
  if (!ctx || !ms) return TL_ERR_ARG;
  CK(cudaEventRecord(ctx->tev1, ctx->stream));
  CK(cudaEventSynchronize(ctx->tev1));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, ctx->tev0, ctx->tev1));
  *ms = t;
  return TL_OK;
}

extern "C" int tl_bench_kernel(tl_ctx *ctx, int kernel, int reps, double *ms_per_launch) {
  if (!ctx || !ms_per_launch || reps < 1 || ctx->cfg.mode != TL_MODE_TEALEAF) return TL_ERR_ARG;
  const Fields &F = ctx->F;
  if (kernel >= 6 && kernel <= 9) return tl_ir_bench_kernel(ctx, kernel, reps, ms_per_launch);
  if (kernel == 2 || kernel == 3) {
    tl_set_error(ctx, "kernel %d: the 48-byte FP32 pair is retired (8 and 9 are the FP32 CG iteration)", kernel);
    return TL_ERR_ARG;
  }
  if (kernel < 0 || kernel > 12) return TL_ERR_ARG;
  if (kernel == 10) launch_init_rdiag(ctx->stream, F, ctx->g);  // the fused Jacobi sweep's reciprocal diagonal
  else launch_init_diag(ctx->stream, F, ctx->g);
  CKL();
  CK(cudaEventRecord(ctx->tev0, ctx->stream));
  for (int k = 0; k < reps; ++k) {
    if (kernel == 0) launch_tl_w(ctx->stream, F, ctx->g, ctx->walk_w64, (k & 1) ? F.pb : F.p, (k & 1) ? F.p : F.pb, 0, 0);
    else if (kernel == 1) launch_tl_ur(ctx->stream, F, ctx->g, ctx->walk_ur64, F.pb, 0, 0, 0, 0);
    else if (kernel == 4)
      launch_cheby_step(ctx->stream, F, ctx->g, ctx->walk_w64, (k & 1) ? F.ub : F.u, (k & 1) ? F.u : F.ub, 0, 0, 0, 0,
                        0);
    else if (kernel == 5)
      launch_ppcg_inner(ctx->stream, F, ctx->g, ctx->walk_w64, (k & 1) ? F.sdb : F.sd, (k & 1) ? F.sd : F.sdb, 1, 0, 0,
                        0, 0, 0);
    else if (kernel == 10)  // the fused Jacobi sweep, on the layout the fused Jacobi solve uses
      launch_jacobi(ctx->stream, F, ctx->g, ctx->walk_w64, (k & 1) ? F.ub : F.u, (k & 1) ? F.u : F.ub, 0, 0);
    else if (kernel == 11) {  // haloupdate! of u and p at depth 1 (CG.jl:23)
      double *ptrs[2] = {F.u, F.p};
      launch_halo(ctx->stream, ptrs, 2, ctx->g, 1, TL_MODE_TEALEAF);
    } else if (kernel == 12)  // PPCG's outer u/r update with sd = r / theta
      launch_ppcg_ur(ctx->stream, F, ctx->g, ctx->walk_ur64, F.p, F.sd, 0, 0);
    else {
      tl_set_error(ctx, "kernel %d has no benchmark", kernel);
      return TL_ERR_ARG;
    }
  }
  CKL();
  CK(cudaEventRecord(ctx->tev1, ctx->stream));
  CK(cudaEventSynchronize(ctx->tev1));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, ctx->tev0, ctx->tev1));
  *ms_per_launch = t / reps;
  return TL_OK;
}

static Walk *layout_of(tl_ctx *ctx, int kernel) {
  if (ctx->cfg.mode != TL_MODE_TEALEAF) return nullptr;
  switch (kernel) {
    case 0: return &ctx->walk_w64;
    case 1: return &ctx->walk_ur64;
    case 8:
    case 9: return tl_ir_walk(ctx, kernel);
    default: return nullptr;
  }
}

extern "C" int tl_get_layout(tl_ctx *ctx, int kernel, int *warps, int *rows, int *blocks) {
  if (!ctx) return TL_ERR_ARG;
  Walk *w = layout_of(ctx, kernel);
  if (!w) {
    tl_set_error(ctx, "no tuned layout for kernel %d in this mode", kernel);
    return TL_ERR_ARG;
  }
  if (warps) *warps = w->warps;
  if (rows) *rows = w->rows;
  if (blocks) *blocks = w->blocks;
  return TL_OK;
}

extern "C" int tl_set_layout(tl_ctx *ctx, int kernel, int warps, int rows, int blocks) {
  if (!ctx) return TL_ERR_ARG;
  Walk *w = layout_of(ctx, kernel);
  if (!w || (warps != 4 && warps != 8) || rows < 1 || blocks < 1 || blocks > ctx->max_blocks) {
    tl_set_error(ctx, "invalid layout for kernel %d: %d warps, %d rows, %d blocks (at most %d)", kernel, warps, rows,
                 blocks, ctx->max_blocks);
    return TL_ERR_ARG;
  }
  const int cols = kernel >= 2 ? 128 : 64;
  const int TW = cols * warps;
  Walk n;
  n.warps = warps;
  n.rows = rows;
  n.ntx = (ctx->g.nx + TW - 1) / TW;
  n.tiles = n.ntx * ((ctx->g.ny + rows - 1) / rows);
  n.blocks = blocks < n.tiles ? blocks : n.tiles;
  *w = n;
  // graphs hold the old launch configuration
  tl_release_graphs(ctx);
  tl_release_ir_graphs(ctx);
  return TL_OK;
}

extern "C" int tl_diffuse(tl_ctx *ctx, const tl_params *prm, double dt, int nsteps, int summaryfrequency,
                          int checkresult, tl_result *results, double *summaries, int maxsummaries,
                          int *nsummaries) {
  if (!ctx || !prm || !results || nsteps < 0 || summaryfrequency < 1) return TL_ERR_ARG;
  if (nsummaries) *nsummaries = 0;
  const double rx = dt / (ctx->cfg.dx * ctx->cfg.dx);  // TeaLeaf.jl:69-70
  const double ry = dt / (ctx->cfg.dy * ctx->cfg.dy);
  int taken = 0, rc;
  auto summary = [&]() -> int {
    if (!checkresult) return TL_OK;
    double out[4];
    int r = tl_field_summary(ctx, out);
    if (r) return r;
    if (summaries && taken < maxsummaries)
      for (int k = 0; k < 4; ++k) summaries[4 * taken + k] = out[k];
    ++taken;
    return TL_OK;
  };
  for (int tt = 1; tt <= nsteps; ++tt) {
    const int ex[2] = {TL_EX_ENERGY, TL_EX_DENSITY};
    if ((rc = tl_halo_update(ctx, 1, ex, 2, 1))) return rc;
    if ((rc = tl_solve(ctx, rx, ry, prm, &results[tt - 1]))) return rc;
    if ((rc = tl_solve_finished(ctx, checkresult))) return rc;
    if (tt % summaryfrequency == 0 && (rc = summary())) return rc;
  }
  if ((rc = summary())) return rc;
  if (nsummaries) *nsummaries = taken < maxsummaries ? taken : maxsummaries;
  return TL_OK;
}
