// tl_warm.cu -- the learned warm start inside CG.solve! (tealeaf mode, FP64
// and FP32-refined CG).  After tea_leaf_init and copyu! the context holds
// u = u0 = u^n and the plain start's residual r = p = u0 - A u^n.  With the
// previous step's u^{n-1} kept on the device, the network predicts
// x = u^n + (1 + g) (u^n - u^{n-1}); the plain start is both the fallback and
// the judge: x replaces u (and its residual replaces r, p) only when
// ||u0 - A x|| < ||u0 - A u^n||.  The solve then runs unchanged and must meet
// eps on the true residual as before.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <new>

#include "tl_conv.h"
#include "tl_march.cuh"
#include "tl_solvers.h"
#include "tl_walk.cuh"

struct tl_warm_state {
  void *wbuf = nullptr;                 // BF16 weights of the six layers, then FP32 biases
  __nv_bfloat16 *w[TL_WARM_LAYERS] = {};
  float *b[TL_WARM_LAYERS] = {};
  void *act = nullptr;                  // feature map (16 ch) + two 32-channel activation maps + g
  __nv_bfloat16 *feat = nullptr, *a0 = nullptr, *a1 = nullptr;
  float *g = nullptr;
  double *uprev = nullptr;              // u^{n-1}, laid out like the context's fields
  double *stats = nullptr;              // block partials of u.u and d.d, then the two totals
  tl_warm_crop *crop = nullptr;         // device copy of the whole-domain crop
  int have_prev = 0;
  // the iteration guard (tl_warm_after): plain-start control solves bracket
  // runs of at most `trust` solves from the prediction
  int ctrl_iters = -1;                  // iterations of the last solve from the plain start
  int run = 0;                          // solves from the prediction since that control
  long long run_iters = 0;              // their iterations
  int trust = 2, cooloff = 0, backoff = 4;
};

namespace tl {
namespace {

constexpr int STAT_BLOCKS = 256;

// Partial sums over the interior of u0.u0 and (u0 - uprev).(u0 - uprev).
__global__ void __launch_bounds__(256) k_warm_stats(Fields F, Geom g, const double *uprev, double *part) {
  double su = 0.0, sd = 0.0;
  const long long n = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const size_t c = g.at((int)(k % g.nx), (int)(k / g.nx));
    const double u = F.u0[c], d = u - uprev[c];
    su += u * u;
    sd += d * d;
  }
  __shared__ double s1[256], s2[256];
  s1[threadIdx.x] = su;
  s2[threadIdx.x] = sd;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      s1[threadIdx.x] += s1[threadIdx.x + w];
      s2[threadIdx.x] += s2[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s1[0];
    part[2 * blockIdx.x + 1] = s2[0];
  }
}

__global__ void k_warm_stats_fold(double *part, int nblk) {
  double su = 0.0, sd = 0.0;
  for (int k = 0; k < nblk; ++k) {
    su += part[2 * k];
    sd += part[2 * k + 1];
  }
  part[2 * nblk] = su;
  part[2 * nblk + 1] = sd;
}

// x = u0 + (1 + g) (u0 - uprev) on the interior, into ub.
__global__ void k_warm_candidate(Fields F, Geom g, const double *uprev, const float *gv) {
  const long long n = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(k % g.nx), j = (int)(k / g.nx);
    const size_t c = g.at(i, j);
    const double u = F.u0[c];
    F.ub[c] = u + (1.0 + (double)gv[k]) * (u - uprev[c]);
  }
}

__global__ void k_copy_u0(Fields F, Geom g, double *uprev) {
  const long long n = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const size_t c = g.at((int)(k % g.nx), (int)(k / g.nx));
    uprev[c] = F.u0[c];
  }
}

// Residual of the candidate: w = u0 - A ub (true residual, 5-point operator), sum w.w.
struct OpWarmResid : NoSkip {
  Fields F;
  Geom g;
  __device__ void cell(int i, int j, double (&acc)[1]) const {
    const size_t c = g.at(i, j);
    const double t = dsub(F.u0[c], smvp_exact(F, g, F.ub, c, TL_MODE_TEALEAF));
    F.w[c] = t;
    acc[0] = dadd(acc[0], dmul(t, t));
  }
  __device__ void tile(int i0, int j0, int j1, double (&acc)[1]) const {
    for (int j = j0; j < j1; ++j) {
      if (i0 < g.nx) cell(i0, j, acc);
      if (i0 + 1 < g.nx) cell(i0 + 1, j, acc);
    }
  }
  __device__ void fin(const double *tot) const { F.sc->red[0] = tot[0]; }
};

// The prediction won: r = p = w and rr = its r.r.
__global__ void k_warm_accept(Fields F, Geom g) {
  const long long n = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const size_t c = g.at((int)(k % g.nx), (int)(k / g.nx));
    F.r[c] = F.w[c];
    F.p[c] = F.w[c];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) F.sc->rro = F.sc->red[0];
}

__global__ void k_to_bf16(const float *src, __nv_bfloat16 *dst, int n) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    dst[k] = __float2bfloat16(src[k]);
}

inline int grid_cells(const Geom &g) {
  long long b = ((long long)g.nx * g.ny + 255) / 256;
  if (b > 152LL * 8) b = 152LL * 8;
  return (int)(b < 1 ? 1 : b);
}

}  // namespace
}  // namespace tl

using namespace tl;

void tl_release_warm(tl_ctx *ctx) {
  tl_warm_state *ws = ctx->warm;
  if (!ws) return;
  if (ws->wbuf) cudaFree(ws->wbuf);
  if (ws->act) cudaFree(ws->act);
  if (ws->uprev) cudaFree(ws->uprev);
  if (ws->stats) cudaFree(ws->stats);
  if (ws->crop) cudaFree(ws->crop);
  delete ws;
  ctx->warm = nullptr;
}

extern "C" int tl_warm_load(tl_ctx *ctx, const float *params, int nparams) {
  if (!ctx || !params) return TL_ERR_ARG;
  if (nparams != TL_WARM_NPARAMS) {
    tl_set_error(ctx, "warm-start network has %d parameters, expected %d", nparams, TL_WARM_NPARAMS);
    return TL_ERR_ARG;
  }
  if (!ctx->warm) {
    ctx->warm = new (std::nothrow) tl_warm_state();
    if (!ctx->warm) return TL_ERR_NOMEM;
  }
  tl_warm_state *ws = ctx->warm;
  long long nw = 0, nb = 0;
  for (int l = 0; l < TL_WARM_LAYERS; ++l) {
    nw += (long long)TL_WARM_COUT[l] * 9 * TL_WARM_CIN[l];
    nb += TL_WARM_COUT[l];
  }
  if (!ws->wbuf) {
    const size_t wbytes = ((size_t)nw * 2 + 255) / 256 * 256;
    CK(cudaMalloc(&ws->wbuf, wbytes + sizeof(float) * (size_t)(nb + nw + nb)));
    long long ow = 0, ob = 0;
    float *bias_base = reinterpret_cast<float *>(static_cast<char *>(ws->wbuf) + wbytes);
    for (int l = 0; l < TL_WARM_LAYERS; ++l) {
      ws->w[l] = static_cast<__nv_bfloat16 *>(ws->wbuf) + ow;
      ws->b[l] = bias_base + ob;
      ow += (long long)TL_WARM_COUT[l] * 9 * TL_WARM_CIN[l];
      ob += TL_WARM_COUT[l];
    }
  }
  // stage the FP32 vector after the biases, then split it into BF16 weights and FP32 biases
  float *stage = ws->b[0] + nb;
  CK(cudaMemcpyAsync(stage, params, sizeof(float) * (size_t)nparams, cudaMemcpyHostToDevice, ctx->stream));
  long long off = 0;
  for (int l = 0; l < TL_WARM_LAYERS; ++l) {
    const int n = TL_WARM_COUT[l] * 9 * TL_WARM_CIN[l];
    k_to_bf16<<<(n + 255) / 256, 256, 0, ctx->stream>>>(stage + off, ws->w[l], n);
    CKL();
    off += n;
    CK(cudaMemcpyAsync(ws->b[l], stage + off, sizeof(float) * TL_WARM_COUT[l], cudaMemcpyDeviceToDevice,
                       ctx->stream));
    off += TL_WARM_COUT[l];
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return tl_warm_reset(ctx);
}

extern "C" int tl_warm_reset(tl_ctx *ctx) {
  if (!ctx) return TL_ERR_ARG;
  if (tl_warm_state *ws = ctx->warm) {
    ws->have_prev = 0;
    ws->ctrl_iters = -1;
    ws->run = 0;
    ws->run_iters = 0;
    ws->trust = 2;
    ws->cooloff = 0;
    ws->backoff = 4;
  }
  return TL_OK;
}

static int ensure_warm_buffers(tl_ctx *ctx) {
  tl_warm_state *ws = ctx->warm;
  const Geom &g = ctx->g;
  if (ws->act) return TL_OK;
  const size_t cells = (size_t)g.nx * g.ny;
  const size_t fbytes = (cells * 16 * 2 + 255) / 256 * 256, abytes = (cells * 32 * 2 + 255) / 256 * 256;
  CK(cudaMalloc(&ws->act, fbytes + 2 * abytes + sizeof(float) * cells));
  char *base = static_cast<char *>(ws->act);
  ws->feat = reinterpret_cast<__nv_bfloat16 *>(base);
  ws->a0 = reinterpret_cast<__nv_bfloat16 *>(base + fbytes);
  ws->a1 = reinterpret_cast<__nv_bfloat16 *>(base + fbytes + abytes);
  ws->g = reinterpret_cast<float *>(base + fbytes + 2 * abytes);
  CK(cudaMalloc(&ws->uprev, sizeof(double) * (size_t)g.pitch * g.Y));
  CK(cudaMemsetAsync(ws->uprev, 0, sizeof(double) * (size_t)g.pitch * g.Y, ctx->stream));
  CK(cudaMalloc(&ws->stats, sizeof(double) * (2 * STAT_BLOCKS + 2)));
  CK(cudaMalloc(&ws->crop, sizeof(tl_warm_crop)));
  return TL_OK;
}

// Called by the CG solves after tea_leaf_init, the halo and copyu!.
int tl_warm_try(tl_ctx *ctx, double rx, double ry, int warmstart, tl_result *res) {
  if (warmstart != TL_WARM_NETWORK && warmstart != TL_WARM_EXTRAPOLATE) {
    tl_set_error(ctx, "unknown warm-start mode %d", warmstart);
    return TL_ERR_ARG;
  }
  if (ctx->cfg.mode != TL_MODE_TEALEAF) {
    tl_set_error(ctx, "the warm start needs the tealeaf (5-point) semantics");
    return TL_ERR_ARG;
  }
  if (!ctx->warm) {
    ctx->warm = new (std::nothrow) tl_warm_state();
    if (!ctx->warm) return TL_ERR_NOMEM;
  }
  tl_warm_state *ws = ctx->warm;
  if (warmstart == TL_WARM_NETWORK && !ws->wbuf) {
    tl_set_error(ctx, "warm start asked before tl_warm_load");
    return TL_ERR_STATE;
  }
  int rc = ensure_warm_buffers(ctx);
  if (rc) return rc;
  const Geom &g = ctx->g;
  const Fields &F = ctx->F;
  cudaStream_t st = ctx->stream;
  if ((rc = tl_read_scalars(ctx))) return rc;
  const double bb = ctx->host_sc->bb, rr_plain = ctx->host_sc->rro;
  res->r0_plain = bb > 0 ? sqrt(rr_plain / bb) : sqrt(rr_plain);
  res->r0_pred = -1.0;
  res->warm = 0;
  const int extrapolate = warmstart == TL_WARM_EXTRAPOLATE;
  if (ws->have_prev && ws->cooloff > 0) {
    --ws->cooloff;
    res->warm = 3;
  } else if (ws->have_prev && (ws->ctrl_iters < 0 || ws->run >= ws->trust)) {
    res->warm = 4;  // control solve from the plain start
  } else if (ws->have_prev) {
    k_warm_stats<<<STAT_BLOCKS, 256, 0, st>>>(F, g, ws->uprev, ws->stats);
    k_warm_stats_fold<<<1, 1, 0, st>>>(ws->stats, STAT_BLOCKS);
    CKL();
    double tot[2];
    CK(cudaMemcpyAsync(tot, ws->stats + 2 * STAT_BLOCKS, sizeof tot, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    ctx->launches += 2;
    const double cells = (double)g.nx * g.ny;
    if (tot[0] > 0 && tot[1] > 0) {
      tl_warm_crop cr{};
      cr.u = F.u0 + g.at(0, 0);
      cr.uprev = ws->uprev + g.at(0, 0);
      cr.rho = F.density + g.at(0, 0);
      cr.pitch = g.pitch;
      cr.nx = g.nx;
      cr.ny = g.ny;
      cr.rx = rx;
      cr.ry = ry;
      cr.inv_su = 1.0 / sqrt(tot[0] / cells);
      cr.inv_sd = 1.0 / sqrt(tot[1] / cells);
      CK(cudaMemcpyAsync(ws->crop, &cr, sizeof cr, cudaMemcpyHostToDevice, st));
      if (extrapolate) {
        CK(cudaMemsetAsync(ws->g, 0, sizeof(float) * (size_t)g.nx * g.ny, st));   // g = 0: u^n + (u^n - u^{n-1})
      } else {
        if ((rc = tl_warm_features_launch(ws->crop, 1, g.ny, g.nx, ws->feat, st))) {
          tl_set_error(ctx, "warm-start feature kernel failed to launch");
          return rc;
        }
        const __nv_bfloat16 *in = ws->feat;
        __nv_bfloat16 *bufs[2] = {ws->a0, ws->a1};
        for (int l = 0; l < TL_WARM_LAYERS; ++l) {
          const int last = l == TL_WARM_LAYERS - 1;
          __nv_bfloat16 *out = last ? nullptr : bufs[l & 1];
          rc = tl_conv_forward(in, ws->w[l], ws->b[l], nullptr, nullptr, out, last ? ws->g : nullptr, 1, g.ny,
                               g.nx, TL_WARM_CIN[l], TL_WARM_COUT[l], last ? 0 : 1, st);
          if (rc) {
            tl_set_error(ctx, "warm-start convolution %d failed to launch", l);
            return rc;
          }
          in = out;
        }
        ctx->launches += 1 + TL_WARM_LAYERS;
      }
      k_warm_candidate<<<grid_cells(g), 256, 0, st>>>(F, g, ws->uprev, ws->g);
      CKL();
      double *ub = F.ub;
      launch_halo(st, &ub, 1, g, 1, TL_MODE_TEALEAF);
      CKL();
      OpWarmResid op;
      op.F = F;
      op.g = g;
      launch_walk<1>(st, op, ctx->walk_exact, g.ny);
      CKL();
      ctx->launches += 3;
      if ((rc = tl_read_scalars(ctx))) return rc;
      const double rr_pred = ctx->host_sc->red[0];
      res->r0_pred = bb > 0 ? sqrt(rr_pred / bb) : sqrt(rr_pred);
      if (rr_pred < rr_plain) {
        launch_copy_full(st, F.u, F.ub, g);
        k_warm_accept<<<grid_cells(g), 256, 0, st>>>(F, g);
        CKL();
        const int up[2] = {TL_EX_U, TL_EX_P};
        if ((rc = tl_halo_update(ctx, 1, up, 2, 1))) return rc;
        ctx->launches += 3;
        res->warm = 1;
      } else {
        res->warm = 2;
      }
    }
  }
  k_copy_u0<<<grid_cells(g), 256, 0, st>>>(F, g, ws->uprev);
  CKL();
  ctx->launches += 1;
  ws->have_prev = 1;
  return TL_OK;
}

// After the solve: the second judgement.  A smaller initial residual does
// not imply fewer CG iterations (error the prediction adds across the whole
// spectrum costs more than the smooth error of the plain start), so runs of at
// most `trust` solves from the prediction are bracketed by control solves
// from the plain start.  When a run's mean iteration count exceeds the mean of
// its two controls, the prediction pauses for `backoff` steps (4, 8, ... 64)
// and trust drops to 2; otherwise trust doubles (up to 32) and the backoff
// returns to 4.  A network prediction rejected by the residual judge
// (outside a run) pauses the next ones the same way, so that rejected
// inference stops costing time.
void tl_warm_after(tl_ctx *ctx, const tl_result *res, int warmstart) {
  tl_warm_state *ws = ctx->warm;
  if (!ws) return;
  if (res->warm == 1) {
    ++ws->run;
    ws->run_iters += res->iters;
    return;
  }
  if (res->warm == 2 && ws->run == 0 && warmstart == TL_WARM_NETWORK) {
    // the network's prediction lost to the plain start by residual: its
    // inference was wasted, so the next attempts back off the same way (the
    // extrapolation candidate costs one pass and is tried every step)
    ws->cooloff = ws->backoff;
    ws->backoff = ws->backoff < 64 ? 2 * ws->backoff : 64;
  }
  if (ws->run > 0 && ws->ctrl_iters >= 0) {
    const double pred = (double)ws->run_iters / ws->run, plain = 0.5 * (ws->ctrl_iters + res->iters);
    if (pred > plain) {
      ws->cooloff = ws->backoff;
      ws->backoff = ws->backoff < 64 ? 2 * ws->backoff : 64;
      ws->trust = 2;
    } else {
      ws->trust = ws->trust < 32 ? 2 * ws->trust : 32;
      ws->backoff = 4;
    }
  }
  ws->run = 0;
  ws->run_iters = 0;
  ws->ctrl_iters = res->iters;
}
