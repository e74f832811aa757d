// tl_warm.cu -- the warm start inside CG.solve! (tealeaf mode, FP64 and
// FP32-refined CG).  After tea_leaf_init and copyu! the context holds
// u = u0 = u^n and the plain start's residual r = p = u0 - A u^n.  The
// context keeps the last six right-hand sides u^{n-1}, ..., u^{n-6}.
//
// The candidate start is the A-norm projection of the solution u^{n+1} =
// A^{-1} u0 onto a small basis: u^n, the increments u^n - u^{n-1},
// u^{n-1} - u^{n-2}, ... (those that exist, up to six), and, with the
// network, the network's correction g (u^n - u^{n-1}) (its prediction is
// u^n + (1 + g)(u^n - u^{n-1})).  With V the basis, the start
// x = V c minimises ||x - A^{-1} u0||_A over the span, from the Gram system
// (V^T A V) c = V^T u0: one pass over the fields forms every A v_j on the fly
// and the m(m+1)/2 + m sums, the host solves the m x m system (m <= 5), and a
// second pass forms x.  The span holds the plain start u^n and the linear
// extrapolation 2u^n - u^{n-1}, so x is never farther from the solution in
// the A-norm than either; the network's term enters with the weight that
// serves that norm best, and with weight ~0 where it does not help.
//
// The plain start is both the fallback and the judge: x replaces u (and its
// residual replaces r, p) only when ||u0 - A x|| < ||u0 - A u^n||.  The solve
// then runs unchanged and must meet eps on the true residual as before.
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
  double *hist[TL_WARM_HIST] = {};      // u^{n-1}, u^{n-2}, ..., laid out like the context's fields
  double *hist_base = nullptr;          // the one allocation they rotate through
  int nhist = 0;                        // how many of them hold an earlier step
  int net_skip = 0;                     // steps left before the network runs again
  int net_backoff = 1;                  // steps the next loss of the network's term skips (1, 2, ... 32)
  double *stats = nullptr;              // block partials of u.u and d.d, then the two totals
  double *gram = nullptr;               // block partials of the Gram system, then its totals
  tl_warm_crop *crop = nullptr;         // device copy of the whole-domain crop
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

// The projection basis.  Slot 0 holds u^n; slots 1..WARM_HIST the
// increments u^n - u^{n-1}, u^{n-1} - u^{n-2}, ... (the first nh of them
// exist, the others are zero); the last slot holds the network's correction
// g (u^n - u^{n-1}) when the network ran, else zero.  Fixed slots keep every
// index compile-time; the host solves the system on the slots in use.
constexpr int WARM_HIST = TL_WARM_HIST;                  // earlier right-hand sides kept
constexpr int PROJ_MAX = WARM_HIST + 2;                   // basis slots
constexpr int PROJ_NET = PROJ_MAX - 1;                    // the network's slot
constexpr int PROJ_NG = PROJ_MAX * (PROJ_MAX + 1) / 2;  // upper triangle of V^T A V
constexpr int PROJ_NACC = PROJ_NG + PROJ_MAX;           // ... then V^T u0
constexpr int GRAM_BLOCKS = 304;

struct ProjBasis {
  const double *u0;                 // u^n
  const double *h[WARM_HIST];       // u^{n-1}, u^{n-2}, ... (the first nh are set)
  const float *gv;                  // network output g (interior, row-major), or null
  int nh;                           // increments in the basis (1..WARM_HIST)
};

// The right-hand sides u^n, u^{n-1}, ... at one cell (zero past nh).
__device__ __forceinline__ void hist_at(const ProjBasis &B, size_t c, double (&hv)[WARM_HIST + 1]) {
  hv[0] = B.u0[c];
#pragma unroll
  for (int i = 1; i <= WARM_HIST; ++i) hv[i] = i <= B.nh ? B.h[i - 1][c] : 0.0;
}

// The basis slots at one cell.
__device__ __forceinline__ void basis_at(const ProjBasis &B, size_t c, long long k, double (&v)[PROJ_MAX]) {
  double hv[WARM_HIST + 1];
  hist_at(B, c, hv);
  v[0] = hv[0];
#pragma unroll
  for (int j = 1; j <= WARM_HIST; ++j) v[j] = j <= B.nh ? hv[j - 1] - hv[j] : 0.0;
  v[PROJ_NET] = B.gv ? (double)B.gv[k] * (hv[0] - hv[1]) : 0.0;
}

// The 5-point operator in difference form, v + sum k (v - v_nbr), with the
// reflective boundary folded in (a neighbour across the edge is the cell).
__device__ __forceinline__ double stencil(double vc, double ve, double vw, double vn, double vs, double kxE, double kxW,
                                          double kyN, double kyS) {
  return vc + kxE * (vc - ve) + kxW * (vc - vw) + kyN * (vc - vn) + kyS * (vc - vs);
}

// One pass: A v_j at every interior cell for every basis slot, from A of each
// earlier right-hand side (an increment's A v is the difference of two), and
// the sums v_a . A v_b (a <= b) and v_a . u0.  Fixed grid and block order:
// the sums are deterministic.
__global__ void __launch_bounds__(256) k_warm_gram(Fields F, Geom g, ProjBasis B, double *part) {
  double acc[PROJ_NACC];
#pragma unroll
  for (int a = 0; a < PROJ_NACC; ++a) acc[a] = 0.0;
  const long long n = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(k % g.nx), j = (int)(k / g.nx);
    const size_t c = g.at(i, j);
    const size_t cE = i + 1 < g.nx ? c + 1 : c, cW = i > 0 ? c - 1 : c;
    const size_t cN = j + 1 < g.ny ? c + g.pitch : c, cS = j > 0 ? c - g.pitch : c;
    const double kxE = F.kx[c + 1], kxW = F.kx[c], kyN = F.ky[c + g.pitch], kyS = F.ky[c];
    double hc[WARM_HIST + 1], ah[WARM_HIST + 1];
    hist_at(B, c, hc);
    ah[0] = stencil(hc[0], B.u0[cE], B.u0[cW], B.u0[cN], B.u0[cS], kxE, kxW, kyN, kyS);
#pragma unroll
    for (int q = 1; q <= WARM_HIST; ++q) {
      ah[q] = 0.0;
      if (q <= B.nh) {
        const double *h = B.h[q - 1];
        ah[q] = stencil(hc[q], h[cE], h[cW], h[cN], h[cS], kxE, kxW, kyN, kyS);
      }
    }
    double v[PROJ_MAX], av[PROJ_MAX];
    v[0] = hc[0];
    av[0] = ah[0];
#pragma unroll
    for (int q = 1; q <= WARM_HIST; ++q) {
      v[q] = q <= B.nh ? hc[q - 1] - hc[q] : 0.0;
      av[q] = q <= B.nh ? ah[q - 1] - ah[q] : 0.0;
    }
    v[PROJ_NET] = av[PROJ_NET] = 0.0;
    if (B.gv) {
      const long long kE = i + 1 < g.nx ? k + 1 : k, kW = i > 0 ? k - 1 : k;
      const long long kN = j + 1 < g.ny ? k + g.nx : k, kS = j > 0 ? k - g.nx : k;
      const double *h0 = B.h[0];
      auto t = [&](size_t cc, long long kk) { return (double)B.gv[kk] * (B.u0[cc] - h0[cc]); };
      v[PROJ_NET] = (double)B.gv[k] * (hc[0] - hc[1]);
      av[PROJ_NET] = stencil(v[PROJ_NET], t(cE, kE), t(cW, kW), t(cN, kN), t(cS, kS), kxE, kxW, kyN, kyS);
    }
    int tt = 0;
#pragma unroll
    for (int a = 0; a < PROJ_MAX; ++a)
#pragma unroll
      for (int b = a; b < PROJ_MAX; ++b, ++tt) acc[tt] = fma(v[a], av[b], acc[tt]);
#pragma unroll
    for (int a = 0; a < PROJ_MAX; ++a) acc[PROJ_NG + a] = fma(v[a], v[0], acc[PROJ_NG + a]);
  }
  __shared__ double ws[8][PROJ_NACC];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < PROJ_NACC; ++a) {
    const double val = warp_butterfly(acc[a]);
    if (lane == 0) ws[warp][a] = val;
  }
  __syncthreads();
  if (threadIdx.x < PROJ_NACC) {
    double val = ws[0][threadIdx.x];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) val += ws[w][threadIdx.x];
    part[(size_t)blockIdx.x * PROJ_NACC + threadIdx.x] = val;
  }
}

__global__ void k_warm_gram_fold(double *part, int nblk) {
  if (threadIdx.x >= PROJ_NACC) return;
  double v = 0.0;
  for (int b = 0; b < nblk; ++b) v += part[(size_t)b * PROJ_NACC + threadIdx.x];
  part[(size_t)nblk * PROJ_NACC + threadIdx.x] = v;
}

struct ProjCoef {
  double c[PROJ_MAX];  // zero on the slots not in use
};

// x = V c on the interior, into ub.
__global__ void k_warm_combine(Fields F, Geom g, ProjBasis B, ProjCoef C) {
  const long long n = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const size_t c = g.at((int)(k % g.nx), (int)(k / g.nx));
    double v[PROJ_MAX];
    basis_at(B, c, k, v);
    double x = 0.0;
#pragma unroll
    for (int a = 0; a < PROJ_MAX; ++a) x = fma(C.c[a], v[a], x);
    F.ub[c] = x;
  }
}

// x = 2 u^n - u^{n-1} on the interior, into ub.
__global__ void k_warm_extrapolate(Fields F, Geom g, const double *h0) {
  const long long n = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const size_t c = g.at((int)(k % g.nx), (int)(k / g.nx));
    const double u = F.u0[c];
    F.ub[c] = u + (u - h0[c]);
  }
}

__global__ void k_copy_u0(Fields F, Geom g, double *dst) {
  const long long n = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const size_t c = g.at((int)(k % g.nx), (int)(k / g.nx));
    dst[c] = F.u0[c];
  }
}

// Residual of the candidate: w = u0 - A ub (true residual, 5-point operator), sum w.w;
// with write 0 only the sum.
struct OpWarmResid : NoSkip {
  Fields F;
  Geom g;
  int write;  // 0: the norm only
  __device__ void cell(int i, int j, double (&acc)[1]) const {
    const size_t c = g.at(i, j);
    const double t = dsub(F.u0[c], smvp_exact(F, g, F.ub, c, TL_MODE_TEALEAF));
    if (write) F.w[c] = t;
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
  if (ws->hist_base) cudaFree(ws->hist_base);  // one allocation holds all of them (hist[] rotates)
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
    ws->nhist = 0;
    ws->net_skip = 0;
    ws->net_backoff = 1;
  }
  return TL_OK;
}

// Buffers of every warm-start mode: the three earlier solutions, the sums;
// the network's feature and activation maps only when `network`.
static int ensure_warm_buffers(tl_ctx *ctx, int network) {
  tl_warm_state *ws = ctx->warm;
  const Geom &g = ctx->g;
  const size_t cells = (size_t)g.nx * g.ny;
  if (!ws->hist_base) {
    const size_t fb = sizeof(double) * (size_t)g.pitch * g.Y;
    double *h = nullptr;
    CK(cudaMalloc(&h, TL_WARM_HIST * fb));
    CK(cudaMemsetAsync(h, 0, TL_WARM_HIST * fb, ctx->stream));
    ws->hist_base = h;
    for (int k = 0; k < TL_WARM_HIST; ++k) ws->hist[k] = h + (size_t)k * g.pitch * g.Y;
    CK(cudaMalloc(&ws->stats, sizeof(double) * (2 * STAT_BLOCKS + 2 + (size_t)(GRAM_BLOCKS + 1) * PROJ_NACC)));
    ws->gram = ws->stats + 2 * STAT_BLOCKS + 2;
    CK(cudaMalloc(&ws->crop, sizeof(tl_warm_crop)));
  }
  if (network && !ws->act) {
    const size_t fbytes = (cells * 16 * 2 + 255) / 256 * 256, abytes = (cells * 32 * 2 + 255) / 256 * 256;
    CK(cudaMalloc(&ws->act, fbytes + 2 * abytes + sizeof(float) * cells));
    char *base = static_cast<char *>(ws->act);
    ws->feat = reinterpret_cast<__nv_bfloat16 *>(base);
    ws->a0 = reinterpret_cast<__nv_bfloat16 *>(base + fbytes);
    ws->a1 = reinterpret_cast<__nv_bfloat16 *>(base + fbytes + abytes);
    ws->g = reinterpret_cast<float *>(base + fbytes + 2 * abytes);
  }
  return TL_OK;
}

// The network's output g for the current step (features from u^n, the
// density and u^n - u^{n-1}, then the six convolutions).
static int run_network(tl_ctx *ctx, double rx, double ry) {
  tl_warm_state *ws = ctx->warm;
  const Geom &g = ctx->g;
  const Fields &F = ctx->F;
  cudaStream_t st = ctx->stream;
  k_warm_stats<<<STAT_BLOCKS, 256, 0, st>>>(F, g, ws->hist[0], ws->stats);
  k_warm_stats_fold<<<1, 1, 0, st>>>(ws->stats, STAT_BLOCKS);
  CKL();
  double tot[2];
  CK(cudaMemcpyAsync(tot, ws->stats + 2 * STAT_BLOCKS, sizeof tot, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  ctx->launches += 2;
  if (!(tot[0] > 0) || !(tot[1] > 0)) return 1;  // no increment: nothing for the network to scale
  const double cells = (double)g.nx * g.ny;
  tl_warm_crop cr{};
  cr.u = F.u0 + g.at(0, 0);
  cr.uprev = ws->hist[0] + g.at(0, 0);
  cr.rho = F.density + g.at(0, 0);
  cr.pitch = g.pitch;
  cr.nx = g.nx;
  cr.ny = g.ny;
  cr.rx = rx;
  cr.ry = ry;
  cr.inv_su = 1.0 / sqrt(tot[0] / cells);
  cr.inv_sd = 1.0 / sqrt(tot[1] / cells);
  CK(cudaMemcpyAsync(ws->crop, &cr, sizeof cr, cudaMemcpyHostToDevice, st));
  int rc = tl_warm_features_launch(ws->crop, 1, g.ny, g.nx, ws->feat, st);
  if (rc) {
    tl_set_error(ctx, "warm-start feature kernel failed to launch");
    return -rc;
  }
  const __nv_bfloat16 *in = ws->feat;
  __nv_bfloat16 *bufs[2] = {ws->a0, ws->a1};
  for (int l = 0; l < TL_WARM_LAYERS; ++l) {
    const int last = l == TL_WARM_LAYERS - 1;
    __nv_bfloat16 *out = last ? nullptr : bufs[l & 1];
    rc = tl_conv_forward(in, ws->w[l], ws->b[l], nullptr, nullptr, out, last ? ws->g : nullptr, 1, g.ny, g.nx,
                         TL_WARM_CIN[l], TL_WARM_COUT[l], last ? 0 : 1, st);
    if (rc) {
      tl_set_error(ctx, "warm-start convolution %d failed to launch", l);
      return -rc;
    }
    in = out;
  }
  ctx->launches += 1 + TL_WARM_LAYERS;
  return 0;
}

// Solves the m x m Gram system G c = h (symmetric, positive semi-definite)
// on the host: the basis is scaled to unit A-norm, the scaled matrix is
// diagonalised by cyclic Jacobi rotations, and directions whose eigenvalue is
// below 1e-12 of the largest are dropped (nearly dependent increments).
// Returns 0 when no usable solution exists.
static int solve_dense(int m, const double *G, const double *h, double *c);

// The same on the basis slots listed in `slot` (the rows and columns of the
// full PROJ_MAX x PROJ_MAX system in use); c is zero on the other slots.
static int solve_gram(int m, const int *slot, const double *G, const double *h, double *c) {
  double Gl[PROJ_MAX * PROJ_MAX], hl[PROJ_MAX], cl[PROJ_MAX];
  for (int a = 0; a < m; ++a) {
    hl[a] = h[slot[a]];
    for (int b = 0; b < m; ++b) Gl[a * PROJ_MAX + b] = G[slot[a] * PROJ_MAX + slot[b]];
  }
  for (int a = 0; a < PROJ_MAX; ++a) c[a] = 0.0;
  if (!solve_dense(m, Gl, hl, cl)) return 0;
  for (int a = 0; a < m; ++a) c[slot[a]] = cl[a];
  return 1;
}

static int solve_dense(int m, const double *G, const double *h, double *c) {
  double S[PROJ_MAX][PROJ_MAX], Q[PROJ_MAX][PROJ_MAX], sc[PROJ_MAX], hs[PROJ_MAX];
  for (int a = 0; a < m; ++a) {
    if (!(G[a * PROJ_MAX + a] > 0) || !std::isfinite(G[a * PROJ_MAX + a])) return 0;
    sc[a] = 1.0 / std::sqrt(G[a * PROJ_MAX + a]);
  }
  for (int a = 0; a < m; ++a) {
    hs[a] = sc[a] * h[a];
    for (int b = 0; b < m; ++b) {
      S[a][b] = sc[a] * G[a * PROJ_MAX + b] * sc[b];
      Q[a][b] = a == b ? 1.0 : 0.0;
    }
  }
  for (int sweep = 0; sweep < 64; ++sweep) {
    double off = 0.0;
    for (int a = 0; a < m; ++a)
      for (int b = a + 1; b < m; ++b) off += S[a][b] * S[a][b];
    if (off < 1e-30) break;
    for (int p = 0; p < m; ++p)
      for (int q = p + 1; q < m; ++q) {
        if (std::fabs(S[p][q]) < 1e-300) continue;
        const double theta = 0.5 * (S[q][q] - S[p][p]) / S[p][q];
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double cs = 1.0 / std::sqrt(t * t + 1.0), sn = t * cs;
        for (int k = 0; k < m; ++k) {  // columns p, q of S
          const double skp = S[k][p], skq = S[k][q];
          S[k][p] = cs * skp - sn * skq;
          S[k][q] = sn * skp + cs * skq;
        }
        for (int k = 0; k < m; ++k) {  // rows p, q
          const double spk = S[p][k], sqk = S[q][k];
          S[p][k] = cs * spk - sn * sqk;
          S[q][k] = sn * spk + cs * sqk;
        }
        for (int k = 0; k < m; ++k) {
          const double qkp = Q[k][p], qkq = Q[k][q];
          Q[k][p] = cs * qkp - sn * qkq;
          Q[k][q] = sn * qkp + cs * qkq;
        }
      }
  }
  double lmax = 0.0;
  for (int a = 0; a < m; ++a) lmax = std::fmax(lmax, S[a][a]);
  if (!(lmax > 0) || !std::isfinite(lmax)) return 0;
  double y[PROJ_MAX] = {};
  for (int e = 0; e < m; ++e) {
    const double lam = S[e][e];
    if (!(lam > 1e-12 * lmax)) continue;
    double qh = 0.0;
    for (int a = 0; a < m; ++a) qh += Q[a][e] * hs[a];
    for (int a = 0; a < m; ++a) y[a] += Q[a][e] * qh / lam;
  }
  for (int a = 0; a < m; ++a) {
    c[a] = sc[a] * y[a];
    if (!std::isfinite(c[a])) return 0;
  }
  return 1;
}

// x = V c into ub, its halo, and ||u0 - A x||^2 (with `write`, the residual
// itself into w for accept_candidate).
static int candidate_residual(tl_ctx *ctx, const ProjBasis &B, const ProjCoef &C, int write, double *rr) {
  const Geom &g = ctx->g;
  const Fields &F = ctx->F;
  cudaStream_t st = ctx->stream;
  k_warm_combine<<<grid_cells(g), 256, 0, st>>>(F, g, B, C);
  CKL();
  double *ub = F.ub;
  launch_halo(st, &ub, 1, g, 1, TL_MODE_TEALEAF);
  CKL();
  OpWarmResid op;
  op.F = F;
  op.g = g;
  op.write = write;
  launch_walk<1>(st, op, ctx->walk_exact, g.ny);
  CKL();
  ctx->launches += 3;
  int rc = tl_read_scalars(ctx);
  if (rc) return rc;
  *rr = ctx->host_sc->red[0];
  return TL_OK;
}

// The candidate in ub (its residual in w) becomes the start: u = ub,
// r = p = w, rr = its r.r, and the halo of u, p.
static int accept_candidate(tl_ctx *ctx) {
  const Geom &g = ctx->g;
  const Fields &F = ctx->F;
  cudaStream_t st = ctx->stream;
  launch_copy_full(st, F.u, F.ub, g);
  k_warm_accept<<<grid_cells(g), 256, 0, st>>>(F, g);
  CKL();
  const int up[2] = {TL_EX_U, TL_EX_P};
  int rc = tl_halo_update(ctx, 1, up, 2, 1);
  if (rc) return rc;
  ctx->launches += 3;
  return TL_OK;
}

// Called by the CG solves after tea_leaf_init, the halo and copyu!.
int tl_warm_try(tl_ctx *ctx, double rx, double ry, int warmstart, tl_result *res) {
  if (warmstart != TL_WARM_NETWORK && warmstart != TL_WARM_EXTRAPOLATE && warmstart != TL_WARM_HISTORY) {
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
  const int network = warmstart == TL_WARM_NETWORK;
  if (network && !ws->wbuf) {
    tl_set_error(ctx, "warm start asked before tl_warm_load");
    return TL_ERR_STATE;
  }
  int rc = ensure_warm_buffers(ctx, network);
  if (rc) return rc;
  const Geom &g = ctx->g;
  const Fields &F = ctx->F;
  cudaStream_t st = ctx->stream;
  if ((rc = tl_read_scalars(ctx))) return rc;
  const double bb = ctx->host_sc->bb, rr_plain = ctx->host_sc->rro;
  res->r0_plain = bb > 0 ? sqrt(rr_plain / bb) : sqrt(rr_plain);
  res->r0_pred = -1.0;
  res->warm = 0;
  for (int a = 0; a < TL_WARM_HIST + 2; ++a) res->warm_coef[a] = 0.0;
  if (ws->nhist >= 1 && warmstart == TL_WARM_EXTRAPOLATE) {
    k_warm_extrapolate<<<grid_cells(g), 256, 0, st>>>(F, g, ws->hist[0]);
    CKL();
    ctx->launches += 1;
    res->warm_coef[0] = 2.0;
    res->warm_coef[1] = -1.0;
  } else if (ws->nhist >= 1) {
    ProjBasis B;
    B.u0 = F.u0;
    for (int q = 0; q < TL_WARM_HIST; ++q) B.h[q] = ws->hist[q];
    B.nh = ws->nhist;
    B.gv = nullptr;
    if (network && ws->net_skip > 0) {
      --ws->net_skip;  // backing off after the network's term lost its judge
    } else if (network) {
      const int nrc = run_network(ctx, rx, ry);
      if (nrc < 0) return -nrc;
      if (nrc == 0) B.gv = ws->g;
    }
    k_warm_gram<<<GRAM_BLOCKS, 256, 0, st>>>(F, g, B, ws->gram);
    k_warm_gram_fold<<<1, 64, 0, st>>>(ws->gram, GRAM_BLOCKS);
    CKL();
    ctx->launches += 2;
    double tot[PROJ_NACC];
    CK(cudaMemcpyAsync(tot, ws->gram + (size_t)GRAM_BLOCKS * PROJ_NACC, sizeof tot, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    double G[PROJ_MAX * PROJ_MAX] = {}, h[PROJ_MAX] = {};
    for (int a = 0, t = 0; a < PROJ_MAX; ++a)
      for (int b = a; b < PROJ_MAX; ++b, ++t) G[a * PROJ_MAX + b] = G[b * PROJ_MAX + a] = tot[t];
    for (int a = 0; a < PROJ_MAX; ++a) h[a] = tot[PROJ_NG + a];
    // the history-only projection (slots 0..nh), and with the network the
    // full one; the network's term is kept only when its candidate's
    // residual is below the history-only candidate's
    int slot[PROJ_MAX];
    const int mh = 1 + B.nh;
    for (int q = 0; q < mh; ++q) slot[q] = q;
    slot[mh] = PROJ_NET;
    ProjCoef Ch{}, Cn{};
    const int okh = solve_gram(mh, slot, G, h, Ch.c);
    const int okn = B.gv ? solve_gram(mh + 1, slot, G, h, Cn.c) : 0;
    const ProjCoef *chosen = nullptr;
    if (okh && okn) {
      double rr_h = 0.0, rr_n = 0.0;
      if ((rc = candidate_residual(ctx, B, Ch, 0, &rr_h))) return rc;
      if ((rc = candidate_residual(ctx, B, Cn, 0, &rr_n))) return rc;
      if (rr_n < rr_h) {
        chosen = &Cn;
        res->warm = 1;
        ws->net_backoff = 1;
      } else {
        // the network's term did not pay: skip the next 1, 2, 4, ... 32 inferences
        chosen = &Ch;
        res->warm = 3;
        ws->net_skip = ws->net_backoff;
        ws->net_backoff = ws->net_backoff < 32 ? 2 * ws->net_backoff : 32;
      }
    } else if (okh) {
      chosen = &Ch;
      res->warm = network ? 3 : 1;
    }
    if (chosen) {
      double rr_pred = 0.0;
      if ((rc = candidate_residual(ctx, B, *chosen, 1, &rr_pred))) return rc;
      // weights on u^n, u^{n-1}, ...: x = c0 u^n + sum_j c_j (u^{n-j+1} - u^{n-j}) + c_net t
      const double *cc = chosen->c;
      res->warm_coef[0] = cc[0] + cc[1];
      for (int q = 1; q <= B.nh; ++q) res->warm_coef[q] = (q < B.nh ? cc[q + 1] : 0.0) - cc[q];
      res->warm_coef[TL_WARM_HIST + 1] = cc[PROJ_NET];
      res->r0_pred = bb > 0 ? sqrt(rr_pred / bb) : sqrt(rr_pred);
      if (rr_pred < rr_plain) {
        if ((rc = accept_candidate(ctx))) return rc;
      } else {
        res->warm = 2;
      }
    }
  }
  if (warmstart == TL_WARM_EXTRAPOLATE && ws->nhist >= 1) {
    double *ub = F.ub;
    launch_halo(st, &ub, 1, g, 1, TL_MODE_TEALEAF);
    CKL();
    OpWarmResid op;
    op.F = F;
    op.g = g;
    op.write = 1;
    launch_walk<1>(st, op, ctx->walk_exact, g.ny);
    CKL();
    ctx->launches += 2;
    if ((rc = tl_read_scalars(ctx))) return rc;
    const double rr_pred = ctx->host_sc->red[0];
    res->r0_pred = bb > 0 ? sqrt(rr_pred / bb) : sqrt(rr_pred);
    if (rr_pred < rr_plain) {
      if ((rc = accept_candidate(ctx))) return rc;
      res->warm = 1;
    } else {
      res->warm = 2;
    }
  }
  // keep u^n as the newest earlier solution for the next step
  double *oldest = ws->hist[TL_WARM_HIST - 1];
  for (int q = TL_WARM_HIST - 1; q > 0; --q) ws->hist[q] = ws->hist[q - 1];
  ws->hist[0] = oldest;
  k_copy_u0<<<grid_cells(g), 256, 0, st>>>(F, g, ws->hist[0]);
  CKL();
  ctx->launches += 1;
  ws->nhist = ws->nhist < TL_WARM_HIST ? ws->nhist + 1 : TL_WARM_HIST;
  return TL_OK;
}
