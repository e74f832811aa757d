// tl_ir_ops.cuh -- the FP32 iteration kernels of the refinement path and
// their FP64 refinement steps, shared by the single-deck solve (tl_ir.cu) and
// the batched solve (tl_batch.cu).
//
// The inner iteration is CG on FP32 vectors (p, r, w and the correction x)
// with FP32 Kx/Ky; each dot sums a lane's four products in FP32 and
// accumulates those partial sums in FP64.  FP32 arrays are pitched like the
// FP64 fields, 32 floats per pitch unit, first interior cell of each row
// 128-byte aligned; each lane owns 4 consecutive cells (one float4).
#pragma once

#include "tl_solvers.h"
#include "tl_walk.cuh"

struct tl_ir_state {
  float *buf = nullptr;
  long long pitch = 0, lead = 0, stride = 0;
  float *kx = nullptr, *ky = nullptr, *p = nullptr, *pb = nullptr, *r = nullptr, *w = nullptr, *x = nullptr;
  float *sd = nullptr, *sdb = nullptr;  // PPCG inner sweeps: the update and its second buffer
  tl::Walk walk_w{}, walk_ur{};  // autotuned layouts of the two FP32 kernels
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // p in the first / second buffer
  cudaGraphExec_t ppcg_graph[2] = {nullptr, nullptr};
  int ppcg_inner = -1;  // inner sweeps recorded in ppcg_graph
  int pwhich = 0;       // after a CG loop: 1 when the search direction is in pb
};

namespace tl {
namespace {

constexpr double IR_DELTA = 0.1;  // refine when ||r32|| < delta * ||r at the last refinement||

struct G32 {
  int nx, ny, hd, X, Y;
  long long pitch;
  __host__ __device__ __forceinline__ size_t at(int i, int j) const {
    return (size_t)(hd + i) + (size_t)(hd + j) * (size_t)pitch;
  }
};

struct IrPtrs {
  float *kx, *ky, *r, *w, *x;
};

__device__ __forceinline__ float4 ld4(const float *p) { return __ldg(reinterpret_cast<const float4 *>(p)); }
__device__ __forceinline__ void st4(float *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }
__device__ __forceinline__ float comp(const float4 &v, int k) { return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w; }

// Walk with four cells per lane: tile = 128*warps columns x rows.
template <class Op>
__global__ void __launch_bounds__(256) k_walk32(const Op op, const Walk wk, const int ny) {
  if (op.skip()) {
    op.on_skip();
    return;
  }
  double acc[1] = {0.0};
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int TW = 128 * wk.warps;
  for (int t = blockIdx.x; t < wk.tiles; t += gridDim.x) {
    const int tx = t % wk.ntx, ty = t / wk.ntx;
    const int i0 = tx * TW + warp * 128 + 4 * lane;
    const int j0 = ty * wk.rows;
    const int j1 = min(j0 + wk.rows, ny);
    op.tile(i0, j0, j1, acc);
  }
  if (Op::REDUCES) finish_reduction<1>(acc, op);
}

// W step: p' = beta*p + r (or p on the first step), w = A32 p', p'.w
struct OpIrW {
  static constexpr bool REDUCES = true;
  Fields F;  // scalars, partials, counter
  G32 g;
  IrPtrs q;
  const float *__restrict__ psrc;
  float *__restrict__ pdst;
  int guard;
  __device__ bool skip() const { return guard && F.sc->done; }
  __device__ void on_skip() const {}

  // Raw loads of one row, issued one row ahead of their use.
  struct Row {
    float4 p, r, kx;
    float ep, er, kxe;  // edge neighbour (lane 0: i0-1, lane 31: i0+4) and kx at i0+4
  };
  __device__ __forceinline__ void load_row(Row &o, int i0, int j, bool valid, bool first, int edge_col) const {
    if (!valid) return;
    const size_t c = g.at(i0, j);
    o.p = ld4(psrc + c);
    if (!first) o.r = ld4(q.r + c);
    if (edge_col >= 0) {
      const size_t e = g.at(edge_col, j);
      o.ep = __ldg(psrc + e);
      if (!first) o.er = __ldg(q.r + e);
    }
  }
  __device__ __forceinline__ void load_coef(Row &o, int i0, int j, bool valid, bool kx_edge) const {
    if (!valid) return;
    const size_t c = g.at(i0, j);
    o.kx = ld4(q.kx + c);
    if (kx_edge) o.kxe = __ldg(q.kx + c + 4);
  }

  __device__ void tile(int i0, int j0, int j1, double (&acc)[1]) const {
    const int nx = g.nx, ny = g.ny;
    const int lane = threadIdx.x & 31;
    const bool valid = i0 < nx;
    const int ncell = valid ? min(4, nx - i0) : 0;  // cells this lane owns
    const bool full = ncell == 4;
    const bool inner = i0 + 4 < nx;                 // the fourth cell has an interior east neighbour
    const float beta = (float)F.sc->beta;
    const bool first = F.sc->first != 0;
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    const int edge_col = !valid ? -1 : (lane == 0 && i0 > 0) ? i0 - 1 : (lane == 31 && inner) ? i0 + 4 : -1;
    const bool kx_edge = full && (!inner || lane == 31);
    auto pnew = [&](const Row &o) {
      return first ? o.p
                   : make_float4(fmaf(beta, o.p.x, o.r.x), fmaf(beta, o.p.y, o.r.y), fmaf(beta, o.p.z, o.r.z),
                                 fmaf(beta, o.p.w, o.r.w));
    };
    auto pnew_edge = [&](const Row &o) { return first ? o.ep : fmaf(beta, o.ep, o.er); };

    Row cur = {}, nxt = {}, tmp = {};
    load_row(cur, i0, j0, valid, first, edge_col);
    load_coef(cur, i0, j0, valid, kx_edge);
    if (j0 > 0) load_row(tmp, i0, j0 - 1, valid, first, -1);
    if (j0 + 1 < ny) load_row(nxt, i0, j0 + 1, valid, first, edge_col);
    float4 kyc = valid ? ld4(q.ky + g.at(i0, j0)) : z;
    float4 kyn = valid ? ld4(q.ky + g.at(i0, j0 + 1)) : z;
    float4 pc = valid ? pnew(cur) : z;
    float4 ps = (j0 > 0 && valid) ? pnew(tmp) : pc;
    for (int j = j0; j < j1; ++j) {
      Row nn = {};
      float4 kyn2 = z;
      if (j + 1 < j1) {
        if (j + 2 < ny) load_row(nn, i0, j + 2, valid, first, edge_col);
        load_coef(nxt, i0, j + 1, valid, kx_edge);
        kyn2 = valid ? ld4(q.ky + g.at(i0, j + 2)) : z;
      }
      const float4 pnn = (j + 1 < ny && valid) ? pnew(nxt) : pc;
      float pw = __shfl_up_sync(FULL, pc.w, 1);
      float pe = __shfl_down_sync(FULL, pc.x, 1);
      float kxe = __shfl_down_sync(FULL, cur.kx.x, 1);
      if (valid) {
        if (i0 == 0) pw = pc.x;
        else if (lane == 0) pw = pnew_edge(cur);
        if (full) {
          if (!inner) {
            pe = pc.w;        // reflect at i = nx-1
            kxe = cur.kxe;    // kx of the halo column
          } else if (lane == 31) {
            pe = pnew_edge(cur);
            kxe = cur.kxe;
          }
        }
        float wv[4];
        float part = 0.f;  // this lane's four products, summed in FP32 before the FP64 accumulation
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          if (k < ncell) {
            const float c = comp(pc, k);
            const float e = (k + 1 < ncell) ? comp(pc, k + 1) : (k == 3 ? pe : c);  // reflect past nx-1
            const float wl = (k == 0) ? pw : comp(pc, k - 1);
            const float k1 = (k == 3) ? kxe : comp(cur.kx, k + 1);
            const float k0 = comp(cur.kx, k);
            const float n = comp(pnn, k), sv = comp(ps, k);
            float t = c;
            t = fmaf(k1, c - e, t);
            t = fmaf(k0, c - wl, t);
            t = fmaf(comp(kyn, k), c - n, t);
            t = fmaf(comp(kyc, k), c - sv, t);
            wv[k] = t;
            part = fmaf(t, c, part);
          } else {
            wv[k] = 0.f;
          }
        }
        acc[0] += (double)part;
        const size_t c0 = g.at(i0, j);
        if (full) {
          st4(q.w + c0, make_float4(wv[0], wv[1], wv[2], wv[3]));
          st4(pdst + c0, pc);
        } else {
          for (int k = 0; k < ncell; ++k) {
            q.w[c0 + k] = wv[k];
            pdst[c0 + k] = comp(pc, k);
          }
        }
      }
      ps = pc;
      pc = pnn;
      kyc = kyn;
      kyn = kyn2;
      cur = nxt;
      nxt = nn;
    }
  }
  __device__ void fin(const double *tot) const {
    DevScalars *sc = F.sc;
    sc->pw = tot[0];
    sc->alpha = sc->rro / sc->pw;
    // as CG presteps of Chebyshev, the coefficient table for the eigenvalue
    // estimate (CG.jl:37; 1-based, maxiters + 2 entries)
    if (sc->switch_rule == 1 && sc->iter < sc->maxiters) F.cgalpha[sc->iter + 1] = sc->alpha;
  }
};

// UR step: x += alpha p', r -= alpha w, r.r; the epilogue decides whether the
// next step is another FP32 iteration or a refinement.
struct OpIrUR {
  static constexpr bool REDUCES = true;
  Fields F;
  G32 g;
  IrPtrs q;
  const float *__restrict__ p;
  int guard;
  cudaGraphConditionalHandle cond;
  int set_cond;
  __device__ bool skip() const { return guard && F.sc->done; }
  __device__ void on_skip() const {
    if (set_cond && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(cond, 0u);
  }
  __device__ void tile(int i0, int j0, int j1, double (&acc)[1]) const {
    if (i0 >= g.nx) return;
    const int ncell = min(4, g.nx - i0);
    const float alpha = (float)F.sc->alpha;
    double a = acc[0];
    for (int j = j0; j < j1; ++j) {
      const size_t c = g.at(i0, j);
      if (ncell == 4) {
        const float4 pv = ld4(p + c), wv = ld4(q.w + c);
        float4 xv = ld4(q.x + c), rv = ld4(q.r + c);
        xv.x = fmaf(alpha, pv.x, xv.x); xv.y = fmaf(alpha, pv.y, xv.y);
        xv.z = fmaf(alpha, pv.z, xv.z); xv.w = fmaf(alpha, pv.w, xv.w);
        rv.x = fmaf(-alpha, wv.x, rv.x); rv.y = fmaf(-alpha, wv.y, rv.y);
        rv.z = fmaf(-alpha, wv.z, rv.z); rv.w = fmaf(-alpha, wv.w, rv.w);
        a += (double)fmaf(rv.w, rv.w, fmaf(rv.z, rv.z, fmaf(rv.y, rv.y, rv.x * rv.x)));
        st4(q.x + c, xv);
        st4(q.r + c, rv);
      } else {
        for (int k = 0; k < ncell; ++k) {
          const float xv = fmaf(alpha, p[c + k], q.x[c + k]);
          const float rv = fmaf(-alpha, q.w[c + k], q.r[c + k]);
          q.x[c + k] = xv;
          q.r[c + k] = rv;
          a = fma((double)rv, (double)rv, a);
        }
      }
    }
    acc[0] = a;
  }
  __device__ void fin(const double *tot) const {
    DevScalars *sc = F.sc;
    const double rrn = tot[0];
    sc->beta = rrn / sc->rro;
    bool sw = false;
    if (sc->switch_rule == 1) {
      // CG presteps of Chebyshev: the beta table and the switch test
      // (Cheby.jl:25-29) on this step's r.r
      if (sc->iter < sc->maxiters) F.cgbeta[sc->iter + 1] = sc->beta;
      const int tt = sc->iter + 2;  // the solver loop's next trip
      sw = sc->errorswitch ? (rrn < sc->epslim && tt > CGEIGENITERS) : (tt > sc->presteps && rrn < ERROR_SWITCH_MAX);
    }
    sc->rro = rrn;
    sc->error = rrn;
    sc->iter += 1;
    sc->first = 0;
    const bool claim = sqrt(rrn / sc->bb) < sc->eps;
    const bool refine = claim || rrn < sc->delta2 * sc->rr_ref;
    sc->converged = 0;
    sc->switched = refine;
    sc->prestep_switch = sw;
    const int done = refine || sw || sc->iter >= sc->maxiters;
    sc->done = done;
    if (set_cond) cudaGraphSetConditional(cond, done ? 0u : 1u);
  }
};

// Refinement: u += x, x = 0 on the interior.
__global__ void k_ir_fold(Fields F, Geom g, G32 g32, float *x) {
  const long long n = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(k % g.nx), j = (int)(k / g.nx);
    const size_t c = g.at(i, j), c32 = g32.at(i, j);
    F.u[c] = F.u[c] + (double)x[c32];
    x[c32] = 0.f;
  }
}

// Refinement: r = u0 - A u in FP64 (reference operation order, u's halo read
// from memory), r32 = (float) r, sum r^2.
struct OpIrResid : NoSkip {
  Fields F;
  Geom g;
  G32 g32;
  float *r32;
  __device__ void cell(int i, int j, double (&acc)[1]) const {
    const size_t c = g.at(i, j);
    const double kxr = F.kx[c + 1], kxc = F.kx[c], kyt = F.ky[c + g.pitch], kyc = F.ky[c];
    const double *a = F.u;
    const double consum = tl::dadd(tl::dadd(tl::dadd(tl::dadd(1.0, kxr), kxc), kyt), kyc);
    double v = tl::dmul(consum, a[c]);
    v = tl::dsub(v, tl::dadd(tl::dmul(kxr, a[c + 1]), tl::dmul(kxc, a[c - 1])));
    v = tl::dsub(v, tl::dadd(tl::dmul(kyt, a[c + g.pitch]), tl::dmul(kyc, a[c - g.pitch])));
    const double t = tl::dsub(F.u0[c], v);
    F.r[c] = t;
    r32[g32.at(i, j)] = (float)t;
    acc[0] = tl::dadd(acc[0], tl::dmul(t, t));
  }
  __device__ void tile(int i0, int j0, int j1, double (&acc)[1]) const {
    for (int j = j0; j < j1; ++j) {
      if (i0 < g.nx) cell(i0, j, acc);
      if (i0 + 1 < g.nx) cell(i0 + 1, j, acc);
    }
  }
  __device__ void fin(const double *tot) const { F.sc->red[0] = tot[0]; }
};

// FP32 copies of kx, ky (whole arrays, halo included); p32 = r32 = (float) r
// and x = 0 on the interior.
__global__ void k_ir_convert(Fields F, Geom g, G32 g32, float *kx, float *ky, float *r, float *p, float *x) {
  const long long n = (long long)g.X * g.Y;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int I = (int)(k % g.X), J = (int)(k / g.X);
    const size_t c = (size_t)I + (size_t)J * g.pitch, c32 = (size_t)I + (size_t)J * g32.pitch;
    kx[c32] = (float)F.kx[c];
    ky[c32] = (float)F.ky[c];
    const bool interior = I >= g.hd && I < g.X - g.hd && J >= g.hd && J < g.Y - g.hd;
    const float rv = interior ? (float)F.r[c] : 0.f;
    r[c32] = rv;
    p[c32] = rv;
    x[c32] = 0.f;
  }
}

// p (FP64) = (double) p32 on the interior: the last search direction.
__global__ void k_ir_export_p(Fields F, Geom g, G32 g32, const float *p32) {
  const long long n = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(k % g.nx), j = (int)(k / g.nx);
    F.p[g.at(i, j)] = (double)p32[g32.at(i, j)];
  }
}

__global__ void k_ir_start(DevScalars *sc, double rr, double delta2) {
  sc->rro = rr;
  sc->rr_ref = rr;
  sc->delta2 = delta2;
  sc->done = 0;
  sc->switched = 0;
  sc->prestep_switch = 0;
}

G32 g32_of(tl_ctx *ctx) {
  G32 g;
  g.nx = ctx->g.nx;
  g.ny = ctx->g.ny;
  g.hd = ctx->g.hd;
  g.X = ctx->g.X;
  g.Y = ctx->g.Y;
  g.pitch = ctx->ir->pitch;
  return g;
}

IrPtrs ptrs_of(tl_ctx *ctx) {
  IrPtrs q;
  q.kx = ctx->ir->kx;
  q.ky = ctx->ir->ky;
  q.r = ctx->ir->r;
  q.w = ctx->ir->w;
  q.x = ctx->ir->x;
  return q;
}

}  // namespace
}  // namespace tl
