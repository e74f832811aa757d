// tl_ir_ops.cuh -- the FP32 iteration kernels of the refinement path and
// their FP64 refinement steps, shared by the single-deck solve (tl_ir.cu) and
// the batched solve (tl_batch.cu).
//
// The inner iteration is CG on FP32 vectors (p, r and the correction x) with
// the stencil faces formed from FP32 inverse weights; each dot sums a lane's
// products over eight rows (32 cells) in FP32 and accumulates those partial
// sums in FP64.  FP32 arrays are pitched like the
// FP64 fields, 32 floats per pitch unit, first interior cell of each row
// 128-byte aligned; each lane owns 4 consecutive cells (one float4).
#pragma once

#include "tl_solvers.h"
#include "tl_walk.cuh"

struct tl_ir_state {
  float *buf = nullptr;
  long long pitch = 0, lead = 0, stride = 0;
  float *p = nullptr, *pb = nullptr, *r = nullptr, *x = nullptr;
  float *sd = nullptr, *sdb = nullptr;  // PPCG inner sweeps: the update and its second buffer
  float *iw = nullptr;                  // 1 / w (w = rho or 1/rho, CG.jl:57-60), halo included
  tl::Walk walk_dir{};              // autotuned layout of OpIrDir
  tl::Walk walk_sweep[4]{};         // autotuned layouts of OpIrSweep, by kind (the last inner sweep shares slot 3)
  int dir_ahead = 2;                // the faster OpIrDir form after tuning (its AHEAD)
  int sweep_ahead[4] = {1, 1, 1, 1};
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
  float *r, *x;
  float *iw;  // inverse weights: Kx = rx/2 (iw_l + iw_c), Ky = ry/2 (iw_d + iw_c)
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

// The epilogue of an FP32 CG step (OpIrUpdate): beta, the iteration
// count, the refinement test and, as CG presteps of Chebyshev or PPCG, the
// coefficient table and the switch test.
__device__ __forceinline__ void ir_cg_epilogue(const Fields &F, double rrn, cudaGraphConditionalHandle cond,
                                             int set_cond) {
  DevScalars *sc = F.sc;
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

// ---- the 40-byte CG step pair ----------------------------------------------
// OpIrDir forms p' = beta p + r and p'.A p' and stores p' (reads p, r, iw:
// 16 B per cell with the store); OpIrUpdate recomputes w = A p' from the
// stored p' and does x += alpha p', r -= alpha w, r.r (reads p', iw, x, r,
// writes x, r: 24 B).  Neither w nor Kx, Ky is stored (a pair that stored
// them would move 48 B): the faces come from the inverse weights,
// Kx = rx/2 (iw_l + iw_c).
// Both kernels evaluate the stencil with the same function on the same
// floats, so the w of the update equals the w of the dot bit for bit.

// The five-point neighbourhood of a lane's four cells, after the reflective
// boundary has been applied (west/east: the edge values beyond the lane's
// cells; s/n: the rows below and above).
struct Hood4 {
  float4 c, s, n;
  float w, e;
};

__device__ __forceinline__ void stencil4(const Hood4 &p, const Hood4 &iw, float rxh, float ryh, int ncell,
                                         float (&out)[4]) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    out[k] = 0.f;
    if (k < ncell) {
      const float c = comp(p.c, k), ic = comp(iw.c, k);
      const bool last = k + 1 == ncell;
      const float e = last ? (k == 3 ? p.e : c) : comp(p.c, k + 1);
      const float ie = last ? (k == 3 ? iw.e : ic) : comp(iw.c, k + 1);
      const float wl = k == 0 ? p.w : comp(p.c, k - 1);
      const float il = k == 0 ? iw.w : comp(iw.c, k - 1);
      float t = c;
      t = fmaf(rxh * (ic + ie), c - e, t);
      t = fmaf(rxh * (ic + il), c - wl, t);
      t = fmaf(ryh * (ic + comp(iw.n, k)), c - comp(p.n, k), t);
      t = fmaf(ryh * (ic + comp(iw.s, k)), c - comp(p.s, k), t);
      out[k] = t;
    }
  }
}

// The west/east edge values of a lane's four cells from a row's float4s:
// neighbours by shuffle, lane 0 / lane 31 from their own edge loads, and the
// reflection at the domain boundary (the cell itself).
__device__ __forceinline__ void edges4(float4 v, float wload, float eload, int i0, int lane, bool full, bool inner,
                                       float &w, float &e) {
  w = __shfl_up_sync(FULL, v.w, 1);
  e = __shfl_down_sync(FULL, v.x, 1);
  if (i0 == 0) w = v.x;
  else if (lane == 0) w = wload;
  if (full) {
    if (!inner) e = v.w;
    else if (lane == 31) e = eload;
  }
}

// p' = beta p + r (p on the first step), p'.A p'; stores p'.  AHEAD: rows
// loaded two rows ahead of their use (2) or as they are reached (1).
template <int AHEAD>
struct OpIrDir {
  static constexpr bool REDUCES = true;
  Fields F;
  G32 g;
  IrPtrs q;
  const float *__restrict__ psrc;
  float *__restrict__ pdst;
  int guard;
  __device__ bool skip() const { return guard && F.sc->done; }
  __device__ void on_skip() const {}

  struct Row {
    float4 p, r, iw;
    float pw, rw, pe, re, iww, iwe;  // edge loads (lane 0: i0-1, lane 31: i0+4)
  };
  __device__ __forceinline__ void load_row(Row &o, int i0, int j, bool valid, bool first, int lane,
                                           bool inner) const {
    if (!valid) return;
    const size_t c = g.at(i0, j);
    o.p = ld4(psrc + c);
    o.iw = ld4(q.iw + c);
    if (!first) o.r = ld4(q.r + c);
    if (lane == 0 && i0 > 0) {
      o.pw = __ldg(psrc + c - 1);
      o.iww = __ldg(q.iw + c - 1);
      if (!first) o.rw = __ldg(q.r + c - 1);
    }
    if (lane == 31 && inner) {
      o.pe = __ldg(psrc + c + 4);
      o.iwe = __ldg(q.iw + c + 4);
      if (!first) o.re = __ldg(q.r + c + 4);
    }
  }

  __device__ void tile(int i0, int j0, int j1, double (&acc)[1]) const {
    const int nx = g.nx, ny = g.ny;
    const int lane = threadIdx.x & 31;
    const bool valid = i0 < nx;
    const int ncell = valid ? min(4, nx - i0) : 0;
    const bool full = ncell == 4;
    const bool inner = i0 + 4 < nx;
    const float beta = (float)F.sc->beta;
    const float rxh = (float)F.sc->rxh, ryh = (float)F.sc->ryh;
    const bool first = F.sc->first != 0;
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    auto pnew = [&](const Row &o) {
      return first ? o.p
                   : make_float4(fmaf(beta, o.p.x, o.r.x), fmaf(beta, o.p.y, o.r.y), fmaf(beta, o.p.z, o.r.z),
                                 fmaf(beta, o.p.w, o.r.w));
    };
    Row cur = {}, nxt = {}, sth = {};
    load_row(cur, i0, j0, valid, first, lane, inner);
    if (j0 > 0) load_row(sth, i0, j0 - 1, valid, first, -1, inner);
    if (AHEAD == 2 && j0 + 1 < ny) load_row(nxt, i0, j0 + 1, valid, first, lane, inner);
    float4 pc = valid ? pnew(cur) : z;
    float4 ps = (j0 > 0 && valid) ? pnew(sth) : pc;
    float4 is = (j0 > 0 && valid) ? sth.iw : cur.iw;
    float fpart = 0.f;
    int nrow = 0;
    for (int j = j0; j < j1; ++j) {
      Row nn = {};
      if (AHEAD == 2) {
        if (j + 1 < j1 && j + 2 < ny) load_row(nn, i0, j + 2, valid, first, lane, inner);
      } else if (j + 1 < ny) {
        load_row(nxt, i0, j + 1, valid, first, lane, inner);
      }
      const bool has_n = j + 1 < ny;
      const float4 pn = (has_n && valid) ? pnew(nxt) : pc;
      const float4 in = has_n ? nxt.iw : cur.iw;
      Hood4 hp, hi;
      hp.c = pc; hp.s = ps; hp.n = pn;
      hi.c = cur.iw; hi.s = is; hi.n = in;
      const float pwl = first ? cur.pw : fmaf(beta, cur.pw, cur.rw);
      const float pel = first ? cur.pe : fmaf(beta, cur.pe, cur.re);
      edges4(pc, pwl, pel, i0, lane, full, inner, hp.w, hp.e);
      edges4(cur.iw, cur.iww, cur.iwe, i0, lane, full, inner, hi.w, hi.e);
      if (valid) {
        float wv[4];
        stencil4(hp, hi, rxh, ryh, ncell, wv);
        float part = 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (k < ncell) part = fmaf(wv[k], comp(pc, k), part);
        fpart += part;
        if (++nrow == 8) {  // eight rows of FP32 partials (32 products) per FP64 add
          acc[0] += (double)fpart;
          fpart = 0.f;
          nrow = 0;
        }
        const size_t c0 = g.at(i0, j);
        if (full) {
          st4(pdst + c0, pc);
        } else {
#pragma unroll
          for (int k = 0; k < 4; ++k)
            if (k < ncell) pdst[c0 + k] = comp(pc, k);
        }
      }
      ps = pc;
      pc = pn;
      is = cur.iw;
      cur = nxt;
      if (AHEAD == 2) nxt = nn;
    }
    acc[0] += (double)fpart;
  }
  __device__ void fin(const double *tot) const {
    DevScalars *sc = F.sc;
    sc->pw = tot[0];
    sc->alpha = sc->rro / sc->pw;
    if (sc->switch_rule == 1 && sc->iter < sc->maxiters) F.cgalpha[sc->iter + 1] = sc->alpha;
  }
};

// The sweep kernels: a five-point stencil w = A s on one FP32 field s (from
// the inverse weights) and an update of two own-cell operands (a, b), with
// up to three stores.  KIND:
//   SWEEP_CG          s = p', a = x, b = r:  x += alpha p', r -= alpha w, r.r
//                     (the FP32 CG update step; the epilogue decides between
//                     another step and a refinement)
//   SWEEP_PPCG_UPDATE s = p', a = x, b = r:  the same, then sd = r / theta
//                     (PPCG.jl:64-72), no reduction
//   SWEEP_CHEBY       s = e, a = r0, b = p:  r = r0 - w, p = alpha_k p + beta_k r,
//                     e' = e + p into `out`, r.r (one Chebyshev step on the
//                     correction of the current refinement)
//   SWEEP_PPCG_INNER  s = sd, a = r, b = x: r -= w, x += sd,
//                     sd' = alpha_pp sd + beta_pp r into `out` (one inner
//                     sweep, PPCG.jl:74-88); the last sweep (LAST) also sums
//                     r.r and closes the outer step
// AHEAD: the stencil rows are loaded two rows ahead of their use (2) or as
// the row is reached (1: fewer registers, more resident warps); a and b are
// loaded one row ahead in both.
enum { SWEEP_CG = 0, SWEEP_PPCG_UPDATE = 1, SWEEP_CHEBY = 2, SWEEP_PPCG_INNER = 3, SWEEP_PPCG_LAST = 4 };

template <int AHEAD, int KIND>
struct OpIrSweep {
  static constexpr bool REDUCES = KIND == SWEEP_CG || KIND == SWEEP_CHEBY || KIND == SWEEP_PPCG_LAST;
  static constexpr bool INNER = KIND == SWEEP_PPCG_INNER || KIND == SWEEP_PPCG_LAST;
  Fields F;
  G32 g;
  const float *__restrict__ s;   // the stencil field
  const float *__restrict__ iw;  // inverse weights
  float *__restrict__ a;         // own-cell operands (updated in place, except r0)
  float *__restrict__ b;
  float *__restrict__ out;       // sd (PPCG update), e' (Chebyshev), sd' (inner sweep)
  int pp;                        // inner sweep (1-based)
  int guard;
  cudaGraphConditionalHandle cond;
  int set_cond;
  __device__ bool skip() const { return guard && F.sc->done; }
  __device__ void on_skip() const {
    if (set_cond && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(cond, 0u);
  }

  struct Nb {  // the stencil operands of one row
    float4 s, iw;
    float sw, se, iww, iwe;
  };
  __device__ __forceinline__ void load_nb(Nb &o, int i0, int j, bool valid, int lane, bool inner) const {
    if (!valid) return;
    const size_t c = g.at(i0, j);
    o.s = ld4(s + c);
    o.iw = ld4(iw + c);
    if (lane == 0 && i0 > 0) {
      o.sw = __ldg(s + c - 1);
      o.iww = __ldg(iw + c - 1);
    }
    if (lane == 31 && inner) {
      o.se = __ldg(s + c + 4);
      o.iwe = __ldg(iw + c + 4);
    }
  }

  __device__ void tile(int i0, int j0, int j1, double (&acc)[1]) const {
    const int nx = g.nx, ny = g.ny;
    const int lane = threadIdx.x & 31;
    const bool valid = i0 < nx;
    const int ncell = valid ? min(4, nx - i0) : 0;
    const bool full = ncell == 4;
    const bool inner = i0 + 4 < nx;
    const DevScalars *sc = F.sc;
    const float rxh = (float)sc->rxh, ryh = (float)sc->ryh;
    float c0 = 0.f, c1 = 0.f;  // alpha (CG, PPCG update) / 1/theta; or the Chebyshev pair
    if (KIND == SWEEP_CG || KIND == SWEEP_PPCG_UPDATE) {
      c0 = (float)sc->alpha;
      c1 = (float)(1.0 / sc->theta);
    } else if (KIND == SWEEP_CHEBY) {
      const int idx = min(sc->cheby_iters + 2, sc->maxiters + 1);
      c0 = (float)F.chebyalpha[idx];
      c1 = (float)F.chebybeta[idx];
    } else {
      c0 = (float)F.chebyalpha[pp];
      c1 = (float)F.chebybeta[pp];
    }
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    auto ld = [&](const float *f, int j) { return valid ? ld4(f + g.at(i0, j)) : z; };
    Nb cur = {}, nxt = {};
    load_nb(cur, i0, j0, valid, lane, inner);
    float4 ac = ld(a, j0), bc = ld(b, j0);
    float4 ss = (j0 > 0 && valid) ? ld(s, j0 - 1) : cur.s;
    float4 is = (j0 > 0 && valid) ? ld(iw, j0 - 1) : cur.iw;
    if (AHEAD == 2 && j0 + 1 < ny) load_nb(nxt, i0, j0 + 1, valid, lane, inner);
    double racc = acc[0];
    float fpart = 0.f;
    int nrow = 0;
    for (int j = j0; j < j1; ++j) {
      Nb nn = {};
      if (AHEAD == 2) {
        if (j + 1 < j1 && j + 2 < ny) load_nb(nn, i0, j + 2, valid, lane, inner);
      } else if (j + 1 < ny) {
        load_nb(nxt, i0, j + 1, valid, lane, inner);
      }
      float4 an = z, bn = z;
      if (j + 1 < j1) {
        an = ld(a, j + 1);
        bn = ld(b, j + 1);
      }
      const bool has_n = j + 1 < ny;
      Hood4 hs, hi;
      hs.c = cur.s; hs.s = ss; hs.n = has_n ? nxt.s : cur.s;
      hi.c = cur.iw; hi.s = is; hi.n = has_n ? nxt.iw : cur.iw;
      edges4(cur.s, cur.sw, cur.se, i0, lane, full, inner, hs.w, hs.e);
      edges4(cur.iw, cur.iww, cur.iwe, i0, lane, full, inner, hi.w, hi.e);
      if (valid) {
        float wv[4];
        stencil4(hs, hi, rxh, ryh, ncell, wv);
        float va[4], vb[4], vo[4];
        float part = 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float sv = comp(cur.s, k), av = comp(ac, k), bv = comp(bc, k);
          float rr;
          if (KIND == SWEEP_CG || KIND == SWEEP_PPCG_UPDATE) {
            va[k] = fmaf(c0, sv, av);        // x + alpha p'
            vb[k] = fmaf(-c0, wv[k], bv);    // r - alpha w
            vo[k] = vb[k] * c1;              // sd = r / theta
            rr = vb[k];
          } else if (KIND == SWEEP_CHEBY) {
            const float r = av - wv[k];      // r0 - w
            vb[k] = fmaf(c0, bv, c1 * r);    // alpha_k p + beta_k r
            vo[k] = sv + vb[k];              // e + p
            va[k] = av;
            rr = r;
          } else {
            va[k] = av - wv[k];              // r - w
            vb[k] = bv + sv;                 // x + sd
            vo[k] = fmaf(c0, sv, c1 * va[k]);
            rr = va[k];
          }
          if (REDUCES && k < ncell) part = fmaf(rr, rr, part);
        }
        if (REDUCES) {
          fpart += part;
          if (++nrow == 8) {  // eight rows of FP32 partials (32 products) per FP64 add
            racc += (double)fpart;
            fpart = 0.f;
            nrow = 0;
          }
        }
        const size_t o = g.at(i0, j);
        const bool st_a = KIND != SWEEP_CHEBY, st_o = KIND != SWEEP_CG;
        if (full) {
          if (st_a) st4(a + o, make_float4(va[0], va[1], va[2], va[3]));
          st4(b + o, make_float4(vb[0], vb[1], vb[2], vb[3]));
          if (st_o) st4(out + o, make_float4(vo[0], vo[1], vo[2], vo[3]));
        } else {
#pragma unroll
          for (int k = 0; k < 4; ++k)
            if (k < ncell) {
              if (st_a) a[o + k] = va[k];
              b[o + k] = vb[k];
              if (st_o) out[o + k] = vo[k];
            }
        }
      }
      ss = cur.s;
      is = cur.iw;
      cur = nxt;
      if (AHEAD == 2) nxt = nn;
      ac = an;
      bc = bn;
    }
    if (REDUCES) racc += (double)fpart;
    acc[0] = racc;
  }
  __device__ void fin(const double *tot) const {
    if (KIND == SWEEP_CG) {
      ir_cg_epilogue(F, tot[0], cond, set_cond);
    } else if (KIND == SWEEP_CHEBY) {
      DevScalars *sc = F.sc;
      const double rr = tot[0];
      sc->cheby_iters += 1;
      sc->iter += 1;
      sc->error = rr;
      const bool claim = sqrt(rr / sc->bb) < sc->eps;
      const bool refine = claim || rr < sc->delta2 * sc->rr_ref;
      sc->converged = 0;
      sc->switched = refine;
      sc->done = refine || sc->iter >= sc->maxiters;
    } else if (KIND == SWEEP_PPCG_LAST) {
      DevScalars *sc = F.sc;
      const double rrn = tot[0];
      sc->beta = rrn / sc->rro;  // PPCG.jl:89-92
      sc->rro = rrn;
      sc->error = rrn;
      sc->iter += 1;
      sc->cheby_iters += 1;
      sc->first = 0;
      const bool claim = sqrt(rrn / sc->bb) < sc->eps;
      const bool refine = claim || rrn < sc->delta2 * sc->rr_ref;
      sc->converged = 0;
      sc->switched = refine;
      const int done = refine || sc->iter >= sc->maxiters;
      sc->done = done;
      if (set_cond) cudaGraphSetConditional(cond, done ? 0u : 1u);
    }
  }
};

template <int AHEAD>
using OpIrUpdate = OpIrSweep<AHEAD, SWEEP_CG>;

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

// The start of an FP32 CG loop: p32 = r32 = (float) r on the interior (0 in
// the halo) and x = 0.
__global__ void k_ir_convert(Fields F, Geom g, G32 g32, float *r, float *p, float *x) {
  const long long n = (long long)g.X * g.Y;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int I = (int)(k % g.X), J = (int)(k / g.X);
    const size_t c = (size_t)I + (size_t)J * g.pitch, c32 = (size_t)I + (size_t)J * g32.pitch;
    const bool interior = I >= g.hd && I < g.X - g.hd && J >= g.hd && J < g.Y - g.hd;
    const float rv = interior ? (float)F.r[c] : 0.f;
    r[c32] = rv;
    p[c32] = rv;
    x[c32] = 0.f;
  }
}

// The FP32 inverse weights iw = 1/w over the whole array (w = rho for
// conductivity, 1/rho for its reciprocal: CG.jl:57-60 over the whole array,
// the tealeaf-mode range) and the face factors rx/2, ry/2, so that
// Kx = rx (w_l + w_c) / (2 w_l w_c) = rx/2 (iw_l + iw_c) (CG.jl:62-67).
__global__ void k_ir_convert_iw(Fields F, Geom g, G32 g32, float *iw, int coefficient, double rx, double ry) {
  const long long n = (long long)g.X * g.Y;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    F.sc->rxh = 0.5 * rx;
    F.sc->ryh = 0.5 * ry;
  }
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int I = (int)(k % g.X), J = (int)(k / g.X);
    const double rho = F.density[(size_t)I + (size_t)J * g.pitch];
    iw[(size_t)I + (size_t)J * g32.pitch] = (float)(coefficient == TL_CONDUCTIVITY ? 1.0 / rho : rho);
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
  q.r = ctx->ir->r;
  q.x = ctx->ir->x;
  q.iw = ctx->ir->iw;
  return q;
}

}  // namespace
}  // namespace tl
