// tl_march.cuh -- the row marcher shared by every fused 5-point kernel.
//
// A lane owns the interior column pair (i0, i0+1) of a tile and walks its rows
// j0..j1-1.  The marcher supplies, for each row and each owned cell, the
// value of the stencil's input field at the cell and its four neighbours, and
// the coefficients kx[i], kx[i+1], ky[j], ky[j+1] (and the stored diagonal):
//   * east/west neighbours come from the neighbouring lanes by shuffle; lane 0
//     and lane 31 load the one neighbour their shuffle cannot supply;
//   * north/south neighbours are the previous and next rows, kept in
//     registers while marching;
//   * a neighbour across the domain boundary is the cell itself: the depth-1
//     reflective halo that the reference refreshes before every stencil
//     (haloupdate! with the field marked) folded into the index math;
//   * every load of the next row is issued before the current row's
//     arithmetic (one row of prefetch).
// The input value is built from raw loads by the Src policy (p itself, or
// beta*p + r for the fused CG step), so a field that is updated on the fly is
// never read back from memory.
#pragma once

#include "tl_walk.cuh"

namespace tl {

// One owned cell's stencil inputs.
struct Nbr {
  double c, e, w, n, s;          // the field at the cell and its E, W, N, S neighbours
  double kx0, kx1, ky0, ky1, dg; // kx[i], kx[i+1], ky[j], ky[j+1], diag
};

// Src policies: raw loads of one row plus the value they make.
// Identity: the field itself.
struct SrcField {
  const double *f;
  struct Raw {
    double2 v;
    double ev;
  };
  __device__ __forceinline__ void load(Raw &o, size_t c, long long ec) const {
    o.v = ld2(f + c);
    if (ec >= 0) o.ev = __ldg(f + ec);
  }
  __device__ __forceinline__ double2 val(const Raw &o) const { return o.v; }
  __device__ __forceinline__ double val_edge(const Raw &o) const { return o.ev; }
};

// beta*p + r (the previous CG iteration's p!), or p on the first iteration.
template <bool EXACT>
struct SrcPUpdate {
  const double *p, *r;
  double beta;
  bool first;
  struct Raw {
    double2 p, r;
    double ep, er;
  };
  __device__ __forceinline__ void load(Raw &o, size_t c, long long ec) const {
    o.p = ld2(p + c);
    if (!first) o.r = ld2(r + c);
    if (ec >= 0) {
      o.ep = __ldg(p + ec);
      if (!first) o.er = __ldg(r + ec);
    }
  }
  __device__ __forceinline__ double2 val(const Raw &o) const {
    return first ? o.p : make_double2(axpy<EXACT>(beta, o.p.x, o.r.x), axpy<EXACT>(beta, o.p.y, o.r.y));
  }
  __device__ __forceinline__ double val_edge(const Raw &o) const {
    return first ? o.ep : axpy<EXACT>(beta, o.ep, o.er);
  }
};

// Walks the rows of one lane's column pair.  body(j, c0, c1, has1, center)
// receives both cells' inputs (c1 only meaningful when has1) and the pair's
// input values; it runs for valid lanes only, and every lane executes the
// shuffles.
template <bool DIAG, class Src, class Body>
__device__ __forceinline__ void march(const Geom &g, const double *kx, const double *ky, const double *diag,
                                      const Src &src, int i0, int j0, int j1, Body &&body) {
  using Raw = typename Src::Raw;
  struct Coef {
    double2 kx, dg;
    double kxe;
  };
  const int nx = g.nx, ny = g.ny;
  const int lane = threadIdx.x & 31;
  const bool valid = i0 < nx;
  const bool has1 = i0 + 1 < nx;
  const bool inner = i0 + 2 < nx;
  const double2 z = make_double2(0.0, 0.0);
  const int edge_col = !valid ? -1 : (lane == 0 && i0 > 0) ? i0 - 1 : (lane == 31 && inner) ? i0 + 2 : -1;
  const bool kx_edge = valid && has1 && (!inner || lane == 31);
  auto eidx = [&](int j) -> long long { return edge_col >= 0 ? (long long)g.at(edge_col, j) : -1LL; };
  auto load_coef = [&](Coef &o, int j) {
    const size_t c = g.at(i0, j);
    o.kx = ld2(kx + c);
    if (DIAG) o.dg = ld2(diag + c);
    if (kx_edge) o.kxe = __ldg(kx + c + 2);
  };

  Raw cur = {}, nxt = {}, prv = {};
  Coef cc = {}, cn = {};
  if (valid) {
    src.load(cur, g.at(i0, j0), eidx(j0));
    load_coef(cc, j0);
    if (j0 > 0) src.load(prv, g.at(i0, j0 - 1), -1);
    if (j0 + 1 < ny) src.load(nxt, g.at(i0, j0 + 1), eidx(j0 + 1));
  }
  double2 kyc = valid ? ld2(ky + g.at(i0, j0)) : z;
  double2 kyn = valid ? ld2(ky + g.at(i0, j0 + 1)) : z;
  double2 pc = valid ? src.val(cur) : z;
  double2 ps = (j0 > 0 && valid) ? src.val(prv) : pc;  // reflect at j = 0
  for (int j = j0; j < j1; ++j) {
    Raw nn = {};
    double2 kyn2 = z;
    if (j + 1 < j1 && valid) {
      if (j + 2 < ny) src.load(nn, g.at(i0, j + 2), eidx(j + 2));
      load_coef(cn, j + 1);
      kyn2 = ld2(ky + g.at(i0, j + 2));
    }
    const double2 pn = (j + 1 < ny && valid) ? src.val(nxt) : pc;  // reflect at j = ny-1
    double vw = __shfl_up_sync(FULL, pc.y, 1);
    double ve = __shfl_down_sync(FULL, pc.x, 1);
    double kxe = __shfl_down_sync(FULL, cc.kx.x, 1);
    if (valid) {
      if (i0 == 0) vw = pc.x;  // reflect at i = 0
      else if (lane == 0) vw = src.val_edge(cur);
      if (has1) {
        if (!inner) {
          ve = pc.y;           // reflect at i = nx-1
          kxe = cc.kxe;        // kx of the halo column
        } else if (lane == 31) {
          ve = src.val_edge(cur);
          kxe = cc.kxe;
        }
      }
      Nbr c0, c1;
      c0.c = pc.x; c0.e = has1 ? pc.y : pc.x; c0.w = vw; c0.n = pn.x; c0.s = ps.x;
      c0.kx0 = cc.kx.x; c0.kx1 = cc.kx.y; c0.ky0 = kyc.x; c0.ky1 = kyn.x; c0.dg = cc.dg.x;
      c1.c = pc.y; c1.e = ve; c1.w = pc.x; c1.n = pn.y; c1.s = ps.y;
      c1.kx0 = cc.kx.y; c1.kx1 = kxe; c1.ky0 = kyc.y; c1.ky1 = kyn.y; c1.dg = cc.dg.y;
      body(j, c0, c1, has1, pc);
    }
    ps = pc;
    pc = pn;
    kyc = kyn;
    kyn = kyn2;
    cur = nxt;
    nxt = nn;
    cc = cn;
  }
}

// The 5-point operator on one cell: reference operation order without FMA
// (EXACT), else diag*c - kx1*e - kx0*w - ky1*n - ky0*s with fused multiply-adds.
template <bool EXACT>
__device__ __forceinline__ double apply_a(const Nbr &q) {
  if (EXACT) {
    const double consum = dadd(dadd(dadd(dadd(1.0, q.kx1), q.kx0), q.ky1), q.ky0);
    double v = dmul(consum, q.c);
    v = dsub(v, dadd(dmul(q.kx1, q.e), dmul(q.kx0, q.w)));
    v = dsub(v, dadd(dmul(q.ky1, q.n), dmul(q.ky0, q.s)));
    return v;
  }
  double t = q.dg * q.c;
  t = fma(-q.kx1, q.e, t);
  t = fma(-q.kx0, q.w, t);
  t = fma(-q.ky1, q.n, t);
  t = fma(-q.ky0, q.s, t);
  return t;
}

// smvp (kernels.jl:178-184) on memory values, reference order, no FMA.
__device__ __forceinline__ double smvp_exact(const Fields &F, const Geom &g, const double *a, size_t c, int mode) {
  const double kxr = F.kx[c + 1], kxc = F.kx[c], kyt = F.ky[c + g.pitch], kyc = F.ky[c];
  const double consum = dadd(dadd(dadd(dadd(1.0, kxr), kxc), kyt), kyc);
  double v = dmul(consum, a[c]);
  if (mode == TL_MODE_REFERENCE) return v;  // kernels.jl:181 returns here
  v = dsub(v, dadd(dmul(kxr, a[c + 1]), dmul(kxc, a[c - 1])));
  v = dsub(v, dadd(dmul(kyt, a[c + g.pitch]), dmul(kyc, a[c - g.pitch])));
  return v;
}

}  // namespace tl
