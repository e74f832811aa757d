// tl_kernels_cg.cu -- the CG iteration (src/solvers/CG.jl:32-44, 82-104).
//
// Reference mode: w! / ur! / p! as three passes with the reference's diagonal
// smvp (kernels.jl:180-181) and explicitly rounded arithmetic.
//
// Tealeaf mode: two fused passes per iteration,
//   step W : p' = beta*p + r (the previous iteration's p!), w = A p', p'.w
//   step UR: u += alpha p', r -= alpha w, r.r
// p' is written to the other buffer of a ping-pong pair because the stencil
// reads p at the neighbours.  The depth-1 reflective halo of p' that the
// reference refreshes every iteration (CG.jl:23) is folded into the index
// math: a neighbour across the boundary is the cell itself.  EXACT keeps the
// reference's operation order with no FMA (bit-identical to the CPU
// restatement); otherwise the stencil is diag*p - kx1*pE - kx0*pW - ky1*pN -
// ky0*pS with the diagonal read from memory and every update fused.
#include "tl_solvers.h"
#include "tl_cg_ops.cuh"

namespace tl {

// ---------------------------------------------------------------------------
// reference mode
// ---------------------------------------------------------------------------

struct OpRefW : NoSkip {
  Fields F;
  Geom g;
  __device__ void cell(int i, int j, double (&acc)[1]) const {
    const size_t c = g.at(i, j);
    const double consum = dadd(dadd(dadd(dadd(1.0, F.kx[c + 1]), F.kx[c]), F.ky[c + g.pitch]), F.ky[c]);
    const double pv = F.p[c];
    const double wv = dmul(consum, pv);
    F.w[c] = wv;
    acc[0] = dadd(acc[0], dmul(wv, pv));
  }
  __device__ void tile(int i0, int j0, int j1, double (&acc)[1]) const {
    for (int j = j0; j < j1; ++j) {
      if (i0 < g.nx) cell(i0, j, acc);
      if (i0 + 1 < g.nx) cell(i0 + 1, j, acc);
    }
  }
  __device__ void fin(const double *tot) const {
    DevScalars *sc = F.sc;
    sc->pw = tot[0];
    sc->alpha = ddiv(sc->rro, sc->pw);
    if (sc->iter < sc->maxiters) F.cgalpha[sc->iter + 1] = sc->alpha;  // table holds maxiters + 2 entries
  }
};

struct OpRefUR : NoSkip {
  Fields F;
  Geom g;
  cudaGraphConditionalHandle cond;
  int set_cond;
  __device__ void cell(int i, int j, double alpha, double (&acc)[1]) const {
    const size_t c = g.at(i, j);
    F.u[c] = dadd(F.u[c], dmul(alpha, F.p[c]));
    const double rv = dsub(F.r[c], dmul(alpha, F.w[c]));
    F.r[c] = rv;
    acc[0] = dadd(acc[0], dmul(rv, rv));
  }
  __device__ void tile(int i0, int j0, int j1, double (&acc)[1]) const {
    const double alpha = F.sc->alpha;
    for (int j = j0; j < j1; ++j) {
      if (i0 < g.nx) cell(i0, j, alpha, acc);
      if (i0 + 1 < g.nx) cell(i0 + 1, j, alpha, acc);
    }
  }
  __device__ void fin(const double *tot) const { ur_epilogue(F, tot[0], cond, set_cond); }
};

struct OpRefP : NoSkip {
  Fields F;
  Geom g;
  __device__ void tile(int i0, int j0, int j1, double (&)[1]) const {
    const double beta = F.sc->beta;
    for (int j = j0; j < j1; ++j) {
      if (i0 < g.nx) {
        const size_t c = g.at(i0, j);
        F.p[c] = dadd(dmul(beta, F.p[c]), F.r[c]);
      }
      if (i0 + 1 < g.nx) {
        const size_t c = g.at(i0 + 1, j);
        F.p[c] = dadd(dmul(beta, F.p[c]), F.r[c]);
      }
    }
  }
};

void launch_ref_w(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk) {
  OpRefW op;
  op.F = F;
  op.g = g;
  launch_walk<1>(st, op, wk, g.ny);
}

void launch_ref_ur(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, cudaGraphConditionalHandle cond,
                   int set_cond) {
  OpRefUR op;
  op.F = F;
  op.g = g;
  op.cond = cond;
  op.set_cond = set_cond;
  launch_walk<1>(st, op, wk, g.ny);
}

void launch_ref_p(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk) {
  OpRefP op;
  op.F = F;
  op.g = g;
  launch_walk<0>(st, op, wk, g.ny);
}

// ---------------------------------------------------------------------------
// tealeaf mode, fused
// ---------------------------------------------------------------------------

template <bool EXACT>
struct OpTlP : NoSkip {
  Fields F;
  Geom g;
  const double *psrc;
  double *pdst;
  __device__ void tile(int i0, int j0, int j1, double (&)[1]) const {
    if (i0 >= g.nx) return;
    const bool has1 = i0 + 1 < g.nx;
    const double beta = F.sc->beta;
    for (int j = j0; j < j1; ++j) {
      const size_t c = g.at(i0, j);
      const double2 pv = ld2(psrc + c), rv = ld2(F.r + c);
      const double2 o = make_double2(axpy<EXACT>(beta, pv.x, rv.x), axpy<EXACT>(beta, pv.y, rv.y));
      if (has1) st2(pdst + c, o);
      else pdst[c] = o.x;
    }
  }
};

}  // namespace tl

int tl_occupancy_cg(int kernel, int threads) {
  int n = 0;
  cudaError_t e = kernel == 0
      ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, tl::k_walk<1, tl::OpTlW<false>>, threads, 0)
      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, tl::k_walk<1, tl::OpTlUR<false>>, threads, 0);
  return e == cudaSuccess ? n : 1;
}

namespace tl {

void launch_tl_w(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, const double *psrc, double *pdst,
                 int exact, int guard, int store_coef) {
  if (exact) {
    OpTlW<true> op;
    op.F = F; op.g = g; op.psrc = psrc; op.pdst = pdst; op.guard = guard; op.store_coef = store_coef;
    launch_walk<1>(st, op, wk, g.ny);
  } else {
    OpTlW<false> op;
    op.F = F; op.g = g; op.psrc = psrc; op.pdst = pdst; op.guard = guard; op.store_coef = store_coef;
    launch_walk<1>(st, op, wk, g.ny);
  }
}

void launch_tl_ur(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, const double *p, int exact,
                  int guard, cudaGraphConditionalHandle cond, int set_cond) {
  if (exact) {
    OpTlUR<true> op;
    op.F = F; op.g = g; op.p = p; op.guard = guard; op.cond = cond; op.set_cond = set_cond;
    launch_walk<1>(st, op, wk, g.ny);
  } else {
    OpTlUR<false> op;
    op.F = F; op.g = g; op.p = p; op.guard = guard; op.cond = cond; op.set_cond = set_cond;
    launch_walk<1>(st, op, wk, g.ny);
  }
}

void launch_tl_p(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, const double *psrc, double *pdst,
                 int exact) {
  if (exact) {
    OpTlP<true> op;
    op.F = F; op.g = g; op.psrc = psrc; op.pdst = pdst;
    launch_walk<0>(st, op, wk, g.ny);
  } else {
    OpTlP<false> op;
    op.F = F; op.g = g; op.psrc = psrc; op.pdst = pdst;
    launch_walk<0>(st, op, wk, g.ny);
  }
}

}  // namespace tl
