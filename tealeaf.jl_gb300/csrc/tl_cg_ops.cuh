// tl_cg_ops.cuh -- the fused CG step operations (tealeaf semantics), shared
// by the single-deck loop (tl_kernels_cg.cu) and the batched loop
// (tl_batch.cu).
#pragma once

#include "tl_march.cuh"

namespace tl {

// ur!: u += alpha p, r -= alpha w, then the epilogue of mainstep! and the
// solver loop's convergence test.
__device__ __forceinline__ void ur_epilogue(const Fields &F, double rrn, cudaGraphConditionalHandle cond,
                                            int set_cond) {
  DevScalars *sc = F.sc;
  sc->rrn = rrn;
  sc->beta = ddiv(rrn, sc->rro);
  if (sc->iter < sc->maxiters) F.cgbeta[sc->iter + 1] = sc->beta;
  if (!sc->stale_rro) sc->rro = rrn;
  sc->error = rrn;
  sc->iter += 1;
  sc->first = 0;
  loop_control(sc, cond, set_cond);
}

template <bool EXACT>
struct OpTlW {
  Fields F;
  Geom g;
  const double *__restrict__ psrc;
  double *__restrict__ pdst;
  int guard;
  int store_coef;  // CG and its presteps record alpha in cgalpha (CG.jl:37); PPCG's outer steps do not
  __device__ bool skip() const { return guard && F.sc->done; }
  __device__ void on_skip() const {}

  __device__ void tile(int i0, int j0, int j1, double (&acc)[1]) const {
    SrcPUpdate<EXACT> src;
    src.p = psrc;
    src.r = F.r;
    src.beta = F.sc->beta;
    src.first = F.sc->first != 0;
    march<!EXACT>(g, F.kx, F.ky, F.diag, src, i0, j0, j1,
                  [&](int j, const Nbr &c0, const Nbr &c1, bool has1, double2 pc) {
                    const size_t c = g.at(i0, j);
                    const double w0 = apply_a<EXACT>(c0);
                    acc[0] = acc_mul<EXACT>(acc[0], w0, c0.c);
                    if (has1) {
                      const double w1 = apply_a<EXACT>(c1);
                      acc[0] = acc_mul<EXACT>(acc[0], w1, c1.c);
                      st2(F.w + c, make_double2(w0, w1));
                      st2(pdst + c, pc);
                    } else {
                      F.w[c] = w0;
                      pdst[c] = pc.x;
                    }
                  });
  }
  __device__ void fin(const double *tot) const {
    DevScalars *sc = F.sc;
    sc->pw = tot[0];
    sc->alpha = ddiv(sc->rro, sc->pw);
    if (store_coef && sc->iter < sc->maxiters) F.cgalpha[sc->iter + 1] = sc->alpha;  // table holds maxiters + 2 entries
  }
};

template <bool EXACT>
struct OpTlUR {
  Fields F;
  Geom g;
  const double *__restrict__ p;
  int guard;
  cudaGraphConditionalHandle cond;
  int set_cond;
  __device__ bool skip() const { return guard && F.sc->done; }
  __device__ void on_skip() const {
    if (set_cond && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(cond, 0u);
  }
  __device__ void tile(int i0, int j0, int j1, double (&acc)[1]) const {
    if (i0 >= g.nx) return;
    const bool has1 = i0 + 1 < g.nx;
    const double alpha = F.sc->alpha;
    for (int j = j0; j < j1; ++j) {
      const size_t c = g.at(i0, j);
      const double2 pv = ld2(p + c), wv = ld2(F.w + c);
      double2 uv = ld2(F.u + c), rv = ld2(F.r + c);
      uv.x = axpy<EXACT>(alpha, pv.x, uv.x);
      uv.y = axpy<EXACT>(alpha, pv.y, uv.y);
      if (EXACT) {
        rv.x = dsub(rv.x, dmul(alpha, wv.x));
        rv.y = dsub(rv.y, dmul(alpha, wv.y));
      } else {
        rv.x = fma(-alpha, wv.x, rv.x);
        rv.y = fma(-alpha, wv.y, rv.y);
      }
      acc[0] = acc_mul<EXACT>(acc[0], rv.x, rv.x);
      if (has1) {
        acc[0] = acc_mul<EXACT>(acc[0], rv.y, rv.y);
        st2(F.u + c, uv);
        st2(F.r + c, rv);
      } else {
        F.u[c] = uv.x;
        F.r[c] = rv.x;
      }
    }
  }
  __device__ void fin(const double *tot) const { ur_epilogue(F, tot[0], cond, set_cond); }
};

}  // namespace tl
