// tl_kernels_cheby.cu -- fused kernels of the Chebyshev, PPCG and Jacobi
// iterations (src/solvers/Cheby.jl, PPCG.jl, Jacobi.jl) in the tealeaf
// semantics.  EXACT keeps the reference's operation order without FMA
// (bit-identical to the CPU restatement); otherwise the stencil uses the
// stored diagonal and fused multiply-adds.  Fields read at the neighbours are
// ping-ponged between two buffers; the depth-1 reflective halo the reference
// refreshes before each stencil is folded into the row marcher.
#include "tl_solvers.h"
#include "tl_march.cuh"

namespace tl {

// ---------------------------------------------------------------------------
// Chebyshev (Cheby.jl:64-106)
// ---------------------------------------------------------------------------

// init!, first half: w = A u, r = u0 - w, p = r / theta (u's halo read from memory).
__global__ void k_cheby_init(Fields F, Geom g, double theta) {
  const long long n = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const size_t c = g.at((int)(k % g.nx), (int)(k / g.nx));
    const double wv = smvp_exact(F, g, F.u, c, TL_MODE_TEALEAF);
    F.w[c] = wv;
    const double rv = dsub(F.u0[c], wv);
    F.r[c] = rv;
    F.p[c] = ddiv(rv, theta);
  }
}

// init!, second half: u += p on the interior.
__global__ void k_add_p_to_u(Fields F, Geom g) {
  const long long n = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const size_t c = g.at((int)(k % g.nx), (int)(k / g.nx));
    F.u[c] = dadd(F.u[c], F.p[c]);
  }
}

// One Chebyshev step: w = A u, r = u0 - w, p = alpha_k p + beta_k r,
// u' = u + p (u' into the other buffer), r.r when this step computes the norm.
template <bool EXACT>
struct OpCheby {
  Fields F;
  Geom g;
  const double *__restrict__ usrc;
  double *__restrict__ udst;
  int guard;
  int force_norm;  // the first step always takes the norm (Cheby.jl:43)
  cudaGraphConditionalHandle cond;
  int set_cond;
  __device__ bool skip() const { return guard && F.sc->done; }
  __device__ void on_skip() const {
    if (set_cond && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(cond, 0u);
  }
  __device__ void tile(int i0, int j0, int j1, double (&acc)[1]) const {
    const int k = F.sc->cheby_iters + 1;  // this step's chebyiters (Cheby.jl:35)
    const int idx = min(k + 1, F.sc->maxiters + 1);  // the tables hold maxiters + 2 entries
    const double ca = F.chebyalpha[idx], cb = F.chebybeta[idx];
    SrcField src;
    src.f = usrc;
    march<!EXACT>(g, F.kx, F.ky, F.diag, src, i0, j0, j1,
                  [&](int j, const Nbr &c0, const Nbr &c1, bool has1, double2) {
                    const size_t c = g.at(i0, j);
                    double wv[2], rv[2], pv[2], uv[2];
                    const Nbr *q[2] = {&c0, &c1};
                    const int nc = has1 ? 2 : 1;
                    for (int m = 0; m < nc; ++m) {
                      wv[m] = apply_a<EXACT>(*q[m]);
                      const double u0 = F.u0[c + m], p0 = F.p[c + m];
                      if (EXACT) {
                        rv[m] = dsub(u0, wv[m]);
                        pv[m] = dadd(dmul(ca, p0), dmul(cb, rv[m]));
                        uv[m] = dadd(q[m]->c, pv[m]);
                        acc[0] = dadd(acc[0], dmul(rv[m], rv[m]));
                      } else {
                        rv[m] = u0 - wv[m];
                        pv[m] = fma(ca, p0, cb * rv[m]);
                        uv[m] = q[m]->c + pv[m];
                        acc[0] = fma(rv[m], rv[m], acc[0]);
                      }
                    }
                    if (has1) {
                      st2(F.w + c, make_double2(wv[0], wv[1]));
                      st2(F.r + c, make_double2(rv[0], rv[1]));
                      st2(F.p + c, make_double2(pv[0], pv[1]));
                      st2(udst + c, make_double2(uv[0], uv[1]));
                    } else {
                      F.w[c] = wv[0];
                      F.r[c] = rv[0];
                      F.p[c] = pv[0];
                      udst[c] = uv[0];
                    }
                  });
  }
  __device__ void fin(const double *tot) const {
    DevScalars *sc = F.sc;
    const int k = sc->cheby_iters + 1;
    const int tt = sc->iter + 1;  // this step's trip of the solver loop
    const bool calc2norm = force_norm || ((k >= sc->est_iters) && ((tt + 1) % 10 == 0));  // Cheby.jl:48
    if (calc2norm) sc->error = tot[0];
    sc->cheby_iters = k;
    sc->iter = tt;
    loop_control(sc, cond, set_cond);
  }
};

// ---------------------------------------------------------------------------
// PPCG (PPCG.jl:64-94)
// ---------------------------------------------------------------------------

// u += alpha p, r -= alpha w, then sd = r / theta (the inner sweeps' start).
// The fused form multiplies by 1/theta, formed once per thread (a division
// per cell made this pass division-bound), and moves column pairs as double2.
template <bool EXACT>
struct OpPpcgUR : NoSkip {
  Fields F;
  Geom g;
  const double *__restrict__ p;
  double *__restrict__ sd;
  int guard;
  __device__ bool skip() const { return guard && F.sc->done; }
  __device__ void tile(int i0, int j0, int j1, double (&)[1]) const {
    if (i0 >= g.nx) return;
    const int nc = i0 + 1 < g.nx ? 2 : 1;
    const double alpha = F.sc->alpha, theta = F.sc->theta;
    if (!EXACT && nc == 2) {
      const double rtheta = 1.0 / theta;
      for (int j = j0; j < j1; ++j) {
        const size_t c = g.at(i0, j);
        const double2 pv = ld2(p + c), wv = ld2(F.w + c);
        double2 uv = ld2(F.u + c), rv = ld2(F.r + c);
        uv.x = fma(alpha, pv.x, uv.x);
        uv.y = fma(alpha, pv.y, uv.y);
        rv.x = fma(-alpha, wv.x, rv.x);
        rv.y = fma(-alpha, wv.y, rv.y);
        st2(F.u + c, uv);
        st2(F.r + c, rv);
        st2(sd + c, make_double2(rv.x * rtheta, rv.y * rtheta));
      }
      return;
    }
    for (int j = j0; j < j1; ++j) {
      const size_t c = g.at(i0, j);
      for (int m = 0; m < nc; ++m) {
        const double pv = p[c + m], wv = F.w[c + m];
        double uv = F.u[c + m], rv = F.r[c + m];
        if (EXACT) {
          uv = dadd(uv, dmul(alpha, pv));
          rv = dsub(rv, dmul(alpha, wv));
        } else {
          uv = fma(alpha, pv, uv);
          rv = fma(-alpha, wv, rv);
        }
        F.u[c + m] = uv;
        F.r[c + m] = rv;
        sd[c + m] = ddiv(rv, theta);
      }
    }
  }
};

// One inner sweep: r -= A sd, u += sd, sd' = alpha_pp sd + beta_pp r (into
// the other buffer).  The last sweep of an outer step also sums r.r and runs
// the outer step's epilogue (PPCG.jl:89-93).
template <bool EXACT>
struct OpPpcgInner {
  Fields F;
  Geom g;
  const double *__restrict__ sdsrc;
  double *__restrict__ sddst;
  int pp;     // 1-based inner step
  int last;
  int guard;
  cudaGraphConditionalHandle cond;
  int set_cond;
  __device__ bool skip() const { return guard && F.sc->done; }
  __device__ void on_skip() const {
    if (set_cond && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(cond, 0u);
  }
  __device__ void tile(int i0, int j0, int j1, double (&acc)[1]) const {
    const double ca = F.chebyalpha[pp], cb = F.chebybeta[pp];
    SrcField src;
    src.f = sdsrc;
    march<!EXACT>(g, F.kx, F.ky, F.diag, src, i0, j0, j1,
                  [&](int j, const Nbr &c0, const Nbr &c1, bool has1, double2) {
                    const size_t c = g.at(i0, j);
                    double rv[2], uv[2], sv[2];
                    const Nbr *q[2] = {&c0, &c1};
                    const int nc = has1 ? 2 : 1;
                    for (int m = 0; m < nc; ++m) {
                      const double av = apply_a<EXACT>(*q[m]);
                      const double s0 = q[m]->c;
                      if (EXACT) {
                        rv[m] = dsub(F.r[c + m], av);
                        uv[m] = dadd(F.u[c + m], s0);
                        sv[m] = dadd(dmul(ca, s0), dmul(cb, rv[m]));
                        if (last) acc[0] = dadd(acc[0], dmul(rv[m], rv[m]));
                      } else {
                        rv[m] = F.r[c + m] - av;
                        uv[m] = F.u[c + m] + s0;
                        sv[m] = fma(ca, s0, cb * rv[m]);
                        if (last) acc[0] = fma(rv[m], rv[m], acc[0]);
                      }
                    }
                    if (has1) {
                      st2(F.r + c, make_double2(rv[0], rv[1]));
                      st2(F.u + c, make_double2(uv[0], uv[1]));
                      st2(sddst + c, make_double2(sv[0], sv[1]));
                    } else {
                      F.r[c] = rv[0];
                      F.u[c] = uv[0];
                      sddst[c] = sv[0];
                    }
                  });
  }
  __device__ void fin(const double *tot) const {
    if (!last) return;
    DevScalars *sc = F.sc;
    const double rrn = tot[0];
    sc->beta = ddiv(rrn, sc->rro);
    sc->rro = rrn;
    sc->error = rrn;
    sc->iter += 1;
    sc->cheby_iters += 1;
    sc->first = 0;
    loop_control(sc, cond, set_cond);
  }
};

// ---------------------------------------------------------------------------
// Jacobi (Jacobi.jl:59-80)
// ---------------------------------------------------------------------------

// One sweep: r = u (interior, plus the depth-1 faces, which hold the
// reflection of u), u' = (u0 + sum k u_nbr) / (1 + sum k), error = sum |u' - u|.
// EXACT: the reference's operation order and the division.  Otherwise the
// numerator is a chain of fused multiply-adds and the division is a product
// with 1 / (1 + sum k), stored once per solve in `diag` (a division per cell
// made the sweep division-bound).
template <bool EXACT>
struct OpJacobi {
  Fields F;
  Geom g;
  const double *__restrict__ usrc;
  double *__restrict__ udst;
  int guard;
  __device__ bool skip() const { return guard && F.sc->done; }
  __device__ void on_skip() const {}
  __device__ void tile(int i0, int j0, int j1, double (&acc)[1]) const {
    SrcField src;
    src.f = usrc;
    march<!EXACT>(g, F.kx, F.ky, F.diag, src, i0, j0, j1,
                  [&](int j, const Nbr &c0, const Nbr &c1, bool has1, double2) {
                    const size_t c = g.at(i0, j);
                    const Nbr *q[2] = {&c0, &c1};
                    const int nc = has1 ? 2 : 1;
                    for (int m = 0; m < nc; ++m) {
                      const Nbr &t = *q[m];
                      double un;
                      if (EXACT) {
                        double num = dadd(F.u0[c + m], dmul(t.kx1, t.e));
                        num = dadd(num, dmul(t.kx0, t.w));
                        num = dadd(num, dmul(t.ky1, t.n));
                        num = dadd(num, dmul(t.ky0, t.s));
                        const double den = dadd(dadd(dadd(dadd(1.0, t.kx0), t.kx1), t.ky0), t.ky1);
                        un = ddiv(num, den);
                      } else {
                        const double num = fma(t.ky0, t.s, fma(t.ky1, t.n, fma(t.kx0, t.w, fma(t.kx1, t.e, F.u0[c + m]))));
                        un = num * t.dg;
                      }
                      udst[c + m] = un;
                      F.r[c + m] = t.c;
                      acc[0] = dadd(acc[0], fabs(dsub(un, t.c)));
                      // r .= u copies u's depth-1 halo, the reflection of u
                      const int i = i0 + m;
                      if (i == 0) F.r[c + m - 1] = t.c;
                      if (i == g.nx - 1) F.r[c + m + 1] = t.c;
                      if (j == 0) F.r[c + m - g.pitch] = t.c;
                      if (j == g.ny - 1) F.r[c + m + g.pitch] = t.c;
                    }
                  });
  }
  __device__ void fin(const double *tot) const {
    DevScalars *sc = F.sc;
    sc->error = tot[0];
    sc->iter += 1;
  }
};

// Every 50th sweep: r = u0 - A u, error += r.r (Jacobi.jl:16-21); then the
// loop's convergence test.
struct OpJacobiCheck {
  Fields F;
  Geom g;
  const double *__restrict__ u;
  int guard;
  cudaGraphConditionalHandle cond;
  int set_cond;
  __device__ bool skip() const { return guard && F.sc->done; }
  __device__ void on_skip() const {
    if (set_cond && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(cond, 0u);
  }
  __device__ void tile(int i0, int j0, int j1, double (&acc)[1]) const {
    if (F.sc->iter % 50 != 0) return;
    SrcField src;
    src.f = u;
    march<false>(g, F.kx, F.ky, F.diag, src, i0, j0, j1,
                 [&](int j, const Nbr &c0, const Nbr &c1, bool has1, double2) {
                   const size_t c = g.at(i0, j);
                   const Nbr *q[2] = {&c0, &c1};
                   const int nc = has1 ? 2 : 1;
                   for (int m = 0; m < nc; ++m) {
                     const double rv = dsub(F.u0[c + m], apply_a<true>(*q[m]));
                     F.r[c + m] = rv;
                     acc[0] = dadd(acc[0], dmul(rv, rv));
                   }
                 });
  }
  __device__ void fin(const double *tot) const {
    DevScalars *sc = F.sc;
    if (sc->iter % 50 == 0) sc->error = dadd(sc->error, tot[0]);
    loop_control(sc, cond, set_cond);
  }
};

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

static inline int grid_for(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152LL * 32) b = 152LL * 32;
  return (int)(b < 1 ? 1 : b);
}

void launch_cheby_init(cudaStream_t st, const Fields &F, const Geom &g, double theta) {
  k_cheby_init<<<grid_for((long long)g.nx * g.ny), 256, 0, st>>>(F, g, theta);
  k_add_p_to_u<<<grid_for((long long)g.nx * g.ny), 256, 0, st>>>(F, g);
}

void launch_cheby_step(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, const double *usrc,
                       double *udst, int exact, int guard, int force_norm, cudaGraphConditionalHandle cond,
                       int set_cond) {
  if (exact) {
    OpCheby<true> op;
    op.F = F; op.g = g; op.usrc = usrc; op.udst = udst; op.guard = guard; op.force_norm = force_norm;
    op.cond = cond; op.set_cond = set_cond;
    launch_walk<1>(st, op, wk, g.ny);
  } else {
    OpCheby<false> op;
    op.F = F; op.g = g; op.usrc = usrc; op.udst = udst; op.guard = guard; op.force_norm = force_norm;
    op.cond = cond; op.set_cond = set_cond;
    launch_walk<1>(st, op, wk, g.ny);
  }
}

void launch_ppcg_ur(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, const double *p, double *sd,
                    int exact, int guard) {
  if (exact) {
    OpPpcgUR<true> op;
    op.F = F; op.g = g; op.p = p; op.sd = sd; op.guard = guard;
    launch_walk<0>(st, op, wk, g.ny);
  } else {
    OpPpcgUR<false> op;
    op.F = F; op.g = g; op.p = p; op.sd = sd; op.guard = guard;
    launch_walk<0>(st, op, wk, g.ny);
  }
}

void launch_ppcg_inner(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, const double *sdsrc,
                       double *sddst, int pp, int last, int exact, int guard, cudaGraphConditionalHandle cond,
                       int set_cond) {
  if (exact) {
    OpPpcgInner<true> op;
    op.F = F; op.g = g; op.sdsrc = sdsrc; op.sddst = sddst; op.pp = pp; op.last = last; op.guard = guard;
    op.cond = cond; op.set_cond = set_cond;
    launch_walk<1>(st, op, wk, g.ny);
  } else {
    OpPpcgInner<false> op;
    op.F = F; op.g = g; op.sdsrc = sdsrc; op.sddst = sddst; op.pp = pp; op.last = last; op.guard = guard;
    op.cond = cond; op.set_cond = set_cond;
    launch_walk<1>(st, op, wk, g.ny);
  }
}

void launch_jacobi(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, const double *usrc, double *udst,
                   int guard, int exact) {
  if (exact) {
    OpJacobi<true> op;
    op.F = F; op.g = g; op.usrc = usrc; op.udst = udst; op.guard = guard;
    launch_walk<1>(st, op, wk, g.ny);
  } else {
    OpJacobi<false> op;
    op.F = F; op.g = g; op.usrc = usrc; op.udst = udst; op.guard = guard;
    launch_walk<1>(st, op, wk, g.ny);
  }
}

// diag = 1 / (1 + kx[i+1] + kx[i] + ky[j+1] + ky[j]): the fused Jacobi sweep's reciprocal.
__global__ void k_init_rdiag(Fields F, Geom g) {
  const long long n = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const size_t c = g.at((int)(k % g.nx), (int)(k / g.nx));
    F.diag[c] = 1.0 / (1.0 + F.kx[c + 1] + F.kx[c] + F.ky[c + g.pitch] + F.ky[c]);
  }
}

void launch_init_rdiag(cudaStream_t st, const Fields &F, const Geom &g) {
  k_init_rdiag<<<grid_for((long long)g.nx * g.ny), 256, 0, st>>>(F, g);
}

void launch_jacobi_check(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk, const double *u, int guard,
                         cudaGraphConditionalHandle cond, int set_cond) {
  OpJacobiCheck op;
  op.F = F; op.g = g; op.u = u; op.guard = guard; op.cond = cond; op.set_cond = set_cond;
  launch_walk<1>(st, op, wk, g.ny);
}

// Interior r.r into red[0] (PPCG's init! after the residual).
struct OpNormR : NoSkip {
  Fields F;
  Geom g;
  __device__ void tile(int i0, int j0, int j1, double (&acc)[1]) const {
    for (int j = j0; j < j1; ++j) {
      if (i0 < g.nx) {
        const double v = F.r[g.at(i0, j)];
        acc[0] = dadd(acc[0], dmul(v, v));
      }
      if (i0 + 1 < g.nx) {
        const double v = F.r[g.at(i0 + 1, j)];
        acc[0] = dadd(acc[0], dmul(v, v));
      }
    }
  }
  __device__ void fin(const double *tot) const { F.sc->red[0] = tot[0]; }
};

void launch_norm_r(cudaStream_t st, const Fields &F, const Geom &g, const Walk &wk) {
  OpNormR op;
  op.F = F;
  op.g = g;
  launch_walk<1>(st, op, wk, g.ny);
}

// The reference's single sd buffer after the inner sweeps: interior = the last
// sd, depth-1 faces = the reflection of the sd before the last sweep (the
// halo update runs before each sweep, PPCG.jl:76).  `fin` holds the last sd,
// `prev` the one before; the result goes to F.sd (which may be either).
__global__ void k_ppcg_sd_final(Fields F, Geom g, const double *fin, const double *prev) {
  const long long n = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(k % g.nx), j = (int)(k / g.nx);
    const size_t c = g.at(i, j);
    const double pv = prev[c];
    if (i == 0) F.sd[c - 1] = pv;
    if (i == g.nx - 1) F.sd[c + 1] = pv;
    if (j == 0) F.sd[c - g.pitch] = pv;
    if (j == g.ny - 1) F.sd[c + g.pitch] = pv;
  }
}

__global__ void k_copy_interior(double *dst, const double *src, Geom g) {
  const long long n = (long long)g.nx * g.ny;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const size_t c = g.at((int)(k % g.nx), (int)(k / g.nx));
    dst[c] = src[c];
  }
}

void launch_ppcg_sd_final(cudaStream_t st, const Fields &F, const Geom &g, const double *fin, const double *prev) {
  // the faces first: when `prev` is F.sd its interior is still intact here
  k_ppcg_sd_final<<<grid_for((long long)g.nx * g.ny), 256, 0, st>>>(F, g, fin, prev);
  if (fin != F.sd) k_copy_interior<<<grid_for((long long)g.nx * g.ny), 256, 0, st>>>(F.sd, fin, g);
}

void launch_copy_interior(cudaStream_t st, double *dst, const double *src, const Geom &g) {
  k_copy_interior<<<grid_for((long long)g.nx * g.ny), 256, 0, st>>>(dst, src, g);
}

}  // namespace tl
