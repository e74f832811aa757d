// tl_solvers.cu -- the Chebyshev, PPCG and Jacobi solver plugins
// (src/solvers/Cheby.jl, PPCG.jl, Jacobi.jl).
//
// Reference mode follows the reference as written: the CG presteps of Cheby
// (with its stale rro, Cheby.jl:33) and PPCG run, and where the reference
// raises (Cheby's one-argument minmax, kernels.jl:39; PPCG's `++`,
// PPCG.jl:36; Jacobi's missing solve!, Jacobi.jl:7) the call returns
// TL_ERR_REFERENCE_THROWS.  The presteps' halo update touches only the fields
// diffuse! marked (energy, density), which the solve does not change, so it
// is left out.
//
// Tealeaf mode runs the intended algorithms (the fixes are listed beside each
// solver in the CPU restatement): the CG phase is the fused CG loop; at the
// switch the host computes the eigenvalue estimate of the Lanczos
// tridiagonal and the Chebyshev coefficients (a few hundred scalars) and the
// device loop takes over again.
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "tl_solvers.h"
#include "tl_walk.cuh"

using namespace tl;

namespace {

struct PhaseState {
  double theta, rro;
  int cheby_iters, est_iters, first, switch_rule, set_rro;
};

__global__ void k_set_phase(DevScalars *sc, PhaseState s) {
  sc->theta = s.theta;
  sc->cheby_iters = s.cheby_iters;
  sc->est_iters = s.est_iters;
  sc->first = s.first;
  sc->switch_rule = s.switch_rule;
  if (s.set_rro == 1) sc->rro = s.rro;
  if (s.set_rro == 2) sc->rro = sc->red[0];  // the r.r just reduced
  sc->done = 0;
  sc->switched = 0;
}

__global__ void k_set_est(DevScalars *sc, int est) { sc->est_iters = est; }

// Jacobi init! (Jacobi.jl:44-46): u0 = u = energy * density on the whole array.
__global__ void k_jacobi_pre(Fields F, Geom g) {
  const long long n = (long long)g.X * g.Y;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const size_t c = g.full((int)(k % g.X), (int)(k / g.X));
    const double t = tl::dmul(F.energy[c], F.density[c]);
    F.u0[c] = t;
    F.u[c] = t;
  }
}

__global__ void k_jacobi_start(DevScalars *sc) {
  sc->iter = 0;
  sc->done = 0;
  sc->converged = 0;
  sc->switched = 0;
  sc->error = ERROR_START;
}

int grid_for(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152LL * 32) b = 152LL * 32;
  return (int)(b < 1 ? 1 : b);
}

// ---- the eigenvalue estimate (kernels.jl:19-51) on the host ---------------

int sturm_count(const double *d, const double *e, int n, double x) {
  int count = 0;
  double q = 1.0;
  for (int i = 0; i < n; ++i) {
    const double off = (i == 0) ? 0.0 : (e[i] * e[i]) / q;
    q = (d[i] - x) - off;
    if (q == 0.0) q = -DBL_MIN;
    if (q < 0.0) ++count;
  }
  return count;
}

// k-th smallest eigenvalue of the symmetric tridiagonal (d, e) by bisection
// on the Gershgorin interval (a fixed 200 halvings).
double tri_eig_bisect(const double *d, const double *e, int n, int k) {
  double lo = d[0], hi = d[0];
  for (int i = 0; i < n; ++i) {
    const double rad = (i > 0 ? fabs(e[i]) : 0.0) + (i + 1 < n ? fabs(e[i + 1]) : 0.0);
    if (d[i] - rad < lo) lo = d[i] - rad;
    if (d[i] + rad > hi) hi = d[i] + rad;
  }
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (sturm_count(d, e, n, mid) > k) hi = mid;
    else lo = mid;
  }
  return 0.5 * (lo + hi);
}

int eigenvalues(tl_ctx *ctx, int cgiters, double *emin, double *emax) {
  const int n = cgiters;
  if (n < 1) {
    tl_set_error(ctx, "no CG iterations for the eigenvalue estimate");
    return TL_ERR_EIGEN;
  }
  std::vector<double> al(n + 1), be(n + 1), d(n), e(n + 1, 0.0);
  CK(cudaMemcpy(al.data(), ctx->F.cgalpha, sizeof(double) * (n + 1), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(be.data(), ctx->F.cgbeta, sizeof(double) * (n + 1), cudaMemcpyDeviceToHost));
  for (int ii = 1; ii <= n; ++ii) {  // kernels.jl:20-31, 1-based tables
    d[ii - 1] = 1.0 / al[ii];
    if (ii > 1) d[ii - 1] += be[ii - 1] / al[ii - 1];
    if (ii < n) e[ii] = sqrt(be[ii]) / al[ii];
  }
  *emin = tri_eig_bisect(d.data(), e.data(), n, 0);
  *emax = tri_eig_bisect(d.data(), e.data(), n, n - 1);
  if (*emin < 0 || *emax < 0 || !(*emin == *emin) || !(*emax == *emax)) {
    tl_set_error(ctx, "Negative eigenvalue found: (%g, %g) (src/kernels.jl:42)", *emin, *emax);
    return TL_ERR_EIGEN;
  }
  *emin *= 0.95;  // kernels.jl:47-48
  *emax *= 1.05;
  return TL_OK;
}

// coef! (Cheby.jl:121-135) into the device tables (1-based).
int cheby_coef(tl_ctx *ctx, double emin, double emax, int n, double *theta) {
  if (n > ctx->cfg.maxiters + 1) n = ctx->cfg.maxiters + 1;
  *theta = (emax + emin) / 2;
  const double delta = (emax - emin) / 2;
  const double sigma = *theta / delta;
  double rho_o = 1 / sigma;
  std::vector<double> a(n + 1, 0.0), b(n + 1, 0.0);
  for (int ii = 1; ii <= n; ++ii) {
    const double rho_n = 1 / (2 * sigma - rho_o);
    a[ii] = rho_n * rho_o;
    b[ii] = 2 * rho_n / delta;
    rho_o = rho_n;
  }
  if (n >= 1) {
    CK(cudaMemcpyAsync(ctx->F.chebyalpha, a.data(), sizeof(double) * (n + 1), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->F.chebybeta, b.data(), sizeof(double) * (n + 1), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return TL_OK;
}

// calciter (Cheby.jl:109-118); a non-finite estimate becomes 0.
int calciter(double emin, double emax, double error, double bb) {
  const double connum = emax / emin;
  const double ita = DBL_EPSILON * bb / (4 * error);
  const double gamma = (sqrt(connum) - 1) / (sqrt(connum) + 1);
  const double est = nearbyint((log(ita) / log(10.0)) / (2 * (log(gamma) / log(10.0))));
  if (!(est == est) || fabs(est) > 2147483647.0) return 0;
  return (int)est;
}

int set_phase(tl_ctx *ctx, double theta, int cheby_iters, int est, int first, int rule, int set_rro, double rro) {
  PhaseState s;
  s.theta = theta;
  s.rro = rro;
  s.cheby_iters = cheby_iters;
  s.est_iters = est;
  s.first = first;
  s.switch_rule = rule;
  s.set_rro = set_rro;
  k_set_phase<<<1, 1, 0, ctx->stream>>>(ctx->F.sc, s);
  CKL();
  return TL_OK;
}

// CG presteps.  Reference mode: the reference's CG steps (Cheby with its
// stale rro).  Tealeaf mode: CG.init! with the halo of u, p and copyu, the
// fused CG loop, then the last step's p! and halo.  On return the host
// scalars hold the loop's end state.
int cg_phase(tl_ctx *ctx, double rx, double ry, const tl_params *prm, int exact, int stale_rro) {
  const int ref = ctx->cfg.mode == TL_MODE_REFERENCE;
  int rc = tl_cg_init(ctx, rx, ry, prm->coefficient, exact);
  if (rc) return rc;
  if ((rc = tl_set_loop_params(ctx, prm, 1, stale_rro))) return rc;
  if (!ref) {
    const int up[2] = {TL_EX_U, TL_EX_P};
    if ((rc = tl_halo_update(ctx, 1, up, 2, 1))) return rc;
    if ((rc = tl_copy_u(ctx))) return rc;
  }
  ctx->last_solve_ms = 0.0;
  if (prm->maxiters >= 1) {
    const int which = ref ? TL_GRAPH_CG_REF_NOHALO : (exact ? TL_GRAPH_CG_EXACT : TL_GRAPH_CG_FAST);
    if ((rc = tl_run_graph(ctx, which, &ctx->last_solve_ms))) return rc;
  }
  if ((rc = tl_read_scalars(ctx))) return rc;
  if (!ref && prm->maxiters >= 1) {
    const double *pcur = (ctx->host_sc->iter & 1) ? ctx->F.pb : ctx->F.p;
    launch_tl_p(ctx->stream, ctx->F, ctx->g, tl_walk_for(ctx, exact), pcur, ctx->F.p, exact);
    CKL();
    if ((rc = tl_halo_update(ctx, 1, nullptr, -1, 1))) return rc;
  }
  return TL_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// loop bodies
// ---------------------------------------------------------------------------

int tl_record_solver_body(tl_ctx *ctx, int which, cudaGraphConditionalHandle h) {
  const Fields &F = ctx->F;
  const Geom &g = ctx->g;
  cudaStream_t st = ctx->stream;
  switch (which) {
    case TL_GRAPH_CHEBY_EXACT:
    case TL_GRAPH_CHEBY_FAST: {
      const int exact = which == TL_GRAPH_CHEBY_EXACT;
      const Walk &wk = exact ? ctx->walk_exact : ctx->walk_w64;
      launch_cheby_step(st, F, g, wk, F.ub, F.u, exact, 0, 0, h, 0);
      launch_cheby_step(st, F, g, wk, F.u, F.ub, exact, 1, 0, h, 1);
      break;
    }
    case TL_GRAPH_PPCG_EXACT:
    case TL_GRAPH_PPCG_FAST: {
      const int exact = which == TL_GRAPH_PPCG_EXACT;
      const Walk &ww = exact ? ctx->walk_exact : ctx->walk_w64;
      const Walk &wu = exact ? ctx->walk_exact : ctx->walk_ur64;
      const int n = ctx->ppcg_graph_inner;
      for (int outer = 0; outer < 2; ++outer) {
        const int guard = outer;
        double *pin = outer ? F.pb : F.p, *pout = outer ? F.p : F.pb;
        launch_tl_w(st, F, g, ww, pin, pout, exact, guard, 0);
        launch_ppcg_ur(st, F, g, wu, pout, F.sd, exact, guard);
        for (int pp = 1; pp <= n; ++pp) {
          const double *src = (pp & 1) ? F.sd : F.sdb;
          double *dst = (pp & 1) ? F.sdb : F.sd;
          const int last = pp == n;
          launch_ppcg_inner(st, F, g, ww, src, dst, pp, last, exact, guard, h, last && outer == 1);
        }
      }
      break;
    }
    case TL_GRAPH_JACOBI:
    case TL_GRAPH_JACOBI_FAST: {
      const int exact = which == TL_GRAPH_JACOBI;
      const Walk &wk = exact ? ctx->walk_exact : ctx->walk_w64;
      const Walk &wc = ctx->walk_exact;
      launch_jacobi(st, F, g, wk, F.u, F.ub, 0, exact);
      launch_jacobi_check(st, F, g, wc, F.ub, 0, h, 0);
      launch_jacobi(st, F, g, wk, F.ub, F.u, 1, exact);
      launch_jacobi_check(st, F, g, wc, F.u, 1, h, 1);
      break;
    }
    default:
      tl_set_error(ctx, "no loop body %d", which);
      return TL_ERR_ARG;
  }
  return cudaGetLastError() == cudaSuccess ? TL_OK : TL_ERR_CUDA;
}

static void fill_result(tl_ctx *ctx, tl_result *res, int cg_iters) {
  const DevScalars &sc = *ctx->host_sc;
  res->iters = sc.iter;
  res->cg_iters = cg_iters;
  res->inner_iters = sc.iter - cg_iters;
  res->error = sc.error;
  res->converged = sc.converged;
  res->rel_residual = -1.0;
  res->launches = (int)ctx->launches;
}

// ---------------------------------------------------------------------------
// Chebyshev
// ---------------------------------------------------------------------------

int tl_cheby_solve(tl_ctx *ctx, double rx, double ry, const tl_params *prm, tl_result *res) {
  const int ref = ctx->cfg.mode == TL_MODE_REFERENCE;
  const int exact = ref || prm->exact;
  // FP32 inner sweeps inside FP64 refinement, for the presteps and the
  // Chebyshev steps (tealeaf mode; exact implies FP64)
  const int fp32 = prm->precision == TL_PREC_FP32_IR && !exact;
  int rc, pre_ref = 0;
  if (fp32) {
    double rr = 0.0, rel = -1.0;
    int sw = 0;
    if ((rc = tl_ir_presteps(ctx, rx, ry, prm, &pre_ref, &rr, &rel, &sw))) return rc;
    if (!sw) {  // converged or out of iterations during the presteps
      fill_result(ctx, res, ctx->host_sc->iter);
      res->refinements = pre_ref;
      res->rel_residual = rel;
      res->converged = rel >= 0 && rel < prm->eps;
      return TL_OK;
    }
  } else {
    if ((rc = cg_phase(ctx, rx, ry, prm, exact, ref ? 1 : 0))) return rc;  // Cheby.jl:33 passes the init rro
    const DevScalars sc0 = *ctx->host_sc;
    if (!sc0.switched) {  // converged or out of iterations during the presteps
      fill_result(ctx, res, sc0.iter);
      res->error = prm->maxiters >= 1 ? sc0.error : ERROR_START;
      return TL_OK;
    }
  }
  const DevScalars sc0 = *ctx->host_sc;
  if (ref) {
    res->iters = sc0.iter + 1;
    res->cg_iters = sc0.iter;
    res->error = sc0.error;
    tl_set_error(ctx, "MethodError: no method matching minmax(::Vector{Float64}) (src/kernels.jl:39)");
    return TL_ERR_REFERENCE_THROWS;
  }
  // the switch (Cheby.jl:38-46)
  const int cgiters = sc0.iter;
  double emin, emax, theta;
  if ((rc = eigenvalues(ctx, cgiters, &emin, &emax))) return rc;
  if ((rc = cheby_coef(ctx, emin, emax, prm->maxiters - cgiters + 1, &theta))) return rc;
  if ((rc = set_phase(ctx, theta, 0, 0, 0, 2, 0, 0.0))) return rc;
  launch_cheby_init(ctx->stream, ctx->F, ctx->g, theta);
  CKL();
  const int fu = TL_EX_U;
  if ((rc = tl_halo_update(ctx, 1, &fu, 1, 1))) return rc;  // Cheby.jl:78
  const Walk &wk = exact ? ctx->walk_exact : ctx->walk_w64;
  launch_cheby_step(ctx->stream, ctx->F, ctx->g, wk, ctx->F.u, ctx->F.ub, exact, 0, 1, 0, 0);
  CKL();
  if ((rc = tl_read_scalars(ctx))) return rc;
  const int est = calciter(emin, emax, ctx->host_sc->error, ctx->host_sc->bb);
  k_set_est<<<1, 1, 0, ctx->stream>>>(ctx->F.sc, est);
  CKL();
  if (!ctx->host_sc->done && fp32) {
    // the rest of the iteration in FP32 inside FP64 refinement
    int nref = 0;
    double rel = -1.0;
    if ((rc = tl_cheby32_run(ctx, prm, &nref, &rel))) return rc;
    const int ex = TL_EX_U;
    if ((rc = tl_halo_update(ctx, 1, &ex, 1, 1))) return rc;
    if ((rc = tl_read_scalars(ctx))) return rc;
    fill_result(ctx, res, cgiters);
    res->inner_iters = ctx->host_sc->cheby_iters;
    res->est_iters = est;
    res->eigmin = emin;
    res->eigmax = emax;
    res->refinements = pre_ref + nref;
    res->rel_residual = rel;
    res->converged = rel >= 0 && rel < prm->eps;
    return TL_OK;
  }
  if (!ctx->host_sc->done) {
    if ((rc = tl_run_graph(ctx, exact ? TL_GRAPH_CHEBY_EXACT : TL_GRAPH_CHEBY_FAST, &ctx->last_solve_ms))) return rc;
    if ((rc = tl_read_scalars(ctx))) return rc;
  }
  // u is in ub after an odd number of Chebyshev steps
  if (ctx->host_sc->cheby_iters & 1) {
    launch_copy_interior(ctx->stream, ctx->F.u, ctx->F.ub, ctx->g);
    CKL();
  }
  if ((rc = tl_halo_update(ctx, 1, nullptr, -1, 1))) return rc;
  if ((rc = tl_read_scalars(ctx))) return rc;
  fill_result(ctx, res, cgiters);
  res->inner_iters = ctx->host_sc->cheby_iters;
  res->est_iters = est;
  res->eigmin = emin;
  res->eigmax = emax;
  return TL_OK;
}

// ---------------------------------------------------------------------------
// PPCG
// ---------------------------------------------------------------------------

int tl_ppcg_solve(tl_ctx *ctx, double rx, double ry, const tl_params *prm, tl_result *res) {
  const int ref = ctx->cfg.mode == TL_MODE_REFERENCE;
  const int exact = ref || prm->exact;
  if (prm->ppcginnersteps < 1) {
    tl_set_error(ctx, "ppcginnersteps %d: PPCG needs at least one inner sweep", prm->ppcginnersteps);
    return TL_ERR_ARG;
  }
  // FP32 inner sweeps inside FP64 refinement, for the presteps and the PPCG
  // steps (tealeaf mode; exact implies FP64)
  const int fp32 = prm->precision == TL_PREC_FP32_IR && !exact;
  int rc, pre_ref = 0;
  double pre_rr = 0.0;
  if (fp32) {
    double rel = -1.0;
    int sw = 0;
    if ((rc = tl_ir_presteps(ctx, rx, ry, prm, &pre_ref, &pre_rr, &rel, &sw))) return rc;
    if (!sw) {  // converged or out of iterations during the presteps
      fill_result(ctx, res, ctx->host_sc->iter);
      res->refinements = pre_ref;
      res->rel_residual = rel;
      res->converged = rel >= 0 && rel < prm->eps;
      return TL_OK;
    }
  } else {
    if ((rc = cg_phase(ctx, rx, ry, prm, exact, 0))) return rc;
    const DevScalars sc0 = *ctx->host_sc;
    if (!sc0.switched) {
      fill_result(ctx, res, sc0.iter);
      res->error = prm->maxiters >= 1 ? sc0.error : ERROR_START;
      return TL_OK;
    }
  }
  const DevScalars sc0 = *ctx->host_sc;
  if (ref) {
    res->iters = sc0.iter + 1;
    res->cg_iters = sc0.iter;
    res->error = sc0.error;
    tl_set_error(ctx, "UndefVarError: ++ not defined (src/solvers/PPCG.jl:36)");
    return TL_ERR_REFERENCE_THROWS;
  }
  const int cgiters = sc0.iter;
  const int n = prm->ppcginnersteps;
  double emin, emax, theta;
  if ((rc = eigenvalues(ctx, cgiters, &emin, &emax))) return rc;  // PPCG.jl:41-42
  if ((rc = cheby_coef(ctx, emin, emax, n, &theta))) return rc;
  if (fp32) {
    // the presteps' last refinement measured the true residual, which
    // init! (PPCG.jl:58-61) would compute here
    if ((rc = set_phase(ctx, theta, 0, 0, 0, 2, 0, 0.0))) return rc;
    int nref = 0;
    double rel = -1.0;
    if ((rc = tl_ppcg32_run(ctx, prm, pre_rr, &nref, &rel))) return rc;
    const int up[2] = {TL_EX_U, TL_EX_P};
    if ((rc = tl_halo_update(ctx, 1, up, 2, 1))) return rc;
    if ((rc = tl_read_scalars(ctx))) return rc;
    fill_result(ctx, res, cgiters);
    res->inner_iters = ctx->host_sc->cheby_iters;
    res->eigmin = emin;
    res->eigmax = emax;
    res->refinements = pre_ref + nref;
    res->rel_residual = rel;
    res->converged = rel >= 0 && rel < prm->eps;
    return TL_OK;
  }
  // init!: residual!, rro = r.r, halo of p (PPCG.jl:58-61)
  launch_residual(ctx->stream, ctx->F, ctx->g, TL_MODE_TEALEAF);
  launch_norm_r(ctx->stream, ctx->F, ctx->g, ctx->walk_exact);
  CKL();
  if ((rc = set_phase(ctx, theta, 0, 0, 1, 2, 2, 0.0))) return rc;
  const int fp = TL_EX_P;
  if ((rc = tl_halo_update(ctx, 1, &fp, 1, 1))) return rc;
  const int which = exact ? TL_GRAPH_PPCG_EXACT : TL_GRAPH_PPCG_FAST;
  if (ctx->ppcg_graph_inner != n) {  // the recorded sweeps depend on the inner step count
    for (int k = TL_GRAPH_PPCG_EXACT; k <= TL_GRAPH_PPCG_FAST; ++k)
      if (ctx->graph[k]) {
        cudaGraphExecDestroy(ctx->graph[k]);
        ctx->graph[k] = nullptr;
      }
    ctx->ppcg_graph_inner = n;
  }
  if ((rc = tl_run_graph(ctx, which, &ctx->last_solve_ms))) return rc;
  if ((rc = tl_read_scalars(ctx))) return rc;
  const int outer = ctx->host_sc->cheby_iters;
  // the last outer step's p! and halo of p (PPCG.jl:92-93, 31)
  const double *pcur = (outer & 1) ? ctx->F.pb : ctx->F.p;
  launch_tl_p(ctx->stream, ctx->F, ctx->g, tl_walk_for(ctx, exact), pcur, ctx->F.p, exact);
  CKL();
  {  // sd: the last sweep's output, with the halo of the one before
    const double *fin = (n & 1) ? ctx->F.sdb : ctx->F.sd;
    const double *prev = (n & 1) ? ctx->F.sd : ctx->F.sdb;
    launch_ppcg_sd_final(ctx->stream, ctx->F, ctx->g, fin, prev);
    CKL();
  }
  if ((rc = tl_halo_update(ctx, 1, &fp, 1, 1))) return rc;
  if ((rc = tl_read_scalars(ctx))) return rc;
  fill_result(ctx, res, cgiters);
  res->inner_iters = outer;
  res->eigmin = emin;
  res->eigmax = emax;
  return TL_OK;
}

// ---------------------------------------------------------------------------
// Jacobi
// ---------------------------------------------------------------------------

int tl_jacobi_solve(tl_ctx *ctx, double rx, double ry, const tl_params *prm, tl_result *res) {
  if (ctx->cfg.mode == TL_MODE_REFERENCE) {
    tl_set_error(ctx, "UndefVarError: solve! not defined in module Jacobi (src/TeaLeaf.jl:74, "
                      "src/solvers/Jacobi.jl:7)");
    return TL_ERR_REFERENCE_THROWS;
  }
  if (prm->coefficient < TL_CONDUCTIVITY) {
    tl_set_error(ctx, "Coefficient %d is not valid. (src/solvers/Jacobi.jl:35)", prm->coefficient);
    return TL_ERR_COEF;
  }
  const Geom &g = ctx->g;
  k_jacobi_pre<<<grid_for((long long)g.X * g.Y), 256, 0, ctx->stream>>>(ctx->F, g);
  CKL();
  launch_init_coef(ctx->stream, ctx->F, g, rx, ry, 1, prm->coefficient);
  CKL();
  const int exact = prm->exact || ctx->cfg.mode == TL_MODE_REFERENCE;
  if (!exact) {
    launch_init_rdiag(ctx->stream, ctx->F, g);
    CKL();
  }
  if (tl_copy_u(ctx)) return TL_ERR_CUDA;
  launch_copy_full(ctx->stream, ctx->F.r, ctx->F.u, g);  // r's corners and outer layers: the first r .= u
  CKL();
  for (int k = 0; k < TL_NEX; ++k) ctx->toexchange[k] = 0;  // Jacobi.jl:54-55 marks u
  ctx->toexchange[TL_EX_U] = 1;
  int rc;
  if ((rc = tl_set_loop_params(ctx, prm, 2, 0))) return rc;
  k_jacobi_start<<<1, 1, 0, ctx->stream>>>(ctx->F.sc);
  CKL();
  ctx->last_solve_ms = 0.0;
  if (prm->maxiters >= 1) {
    if ((rc = tl_run_graph(ctx, exact ? TL_GRAPH_JACOBI : TL_GRAPH_JACOBI_FAST, &ctx->last_solve_ms))) return rc;
  }
  if ((rc = tl_read_scalars(ctx))) return rc;
  if (ctx->host_sc->iter & 1) {
    launch_copy_interior(ctx->stream, ctx->F.u, ctx->F.ub, g);
    CKL();
  }
  if ((rc = tl_halo_update(ctx, 1, nullptr, -1, 1))) return rc;
  if ((rc = tl_read_scalars(ctx))) return rc;
  fill_result(ctx, res, 0);
  res->inner_iters = 0;
  return TL_OK;
}
