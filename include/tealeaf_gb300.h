/*
 * tealeaf_gb300.h -- C ABI of the GB300 (sm_103a) TeaLeaf solve library.
 *
 * The library replaces the solve path of Laura7089/TeaLeaf.jl: the solver
 * plugins called as `set.solver.solve!(chunk, set, rx, ry)`
 * (src/TeaLeaf.jl:74) and the kernels they drive (src/kernels.jl).  A caller
 * (the Julia shim, the Python host mirror, a C driver) owns one tl_ctx per
 * Chunk; the context keeps every field resident in HBM across timesteps and
 * host arrays are only borrowed for the duration of an upload/download.
 *
 * Conventions
 *  - every entry point returns an int status (TL_OK == 0); tl_last_error()
 *    gives the message of the last failure on that context;
 *  - host field arrays use the reference's Chunk layout (src/chunk.jl:19-38):
 *    Float64, column-major (X, Y), X = xcells + 2*halodepth, with a leading
 *    dimension ld >= X;
 *  - a context is not thread-safe; all work runs on the context's stream.
 */
#ifndef TEALEAF_GB300_H
#define TEALEAF_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define TL_API_VERSION 1

typedef struct tl_ctx tl_ctx;

/* status codes */
enum {
  TL_OK = 0,
  TL_ERR_ARG = 1,               /* invalid argument or size                                  */
  TL_ERR_CUDA = 2,              /* CUDA runtime error (message names the call)               */
  TL_ERR_COEF = 3,              /* invalid coefficient: src/solvers/CG.jl:48-50, Jacobi.jl:34-36 */
  TL_ERR_EIGEN = 4,             /* negative eigenvalue estimate: src/kernels.jl:41-43        */
  TL_ERR_REFERENCE_THROWS = 5,  /* reference mode reached a statement where the reference raises */
  TL_ERR_NOMEM = 6,             /* device allocation failed                                  */
  TL_ERR_STATE = 7              /* call out of order (e.g. solve before initialise)          */
};

/* Chunk fields, in the order of the reference's Chunk struct (src/chunk.jl:24-38), plus volume (:46) */
enum {
  TL_DENSITY0 = 0, TL_DENSITY, TL_ENERGY0, TL_ENERGY, TL_U, TL_U0, TL_P, TL_R, TL_MI, TL_W, TL_KX, TL_KY,
  TL_SD, TL_VOLUME, TL_NFIELDS
};

/* EXCHANGE_FIELDS (src/chunk.jl:12) */
enum { TL_EX_DENSITY = 0, TL_EX_P, TL_EX_ENERGY0, TL_EX_ENERGY, TL_EX_U, TL_EX_SD, TL_NEX };

/* semantics */
enum {
  TL_MODE_REFERENCE = 0,  /* the reference as written: diagonal smvp, off-by-one halo, transposed geometry */
  TL_MODE_TEALEAF = 1     /* the intended algorithm: 5-point operator, reflective halo                    */
};

enum { TL_SOLVER_CG = 0, TL_SOLVER_CHEBY = 1, TL_SOLVER_PPCG = 2, TL_SOLVER_JACOBI = 3 };
enum { TL_CONDUCTIVITY = 1, TL_RECIP_CONDUCTIVITY = 2 };     /* src/settings.jl:13-14 */
enum { TL_GEOM_RECTANGULAR = 0, TL_GEOM_CIRCULAR = 1, TL_GEOM_POINT = 2 };
enum {
  TL_CRIT_REFERENCE = 0,  /* each solver's own test: CG sqrt|rr| < eps (CG.jl:24), others |error| < eps */
  TL_CRIT_RELATIVE = 1    /* sqrt(rr / (u0.u0)) < eps on the recursive residual, then checked on the true one */
};
/* TL_PREC_FP32_IR (tealeaf mode, fused kernels): CG, Chebyshev and PPCG
 * (their CG presteps included) iterate in FP32 inside FP64 refinement to the
 * relative true residual; also in tl_batch_solve (CG).  Jacobi stays FP64. */
enum { TL_PREC_FP64 = 0, TL_PREC_FP32_IR = 1 };

/* Chunk(settings) (src/chunk.jl:68-89) */
typedef struct {
  int xcells, ycells, halodepth;
  int maxiters;             /* length of the cg/cheby coefficient tables */
  double xmin, ymin, dx, dy;
  int mode;                 /* TL_MODE_* */
} tl_config;

/* State (src/settings.jl:20-29) with the bounds already inset by the caller
 * (src/settings.jl:159-162). */
typedef struct {
  double density, energy, xmin, ymin, xmax, ymax, radius;
  int geometry;
} tl_state;

/* The Settings fields a solve reads (src/settings.jl:39-78) */
typedef struct {
  int solver;               /* TL_SOLVER_*                                   */
  int coefficient;          /* TL_CONDUCTIVITY / TL_RECIP_CONDUCTIVITY       */
  int maxiters;             /* <= tl_config.maxiters                         */
  int presteps;             /* Cheby/PPCG CG steps before the switch         */
  int ppcginnersteps;
  int errorswitch;
  double eps;
  double epslim;
  int criterion;            /* TL_CRIT_*                                     */
  int precision;            /* TL_PREC_*                                     */
  int exact;                /* 1: tealeaf mode reproduces the reference's operation order with no FMA
                               contraction (bit-identical to the CPU restatement); 0: fused FMA kernels */
  int warmstart;            /* CG in tealeaf mode, the start when it beats the plain start u^n by
                               residual: 0 off; TL_WARM_NETWORK: the A-norm projection onto u^n, the
                               last TL_WARM_HIST increments and the warm-start network's correction
                               (tl_warm_load); TL_WARM_HISTORY: the same projection without the
                               network; TL_WARM_EXTRAPOLATE: u^n + (u^n - u^{n-1}) */
} tl_params;
enum { TL_WARM_OFF = 0, TL_WARM_NETWORK = 1, TL_WARM_EXTRAPOLATE = 2, TL_WARM_HISTORY = 3 };
#define TL_WARM_HIST 6      /* earlier right-hand sides the warm-start projection keeps */

typedef struct {
  int iters;                /* trips of the solver's main loop                  */
  int cg_iters;             /* CG iterations (presteps for Cheby/PPCG)          */
  int inner_iters;          /* Chebyshev / PPCG iterations after the switch     */
  int est_iters;            /* Chebyshev iteration estimate (Cheby.jl:109-118)  */
  double error;             /* the solver loop's final error value              */
  double eigmin, eigmax;    /* eigenvalue estimates (Cheby/PPCG)                */
  int converged;            /* the loop ended on its convergence test           */
  int refinements;          /* FP64 refinement passes (TL_PREC_FP32_IR)         */
  double rel_residual;      /* ||u0 - A u|| / ||u0|| after the solve (TL_CRIT_RELATIVE), else -1 */
  int launches;             /* kernels this solve launched (graph-body kernels counted per trip) */
  int warm;                 /* 0: plain start (no warm start asked or no previous step), 1: the
                               prediction was used, 2: the prediction lost to the plain start,
                               3 (TL_WARM_NETWORK): the projection without the network's term had
                               the smaller residual and was used */
  double r0_plain;          /* ||u0 - A u^n|| / ||u0|| of the plain start (warm start asked), else -1 */
  double r0_pred;           /* the same for the prediction, -1 when none was made */
  double warm_coef[TL_WARM_HIST + 2]; /* the prediction's weights on u^n, u^{n-1}, ..., u^{n-TL_WARM_HIST}
                               and on the network's correction g (u^n - u^{n-1}); zero when none */
} tl_result;

/* Creation.  Replaces Chunk(set) (src/chunk.jl:68-89): allocates every field
 * in HBM, zeroed, volume = dx*dy. */
int tl_create(tl_ctx **out, const tl_config *cfg);
int tl_destroy(tl_ctx *ctx);
const char *tl_last_error(const tl_ctx *ctx);

/* Host <-> device copies of one field (column-major (X, Y), leading dimension ld). */
int tl_upload(tl_ctx *ctx, int field, const double *host, int ld);
int tl_download(tl_ctx *ctx, int field, double *host, int ld);

/* setchunkstate! (src/chunk.jl:122-151) */
int tl_set_states(tl_ctx *ctx, const tl_state *states, int nstates);

/* initialiseapp! (src/TeaLeaf.jl:35-44): states, halo of density, energy0,
 * energy, then energy = energy0. */
int tl_initialise(tl_ctx *ctx, const tl_state *states, int nstates);

/* haloupdate!(chunk, set, depth[, toex][, reset]) (src/kernels.jl:146-159):
 * nfields >= 0 marks `fields` (TL_EX_*) for exchange (clearing the others
 * first when reset != 0) and updates them; nfields < 0 updates the fields
 * currently marked. */
int tl_halo_update(tl_ctx *ctx, int depth, const int *fields, int nfields, int reset);

/* solve!(chunk, set, rx, ry): CG.jl:7-29, Cheby.jl:10-61, PPCG.jl:9-55,
 * Jacobi.jl:7-30. */
int tl_solve(tl_ctx *ctx, double rx, double ry, const tl_params *params, tl_result *result);

/* solvefinished! (src/kernels.jl:166-170) */
int tl_solve_finished(tl_ctx *ctx, int checkresult);

/* fieldsummary (src/kernels.jl:119-133): out = {vol, mass, ie, temp} over the
 * interior; temp is the reference's quantity, the other three are added. */
int tl_field_summary(tl_ctx *ctx, double out[4]);

/* diffuse! (src/TeaLeaf.jl:62-83) inside the library: for each of `nsteps`
 * timesteps, rx = dt/dx^2, ry = dt/dy^2, the halo of energy and density, the
 * solve, solvefinished!, and the field summary every `summaryfrequency`
 * steps and after the last.  results[nsteps]; summaries[4 * n] receives up
 * to `maxsummaries` summaries, *nsummaries how many were taken (checkresult
 * 0 takes none, like fieldsummary). */
int tl_diffuse(tl_ctx *ctx, const tl_params *params, double dt, int nsteps, int summaryfrequency, int checkresult,
               tl_result *results, double *summaries, int maxsummaries, int *nsummaries);

/* copyu! (src/kernels.jl:217-220), residual! (:227-232), finalise! (:239-242) */
int tl_copy_u(tl_ctx *ctx);
int tl_residual(tl_ctx *ctx);
int tl_finalise(tl_ctx *ctx);

/* CG coefficient tables cgalpha[1..n], cgbeta[1..n] (src/chunk.jl:56-57) */
int tl_get_cg_coefficients(tl_ctx *ctx, double *alpha, double *beta, int n);

/* Launch layout of the deterministic reduction tree: warps per block, rows
 * per tile, persistent blocks.  Lets a checker reproduce the summation order. */
int tl_reduction_layout(tl_ctx *ctx, int *warps, int *rows, int *blocks);

/* Launch layout (warps per block, rows per tile, persistent blocks) of one
 * fused iteration kernel (ids as in tl_bench_kernel): get the autotuned
 * choice, or override it (both for tuning studies; a set layout holds until
 * the context is destroyed). */
int tl_get_layout(tl_ctx *ctx, int kernel, int *warps, int *rows, int *blocks);
int tl_set_layout(tl_ctx *ctx, int kernel, int warps, int rows, int blocks);

/* Wait for all work queued on the context. */
int tl_synchronize(tl_ctx *ctx);

/* Device time in milliseconds of the iteration loop of the last tl_solve. */
int tl_last_solve_ms(tl_ctx *ctx, double *ms);

/* A device timer on the context stream (CUDA events): stop returns the
 * milliseconds since start. */
int tl_timer_start(tl_ctx *ctx);
int tl_timer_stop(tl_ctx *ctx, double *ms);

/* Times `reps` back-to-back launches of one fused iteration kernel (0: the CG
 * p-update + stencil + p.w step, 1: the u/r update + r.r step, 4: the
 * Chebyshev step, 5: a PPCG inner sweep, 6: the FP32 Chebyshev step, 7: an
 * FP32 PPCG inner sweep, 8: the FP32 CG direction step p' = beta p + r with
 * p'.A p', 9: the FP32 CG update step with A p' recomputed; 8 and 9 are the
 * FP32 CG iteration; 10: a Jacobi sweep, 11: the depth-1 halo update of u and
 * p, 12: PPCG's outer u/r update; 2 and 3, an earlier FP32 pair, are retired
 * and return TL_ERR_ARG) on the current fields; for roofline measurements.  The launches overwrite
 * solver work fields (p, w, r, u, sd, their second buffers and the FP32
 * copies): call it after the solves whose fields matter. */
int tl_bench_kernel(tl_ctx *ctx, int kernel, int reps, double *ms_per_launch);

/* Many independent decks (tealeaf-mode contexts of any sizes on the current
 * device) solved by the fused FP64 CG in one graph launch: the persistent
 * blocks are shared over the decks in proportion to their cells, a converged
 * deck drops out (per-deck convergence mask) and its blocks go to the decks
 * still running.  Each deck's solve is CG.solve! (src/solvers/CG.jl:7-29)
 * with that deck's rx[k], ry[k]; results[k] is the deck's result.  The batch
 * borrows the contexts: destroy it before them. */
typedef struct tl_batch tl_batch;
int tl_batch_create(tl_batch **out, tl_ctx *const *ctxs, int n);
int tl_batch_destroy(tl_batch *batch);
const char *tl_batch_last_error(const tl_batch *batch);
int tl_batch_solve(tl_batch *batch, const double *rx, const double *ry, const tl_params *params, tl_result *results);
int tl_batch_last_ms(tl_batch *batch, double *ms);  /* device time of the last batched iteration loop */

/* Field summary {vol, mass, ie, temp} of caller-owned device arrays, with no
 * device allocation by the library.  No counterpart in the reference: it is
 * for callers that cannot let a library call cudaMalloc, such as a host
 * framework that owns all device memory through its own pool and hands
 * libraries ready-made buffers, or a driver that must not pay for the device
 * synchronisation that cudaFree implies.
 *
 * volume, density, energy, u: device pointers to element (0, 0) of pitched
 * (X, Y) arrays, X = xcells + 2*halodepth, `pitch` doubles between columns;
 * out: device pointer to 4 doubles; stream: a cudaStream_t (NULL = legacy
 * default stream); err/errlen: optional buffer for the error message.
 * Limits: at most 2147483647 interior cells per call, xcells and ycells at
 * most 1073741824 each and halodepth at most 1048576; larger sizes are
 * rejected with TL_ERR_ARG.
 * The reduction scratch (4 x 1024 block partials and a ticket, about 33 KB)
 * is a static device array: each GPU that loads the library holds it until
 * the process exits.  The first call in each device context looks up its
 * address (cudaGetSymbolAddress) with that device current, so make that first
 * call before any stream capture; after cudaDeviceReset the next call is a
 * first call again.  All calls on a device share the scratch: calls
 * that overlap on the GPU (different streams, no ordering) race and give
 * wrong sums.  The call is asynchronous on `stream`. */
int tl_field_summary_noalloc(const double *volume, const double *density, const double *energy, const double *u,
                             int xcells, int ycells, int halodepth, long long pitch, double *out, void *stream,
                             char *err, int errlen);

/* ---- the tea.in reader ---------------------------------------------------
 * Settings(infile) (src/settings.jl:90-135) and readstate (:142-173): `text`
 * is a deck's contents.  `deck` receives the Settings fields (the reference's
 * defaults where the deck is silent; dx, dy from the domain); states[0..n)
 * receive the first n = min(deck->nstates, maxstates) states with their bounds
 * inset as `mode` tests them (reference: dx/100 with dx as it stood when the
 * state line was read; tealeaf: the deck's final dx/100), ready for
 * tl_initialise.  Unknown keys and values that do not parse are skipped and
 * counted in deck->warnings, as the reference warns; a malformed state line
 * returns TL_ERR_ARG with the message in err.  Host only: no device work. */
typedef struct {
  long long endstep;
  int presteps, maxiters, coefficient, ppcginnersteps, summaryfrequency, halodepth, xcells, ycells;
  int errorswitch, checkresult, solver;
  double eps, dtinit, endtime, epslim, xmin, ymin, xmax, ymax, dx, dy;
  int nstates;              /* states in the deck (may exceed maxstates) */
  int warnings;             /* lines skipped with a warning */
} tl_deck;
int tl_parse_deck(const char *text, int mode, tl_deck *deck, tl_state *states, int maxstates, char *err, int errlen);

/* ---- learned warm start ------------------------------------------------
 * No counterpart in the reference.  A 6-layer 3x3 convolutional network (32
 * channels, GELU between layers, BF16 weights, FP32 accumulation on the
 * tensor cores) reads, per cell, u^n / rms(u^n), log(rx / density) / 4 and
 * (u^n - u^{n-1}) / rms(u^n - u^{n-1}) and returns a factor g; its prediction
 * of u^{n+1} is u^n + (1 + g) (u^n - u^{n-1}).  In the solve, the start is
 * the A-norm projection of the solution onto u^n, the last six increments
 * u^{n-k} - u^{n-k-1} and the network's correction g (u^n - u^{n-1}): the
 * combination closest to A^{-1} u^n in the A-norm, so never farther than the
 * plain start or the linear extrapolation.  The network's term is kept only
 * when that candidate's residual ||u^n - A x|| is below the residual of the
 * same projection without it; after a step where it was not, the next 1, 2,
 * 4, ... 32 steps (doubling with each such step, back to 1 after a step where
 * it was) skip the network.  CG starts from the prediction only when its
 * residual is below the plain start's, and must still meet eps on the true
 * residual.
 *
 * Parameter vector (FP32, TL_WARM_NPARAMS values), layer by layer:
 * W[cout][9][cin] then b[cout], with (cin, cout) = (16, 32), (32, 32) x 4,
 * (32, 16); input channels 3..15 and output channels 1..15 are padding. */
#define TL_WARM_NPARAMS (32 * 9 * 16 + 32 + 4 * (32 * 9 * 32 + 32) + 16 * 9 * 32 + 16)

/* Loads the network into the context (copies; the weights are rounded to BF16). */
int tl_warm_load(tl_ctx *ctx, const float *params, int nparams);
/* Forgets the previous step (the next warm-start solve makes no prediction). */
int tl_warm_reset(tl_ctx *ctx);

/* Building blocks of training (device pointers, asynchronous on `stream`). */
/* A crop of a deck's fields for the feature and loss kernels: pointers to
 * cell (0, 0) of the interior, `pitch` doubles between rows, crop origin
 * (ox, oy) of size given per call, inside the nx x ny domain. */
typedef struct {
  const double *u, *uprev, *rho;
  long long pitch;
  int nx, ny, ox, oy;
  double rx, ry;
  double inv_su, inv_sd;    /* 1 / rms(u), 1 / rms(u - uprev) over the domain */
} tl_warm_crop;

/* y = conv3x3(x, w) + b over N images of H x W (NHWC BF16, zero padding);
 * mode 0: out = y; 1: out = GELU(y) and z = y (z may be NULL); 2: out = y *
 * GELU'(gz) (input gradient through the previous layer's GELU; b may be NULL).
 * out32 (may be NULL) receives channel 0 of y in FP32.  (cin, cout) in
 * {(16, 32), (32, 32), (32, 16)}.  x, w, gz, z and out must be 16-byte
 * aligned and out32 4-byte aligned (TL_ERR_ARG otherwise).  Runs on the
 * tcgen05 tensor cores, the input rows staged by tensor copies
 * (TEALEAF_GB300_CONV=mma selects the warp-level mma.sync kernel). */
int tl_conv3x3_forward(const void *x, const void *w, const float *bias, const void *gz, void *z, void *out,
                       float *out32, int N, int H, int W, int cin, int cout, int mode, void *stream);
/* Synchronises the device, then returns in *timeouts the number of blocks of
 * the tcgen05 convolution whose bounded wait for their MMAs ran out since the
 * last call (0 in a correct run; such a block stops and leaves its rows
 * unwritten), and resets the count. */
int tl_conv_status(int *timeouts);
/* dw[cout][9][cin], then db[cout] = the weight and bias gradients; partials
 * holds nparts * (cout*9*cin + cout) floats.  x and dz must be 16-byte
 * aligned (TL_ERR_ARG otherwise). */
int tl_conv3x3_weight_grad(const void *x, const void *dz, float *partials, int nparts, float *dw, int N, int H, int W,
                           int cin, int cout, void *stream);
/* wt[ci][tap][co] = w[co][8 - tap][ci]: weights of the input-gradient convolution. */
int tl_conv3x3_flip(const void *w, void *wt, int cin, int cout, void *stream);
/* Adam (bias-corrected, step >= 1) on FP32 weights with gradient scale and
 * elementwise clip; wbf16 (may be NULL) receives the BF16 copy. */
int tl_adam_step(float *w, float *m, float *v, const float *grad, void *wbf16, int n, float lr, float b1, float b2,
                 float eps, int step, float clip, float gscale, void *stream);
/* feat[B][H][W][16] = the network input of B crops. */
int tl_warm_features(const tl_warm_crop *crops, int B, int H, int W, void *feat, void *stream);
/* Loss of B crops of H x W.  Per crop, term = mean((inv_sd r)^2) with
 * r = d - A((1 + g) d) over the cells at least `margin` (>= 2) from the crop
 * edge, d = u - uprev, A the 5-point operator of the crop's deck, and
 * plain = mean((inv_sd d)^2) (the plain start's value).  objective 0:
 * L = mean of the terms; 1: L = mean of log(term / plain).
 * crop_loss[2b] = term, crop_loss[2b+1] = plain; dz[B][H][W][16] = dL/dg in
 * channel 0, 0 elsewhere.  resid: B*H*W doubles, sums: B*nblk*2 doubles of
 * scratch. */
int tl_warm_loss(const tl_warm_crop *crops, int B, int H, int W, int margin, int objective, const float *g,
                 double *resid, double *sums, int nblk, double *crop_loss, void *dz, void *stream);

#ifdef __cplusplus
}
#endif
#endif
