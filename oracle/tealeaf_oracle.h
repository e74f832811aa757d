/*
 * tealeaf_oracle.h -- CPU restatement of TeaLeaf.jl's implicit heat-conduction
 * solve path.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and
 * the CPU-baseline leg of the benchmark link this library as the checker.  The
 * product (the CUDA library) never calls it.
 *
 * PARITY UNPINNED: the reference (Laura7089/TeaLeaf.jl) is Julia 1.7 code, no
 * Julia toolchain exists on either build machine, and the reference ships no
 * tests, golden vectors or tea.problems checking values (its .gitignore lists
 * tea.problems).  This file is therefore a line-by-line restatement of the
 * reference's Julia source; each function cites the file:line it follows.
 * The committed golden fixtures under tests/golden/ were produced by this
 * restatement plus hand-derived known answers, not by running the reference.
 *
 * Two semantics are provided (see tlo_opts.mode):
 *   TLO_MODE_REFERENCE  the reference exactly as written, quirks included:
 *                       the diagonal smvp (src/kernels.jl:180-181 returns
 *                       before the neighbour terms), the off-by-one halo index
 *                       math (src/kernels.jl:195-209), transposed state
 *                       geometry (src/chunk.jl:130-145), CG's absolute
 *                       sqrt(rr) < eps test (src/solvers/CG.jl:24).  Where the
 *                       reference raises (Cheby minmax, PPCG `++`, Jacobi
 *                       without solve!) the restatement returns
 *                       TLO_ERR_REFERENCE_THROWS at the same point.
 *   TLO_MODE_TEALEAF    the intended algorithm: the 5-point operator of the
 *                       dead code in src/kernels.jl:182-183, a reflective halo,
 *                       and the Cheby/PPCG/Jacobi fixes listed in
 *                       tealeaf_oracle.c beside each solver.
 *
 * Two summation orders are provided (see tlo_opts.order):
 *   TLO_ORDER_REFERENCE sequential loops where the reference accumulates with
 *                       `temp +=` (CG.jl:76,87), Julia Base's pairwise
 *                       mapreduce (1024-element sequential leaves) where the
 *                       reference calls sum().  Julia's @simd reassociation
 *                       inside a leaf is machine-dependent and is not
 *                       reproduced: leaves are summed in index order.
 *   TLO_ORDER_DEVICE    the fixed reduction tree of the CUDA kernels (tile
 *                       walk, warp butterfly, warp-ordered block sum, block
 *                       partials summed by the last block), parameterised by
 *                       the launch layout the CUDA library reports.  With it the
 *                       reference-mode GPU solve is bit-identical to this code.
 *
 * Arrays follow the reference's Chunk layout (src/chunk.jl:19-38): Float64,
 * column-major (X, Y), X = xcells + 2*halodepth, dimension 1 contiguous.
 * Indices here are 0-based: element (i, j) lives at i + j*X.
 */
#ifndef TEALEAF_ORACLE_H
#define TEALEAF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define TLO_MAX_STATES 64

/* Chunk fields, in the order of the reference's Chunk struct (src/chunk.jl:24-38),
 * plus the volume array (src/chunk.jl:46). */
enum {
  TLO_DENSITY0 = 0, TLO_DENSITY, TLO_ENERGY0, TLO_ENERGY, TLO_U, TLO_U0, TLO_P,
  TLO_R, TLO_MI, TLO_W, TLO_KX, TLO_KY, TLO_SD, TLO_VOLUME, TLO_NFIELDS
};
/* EXCHANGE_FIELDS order (src/chunk.jl:12). */
enum { TLO_EX_DENSITY = 0, TLO_EX_P, TLO_EX_ENERGY0, TLO_EX_ENERGY, TLO_EX_U, TLO_EX_SD, TLO_NEX };

enum { TLO_RECTANGULAR = 0, TLO_CIRCULAR = 1, TLO_POINT = 2 };           /* settings.jl:11 */
enum { TLO_CONDUCTIVITY = 1, TLO_RECIP_CONDUCTIVITY = 2 };               /* settings.jl:13-14 */
enum { TLO_CG = 0, TLO_CHEBY = 1, TLO_PPCG = 2, TLO_JACOBI = 3 };
enum { TLO_MODE_REFERENCE = 0, TLO_MODE_TEALEAF = 1 };
enum { TLO_ORDER_REFERENCE = 0, TLO_ORDER_DEVICE = 1 };

enum {
  TLO_OK = 0,
  TLO_ERR_ARG = 1,
  TLO_ERR_DECK = 2,            /* deck line the reference parser would reject  */
  TLO_ERR_COEF = 3,            /* CG.jl:48-50, Jacobi.jl:34-36                   */
  TLO_ERR_EIGEN = 4,           /* kernels.jl:41-43 negative eigenvalue           */
  TLO_ERR_REFERENCE_THROWS = 5,/* the reference raises at this point            */
  TLO_ERR_NOMEM = 6
};

typedef struct {                /* settings.jl:20-29 */
  double density, energy;
  double xmin, ymin, xmax, ymax;  /* as written in the deck, before the inset */
  double radius;
  int geometry;
  int given;                      /* bit 0 xmin, 1 ymin, 2 xmax, 3 ymax present */
  double pdx, pdy;                /* dx, dy while the line was read (settings.jl:159-162) */
} tlo_state;

typedef struct {                /* settings.jl:39-78 */
  long long endstep;
  int presteps, maxiters, coefficient, ppcginnersteps, summaryfrequency, halodepth;
  int errorswitch, checkresult;
  double eps, dtinit, endtime, epslim;
  int solver;
  int xcells, ycells;
  double xmin, ymin, xmax, ymax, dx, dy;
  int nstates;
  tlo_state states[TLO_MAX_STATES];
  int toexchange[TLO_NEX];
} tlo_settings;

typedef struct {
  int mode;         /* TLO_MODE_*  */
  int order;        /* TLO_ORDER_* */
  /* launch layout of the device reduction tree (TLO_ORDER_DEVICE only) */
  int dev_warps;    /* warps per block                         */
  int dev_rows;     /* rows of cells one warp walks per tile   */
  int dev_blocks;   /* persistent blocks in the grid           */
  int nthreads;     /* OpenMP threads for elementwise loops (1 = scalar) */
  int criterion;    /* CG only: 0 the reference's sqrt|rr| < eps (CG.jl:24); 1 the relative test
                       sqrt(|rr| / u0.u0) < eps on the recursive residual, then on the true residual
                       u0 - A u, restarting from it (at most 8 times) while it is above eps */
} tlo_opts;

typedef struct {
  double *f[TLO_NFIELDS];
  double *vertexx, *vertexy, *cellx, *celly;
  double theta, eigmin, eigmax;
  double *cgalpha, *cgbeta, *chebyalpha, *chebybeta;
  int x, y, hd, maxiters;
} tlo_chunk;

typedef struct {
  int iters;        /* loop trips of the solver's main loop            */
  int cg_iters;     /* CG iterations (presteps for Cheby/PPCG)         */
  int inner_iters;  /* Chebyshev or PPCG outer iterations after switch */
  int est_iters;    /* Cheby.calciter estimate                          */
  double error;     /* the error value the solver loop ended with      */
  double eigmin, eigmax;
  int status;       /* TLO_OK or an error code                          */
  int converged;    /* CG: the loop ended on its convergence test       */
  double rel_residual; /* CG with criterion 1: ||u0 - A u|| / ||u0|| at the end, else -1 */
} tlo_result;

typedef struct {
  double vol, mass, ie, temp;
} tlo_summary;

/* Deck */
void tlo_default_settings(tlo_settings *s);
int tlo_parse_deck(const char *text, tlo_settings *s, char *msg, int msglen);
/* The bounds setchunkstate! tests: reference mode insets by the dx/100 seen at
 * parse time (settings.jl:159-162, dx still the default 10 for any state line
 * before the end of the file); tealeaf mode insets by the deck's final dx/100. */
void tlo_effective_bounds(const tlo_settings *s, const tlo_state *st, int mode, double out[4]);

/* Chunk (src/chunk.jl:68-89) and initialiseapp! (src/TeaLeaf.jl:35-44) */
tlo_chunk *tlo_chunk_create(const tlo_settings *s, const tlo_opts *o, int *status);
void tlo_chunk_free(tlo_chunk *c);
double *tlo_field(tlo_chunk *c, int field);
int tlo_set_chunk_state(tlo_chunk *c, const tlo_settings *s, const tlo_opts *o);
int tlo_initialise_app(tlo_chunk *c, tlo_settings *s, const tlo_opts *o);

/* Kernels (src/kernels.jl) */
int tlo_halo_update(tlo_chunk *c, tlo_settings *s, const tlo_opts *o, int depth,
                    const int *fields, int nfields, int reset);
void tlo_copy_u(tlo_chunk *c, const tlo_opts *o);
void tlo_residual(tlo_chunk *c, const tlo_opts *o);
void tlo_finalise(tlo_chunk *c, const tlo_opts *o);
int tlo_solve_finished(tlo_chunk *c, tlo_settings *s, const tlo_opts *o);
void tlo_field_summary(tlo_chunk *c, const tlo_opts *o, tlo_summary *out);
int tlo_eigenvalues(tlo_chunk *c, int cgiters, const tlo_opts *o);

/* CG pieces (src/solvers/CG.jl), exposed for per-kernel parity tests */
int tlo_cg_init(tlo_chunk *c, int coefficient, double rx, double ry, const tlo_opts *o, double *rro);
double tlo_cg_calc_w(tlo_chunk *c, const tlo_opts *o);
double tlo_cg_calc_ur(tlo_chunk *c, double alpha, const tlo_opts *o);
void tlo_cg_calc_p(tlo_chunk *c, double beta, const tlo_opts *o);

/* Solver plugins: solve!(chunk, settings, rx, ry) */
int tlo_solve(tlo_chunk *c, tlo_settings *s, const tlo_opts *o, double rx, double ry, tlo_result *res);

/* diffuse! (src/TeaLeaf.jl:62-83): runs endstep timesteps; per step records the
 * solver result and, at each fieldsummary call, the summary. */
int tlo_diffuse(tlo_chunk *c, tlo_settings *s, const tlo_opts *o, tlo_result *steps, int maxsteps,
                tlo_summary *summaries, int maxsummaries, int *nsummaries);

/* Reductions, exposed for tests */
double tlo_pairwise_sum(const double *a, long long n);
double tlo_device_sum(const double *v, int nx, int ny, const tlo_opts *o);

/* Diagnostics: last error message */
const char *tlo_last_message(void);

#ifdef __cplusplus
}
#endif
#endif
