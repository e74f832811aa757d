/*
 * tealeaf_oracle.c -- CPU restatement of TeaLeaf.jl's solve path.
 * TEST INFRASTRUCTURE ONLY (the checker, never the product).  PARITY UNPINNED:
 * the Julia reference cannot run on these machines and ships no golden data;
 * see tealeaf_oracle.h for the two modes and the two summation orders.
 *
 * Build with -ffp-contract=off: the reference's Julia broadcasts never fuse
 * a*b+c into an FMA, and aarch64 gcc contracts by default.
 */
#include "tealeaf_oracle.h"

#include <ctype.h>
#include <errno.h>
#include <float.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define TLO_ORDER_THREADS 2 /* per-thread OpenMP partials: the timed CPU baseline */

static const double ERROR_START = 1e10;      /* kernels.jl:7   */
static const double ERROR_SWITCH_MAX = 1.0;  /* kernels.jl:8   */
static const int CGEIGENITERS = 20;          /* Cheby.jl:7     */

static char g_msg[512];
const char *tlo_last_message(void) { return g_msg; }
static void set_msg(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_msg, sizeof g_msg, fmt, ap);
  va_end(ap);
}

#define IDX(i, j) ((size_t)(i) + (size_t)(j) * (size_t)X)
#define NT(o) ((o)->nthreads > 1 ? (o)->nthreads : 1)

/* ------------------------------------------------------------------------- */
/* Reductions                                                                 */
/* ------------------------------------------------------------------------- */

/* Julia Base mapreduce_impl: pairwise split down to 1024-element leaves that
 * are summed in index order (the @simd reassociation is not reproduced). */
static double mr_impl(const double *a, long long lo, long long hi) {
  if (lo == hi) return a[lo];
  if (hi - lo < 1024) {
    double v = a[lo] + a[lo + 1];
    for (long long i = lo + 2; i <= hi; ++i) v += a[i];
    return v;
  }
  long long mid = lo + ((hi - lo) >> 1);
  double v1 = mr_impl(a, lo, mid);
  double v2 = mr_impl(a, mid + 1, hi);
  return v1 + v2;
}

/* Julia Base _mapreduce(f, +, IndexLinear(), A) for a dense array. */
double tlo_pairwise_sum(const double *a, long long n) {
  if (n <= 0) return 0.0;
  if (n == 1) return a[0];
  if (n < 16) {
    double s = a[0] + a[1];
    for (long long i = 2; i < n; ++i) s += a[i];
    return s;
  }
  return mr_impl(a, 0, n - 1);
}

static void warp_butterfly(double *lane) {
  double tmp[32];
  for (int off = 16; off >= 1; off >>= 1) {
    for (int l = 0; l < 32; ++l) tmp[l] = lane[l] + lane[l ^ off];
    memcpy(lane, tmp, sizeof tmp);
  }
}

/* The CUDA kernels' reduction tree.  Interior cells are walked in tiles of
 * (64*warps) columns x rows; tile t -> (t % ntx, t / ntx); block b walks tiles
 * b, b+G, ...; lane l of warp w owns the column pair i0 = 64*w + 2*l of each
 * tile and adds its two cells row by row; lanes are combined by an xor
 * butterfly (16,8,4,2,1), warps in warp order; the last block to finish adds
 * the G block partials with the same lane/butterfly/warp scheme. */
double tlo_device_sum(const double *v, int nx, int ny, const tlo_opts *o) {
  const int NW = o->dev_warps, TY = o->dev_rows, G = o->dev_blocks;
  const int TW = 64 * NW, F = 32 * NW;
  if (NW <= 0 || TY <= 0 || G <= 0 || NW > 32) return NAN;
  const long long ntx = (nx + TW - 1) / TW, nty = (ny + TY - 1) / TY, T = ntx * nty;
  double *partial = (double *)calloc((size_t)G, sizeof(double));
  double *acc = (double *)malloc(sizeof(double) * (size_t)F);
  if (!partial || !acc) { free(partial); free(acc); return NAN; }
  /* Blocks are independent until the last block's pass, so they may be
   * computed by several host threads without changing any partial. */
#pragma omp parallel for num_threads(NT(o)) schedule(dynamic, 1)
  for (int b = 0; b < G; ++b) {
    double bacc[32 * 32];
    for (int t = 0; t < F; ++t) bacc[t] = 0.0;
    for (long long t = b; t < T; t += G) {
      const long long tx = t % ntx, ty = t / ntx;
      const int j0 = (int)(ty * TY), j1 = (int)((ty * TY + TY) < ny ? ty * TY + TY : ny);
      for (int w = 0; w < NW; ++w)
        for (int l = 0; l < 32; ++l) {
          const long long i0 = tx * TW + 64 * w + 2 * l;
          double a = bacc[w * 32 + l];
          for (int j = j0; j < j1; ++j) {
            if (i0 < nx) a += v[i0 + (size_t)j * nx];
            if (i0 + 1 < nx) a += v[i0 + 1 + (size_t)j * nx];
          }
          bacc[w * 32 + l] = a;
        }
    }
    double blk = 0.0;
    for (int w = 0; w < NW; ++w) {
      warp_butterfly(bacc + 32 * w);
      blk = (w == 0) ? bacc[0] : blk + bacc[32 * w];
    }
    partial[b] = blk;
  }
  for (int t = 0; t < F; ++t) {
    double a = 0.0;
    for (int k = t; k < G; k += F) a += partial[k];
    acc[t] = a;
  }
  double total = 0.0;
  for (int w = 0; w < NW; ++w) {
    warp_butterfly(acc + 32 * w);
    total = (w == 0) ? acc[0] : total + acc[32 * w];
  }
  free(partial);
  free(acc);
  return total;
}

/* scratch arrays owned by the chunk */
typedef struct {
  double *interior; /* nx*ny */
  double *full;     /* X*Y   */
} tlo_scratch;
static tlo_scratch g_scr = {0, 0};
static size_t g_scr_n = 0, g_scr_full = 0;

static int ensure_scratch(const tlo_chunk *c) {
  size_t nx = (size_t)(c->x - 2 * c->hd), ny = (size_t)(c->y - 2 * c->hd);
  size_t n = nx * ny, nf = (size_t)c->x * (size_t)c->y;
  if (n > g_scr_n) {
    free(g_scr.interior);
    g_scr.interior = (double *)malloc(n * sizeof(double));
    g_scr_n = g_scr.interior ? n : 0;
  }
  if (nf > g_scr_full) {
    free(g_scr.full);
    g_scr.full = (double *)malloc(nf * sizeof(double));
    g_scr_full = g_scr.full ? nf : 0;
  }
  return g_scr.interior && g_scr.full;
}

/* How the reference accumulates at a given site. */
enum { SEQ = 0, PAIRWISE = 1 };

/* Reduce per-cell values stored in the interior scratch. */
static double reduce_interior(const tlo_chunk *c, const tlo_opts *o, int kind) {
  const int nx = c->x - 2 * c->hd, ny = c->y - 2 * c->hd;
  const long long n = (long long)nx * ny;
  if (o->order == TLO_ORDER_DEVICE) return tlo_device_sum(g_scr.interior, nx, ny, o);
  if (kind == PAIRWISE) return tlo_pairwise_sum(g_scr.interior, n);
  double t = 0.0;
  for (long long k = 0; k < n; ++k) t += g_scr.interior[k];
  return t;
}

/* ------------------------------------------------------------------------- */
/* Settings and deck parsing (src/settings.jl)                                */
/* ------------------------------------------------------------------------- */

void tlo_default_settings(tlo_settings *s) {   /* settings.jl:39-78 */
  memset(s, 0, sizeof *s);
  s->endstep = 9223372036854775807LL;          /* typemax(Int) */
  s->presteps = 30;
  s->maxiters = 10000;
  s->coefficient = TLO_CONDUCTIVITY;
  s->ppcginnersteps = 10;
  s->summaryfrequency = 10;
  s->halodepth = 2;
  s->errorswitch = 0;
  s->checkresult = 1;
  s->eps = 1e-15;
  s->dtinit = 0.1;
  s->endtime = 10.0;
  s->epslim = 1e-5;
  s->solver = TLO_CG;
  s->xcells = 10;
  s->ycells = 10;
  s->xmin = 0.0;
  s->ymin = 0.0;
  s->xmax = 100.0;
  s->ymax = 100.0;
  s->dx = (s->xmax - s->xmin) / s->xcells;
  s->dy = (s->ymax - s->ymin) / s->ycells;
}

static void strip_inplace(char *s) {
  size_t n = strlen(s), a = 0;
  while (n > 0 && isspace((unsigned char)s[n - 1])) s[--n] = 0;
  while (s[a] && isspace((unsigned char)s[a])) ++a;
  if (a) memmove(s, s + a, n - a + 1);
}

/* parse(Int, s): optional surrounding whitespace and sign, decimal digits. */
static int parse_int(const char *v, long long *out) {
  char buf[128];
  if (strlen(v) >= sizeof buf) return 0;
  strcpy(buf, v);
  strip_inplace(buf);
  const char *p = buf;
  int neg = 0;
  if (*p == '+' || *p == '-') neg = (*p++ == '-');
  if (!*p) return 0;
  long long x = 0;
  for (; *p; ++p) {
    if (!isdigit((unsigned char)*p)) return 0;
    if (x > (9223372036854775807LL - (*p - '0')) / 10) return 0;
    x = x * 10 + (*p - '0');
  }
  *out = neg ? -x : x;
  return 1;
}

/* parse(Float64, s): strtod over the whole stripped string. */
static int parse_f64(const char *v, double *out) {
  char buf[128];
  if (strlen(v) >= sizeof buf) return 0;
  strcpy(buf, v);
  strip_inplace(buf);
  if (!buf[0]) return 0;
  char *end = NULL;
  errno = 0;
  double x = strtod(buf, &end);
  if (end == buf || *end) return 0;
  *out = x;
  return 1;
}

/* parse(Bool, s) */
static int parse_bool(const char *v, int *out) {
  char buf[32];
  if (strlen(v) >= sizeof buf) return 0;
  strcpy(buf, v);
  strip_inplace(buf);
  if (!strcmp(buf, "true") || !strcmp(buf, "1")) { *out = 1; return 1; }
  if (!strcmp(buf, "false") || !strcmp(buf, "0")) { *out = 0; return 1; }
  return 0;
}

/* readstate (settings.jl:142-173).  Bounds get the inset dx/100 (dy/100) with
 * dx, dy as they stand while the line is read (settings.jl:159-162). */
static int read_state(char *line, tlo_settings *s) {
  if (s->nstates >= TLO_MAX_STATES) { set_msg("too many states"); return TLO_ERR_DECK; }
  /* split(line, " ") : single spaces, empty pieces kept */
  char *pieces[256];
  int np = 0;
  char *p = line;
  pieces[np++] = p;
  for (; *p; ++p)
    if (*p == ' ') {
      *p = 0;
      if (np >= 256) { set_msg("state line too long"); return TLO_ERR_DECK; }
      pieces[np++] = p + 1;
    }
  if (np < 2) { set_msg("state line without a number"); return TLO_ERR_DECK; }
  long long num;
  if (!parse_int(pieces[1], &num)) { set_msg("bad state number '%s'", pieces[1]); return TLO_ERR_DECK; }
  tlo_state st;
  memset(&st, 0, sizeof st);
  st.geometry = TLO_RECTANGULAR;
  st.pdx = s->dx;
  st.pdy = s->dy;
  for (int k = 2; k < np; ++k) {
    char *eq = strchr(pieces[k], '=');
    if (!eq) { set_msg("state item '%s' has no '='", pieces[k]); return TLO_ERR_DECK; }
    *eq = 0;
    const char *key = pieces[k];
    char *val = eq + 1;
    char *eq2 = strchr(val, '=');
    if (eq2) *eq2 = 0; /* split keeps only the first two pieces */
    double d;
    if (!strcmp(key, "density")) {
      if (!parse_f64(val, &d)) { set_msg("bad density '%s'", val); return TLO_ERR_DECK; }
      st.density = d;
    } else if (!strcmp(key, "energy")) {
      if (!parse_f64(val, &d)) { set_msg("bad energy '%s'", val); return TLO_ERR_DECK; }
      st.energy = d;
    }
    if (num == 1) continue;
    if (!strcmp(key, "xmin") || !strcmp(key, "ymin") || !strcmp(key, "xmax") || !strcmp(key, "ymax") ||
        !strcmp(key, "radius")) {
      if (!parse_f64(val, &d)) { set_msg("bad %s '%s'", key, val); return TLO_ERR_DECK; }
      if (!strcmp(key, "xmin")) { st.xmin = d; st.given |= 1; }
      else if (!strcmp(key, "ymin")) { st.ymin = d; st.given |= 2; }
      else if (!strcmp(key, "xmax")) { st.xmax = d; st.given |= 4; }
      else if (!strcmp(key, "ymax")) { st.ymax = d; st.given |= 8; }
      else st.radius = d;
    } else if (!strcmp(key, "geometry")) {
      if (!strcmp(val, "rectangle")) st.geometry = TLO_RECTANGULAR;
      else if (!strcmp(val, "circular")) st.geometry = TLO_CIRCULAR;
      else if (!strcmp(val, "point")) st.geometry = TLO_POINT;
      else { set_msg("unknown geometry '%s'", val); return TLO_ERR_DECK; }
    }
  }
  s->states[s->nstates++] = st;
  return TLO_OK;
}

/* Settings(infile) (settings.jl:90-135).  Unknown keys and unparsable values
 * are skipped, as the reference only warns about them. */
int tlo_parse_deck(const char *text, tlo_settings *s, char *msg, int msglen) {
  tlo_default_settings(s);
  const char *p = text;
  char line[4096];
  int rc = TLO_OK;
  while (*p) {
    const char *e = strchr(p, '\n');
    size_t n = e ? (size_t)(e - p) : strlen(p);
    if (n >= sizeof line) n = sizeof line - 1;
    memcpy(line, p, n);
    line[n] = 0;
    p = e ? e + 1 : p + strlen(p);
    strip_inplace(line);
    if (!strncmp(line, "state", 5)) {
      rc = read_state(line, s);
      if (rc) break;
      continue;
    }
    if (!strncmp(line, "use_", 4)) {
      const char *v = line + 4;
      if (!strcmp(v, "cg")) s->solver = TLO_CG;
      else if (!strcmp(v, "ppcg")) s->solver = TLO_PPCG;
      else if (!strcmp(v, "cheby")) s->solver = TLO_CHEBY;
      else if (!strcmp(v, "jacobi")) s->solver = TLO_JACOBI;
      continue;
    }
    if (line[0] == '*' || !strchr(line, '=')) continue;
    char *eq = strchr(line, '=');
    *eq = 0;
    char *val = eq + 1;
    char *eq2 = strchr(val, '=');
    if (eq2) *eq2 = 0;
    char key[256];
    size_t kn = 0;
    for (const char *k = line; *k && kn + 1 < sizeof key; ++k)
      if (*k != '_') key[kn++] = *k;
    key[kn] = 0;
    strip_inplace(key);
    if (!strcmp(key, "initialtimestep")) strcpy(key, "dtinit");
    long long iv;
    double dv;
    int bv;
#define INTKEY(name, field)                                        \
  if (!strcmp(key, name)) {                                        \
    if (parse_int(val, &iv)) s->field = iv;                        \
    continue;                                                      \
  }
#define F64KEY(name, field)                                        \
  if (!strcmp(key, name)) {                                        \
    if (parse_f64(val, &dv)) s->field = dv;                        \
    continue;                                                      \
  }
#define BOOLKEY(name, field)                                       \
  if (!strcmp(key, name)) {                                        \
    if (parse_bool(val, &bv)) s->field = bv;                       \
    continue;                                                      \
  }
    INTKEY("endstep", endstep)
    INTKEY("presteps", presteps)
    INTKEY("maxiters", maxiters)
    INTKEY("coefficient", coefficient)
    INTKEY("ppcginnersteps", ppcginnersteps)
    INTKEY("summaryfrequency", summaryfrequency)
    INTKEY("halodepth", halodepth)
    INTKEY("xcells", xcells)
    INTKEY("ycells", ycells)
    BOOLKEY("errorswitch", errorswitch)
    BOOLKEY("checkresult", checkresult)
    F64KEY("eps", eps)
    F64KEY("dtinit", dtinit)
    F64KEY("endtime", endtime)
    F64KEY("epslim", epslim)
    F64KEY("xmin", xmin)
    F64KEY("ymin", ymin)
    F64KEY("xmax", xmax)
    F64KEY("ymax", ymax)
    F64KEY("dx", dx)
    F64KEY("dy", dy)
#undef INTKEY
#undef F64KEY
#undef BOOLKEY
  }
  if (rc) {
    if (msg && msglen > 0) snprintf(msg, (size_t)msglen, "%s", g_msg);
    return rc;
  }
  s->dx = (s->xmax - s->xmin) / s->xcells;   /* settings.jl:132-133 */
  s->dy = (s->ymax - s->ymin) / s->ycells;
  return TLO_OK;
}

void tlo_effective_bounds(const tlo_settings *s, const tlo_state *st, int mode, double out[4]) {
  const double ix = mode == TLO_MODE_REFERENCE ? st->pdx : s->dx;
  const double iy = mode == TLO_MODE_REFERENCE ? st->pdy : s->dy;
  out[0] = (st->given & 1) ? st->xmin + ix / 100 : st->xmin;
  out[1] = (st->given & 2) ? st->ymin + iy / 100 : st->ymin;
  out[2] = (st->given & 4) ? st->xmax - ix / 100 : st->xmax;
  out[3] = (st->given & 8) ? st->ymax - iy / 100 : st->ymax;
}

/* ------------------------------------------------------------------------- */
/* Chunk (src/chunk.jl)                                                        */
/* ------------------------------------------------------------------------- */

tlo_chunk *tlo_chunk_create(const tlo_settings *s, const tlo_opts *o, int *status) {
  *status = TLO_OK;
  const int hd = s->halodepth;
  if (s->xcells < 1 || s->ycells < 1 || hd < 1 || s->maxiters < 1) { *status = TLO_ERR_ARG; set_msg("bad sizes"); return NULL; }
  const int X = s->xcells + 2 * hd, Y = s->ycells + 2 * hd;
  if (o->mode == TLO_MODE_REFERENCE && X != Y) {
    /* chunk.jl:44 broadcasts vertexy (Y+1) against vertexx (X+1) */
    *status = TLO_ERR_REFERENCE_THROWS;
    set_msg("DimensionMismatch: celly broadcasts vertexy against vertexx (src/chunk.jl:44) on a non-square deck");
    return NULL;
  }
  tlo_chunk *c = (tlo_chunk *)calloc(1, sizeof *c);
  if (!c) { *status = TLO_ERR_NOMEM; return NULL; }
  c->x = X; c->y = Y; c->hd = hd; c->maxiters = s->maxiters;
  size_t n = (size_t)X * Y;
  for (int f = 0; f < TLO_NFIELDS; ++f) {
    c->f[f] = (double *)calloc(n, sizeof(double));
    if (!c->f[f]) { *status = TLO_ERR_NOMEM; tlo_chunk_free(c); return NULL; }
  }
  c->vertexx = (double *)malloc(sizeof(double) * (X + 1));
  c->vertexy = (double *)malloc(sizeof(double) * (Y + 1));
  c->cellx = (double *)malloc(sizeof(double) * X);
  c->celly = (double *)malloc(sizeof(double) * Y);
  size_t m = (size_t)s->maxiters + 2;
  c->cgalpha = (double *)calloc(m, sizeof(double));
  c->cgbeta = (double *)calloc(m, sizeof(double));
  c->chebyalpha = (double *)calloc(m, sizeof(double));
  c->chebybeta = (double *)calloc(m, sizeof(double));
  if (!c->vertexx || !c->vertexy || !c->cellx || !c->celly || !c->cgalpha || !c->cgbeta || !c->chebyalpha || !c->chebybeta) {
    *status = TLO_ERR_NOMEM; tlo_chunk_free(c); return NULL;
  }
  /* chunk.jl:76-77: vertex k (1-based) = xmin + dx*(k - hd - 1) */
  for (int k = 0; k <= X; ++k) c->vertexx[k] = s->xmin + s->dx * (double)(k - hd);
  for (int k = 0; k <= Y; ++k) c->vertexy[k] = s->ymin + s->dy * (double)(k - hd);
  /* chunk.jl:43-44 (celly adds vertexx in the reference) */
  for (int k = 0; k < X; ++k) c->cellx[k] = 0.5 * (c->vertexx[k] + c->vertexx[k + 1]);
  for (int k = 0; k < Y; ++k)
    c->celly[k] = 0.5 * (c->vertexy[k] + (o->mode == TLO_MODE_REFERENCE ? c->vertexx[k + 1] : c->vertexy[k + 1]));
  const double vol = s->dx * s->dy;  /* chunk.jl:79 */
  for (size_t k = 0; k < n; ++k) c->f[TLO_VOLUME][k] = vol;
  c->theta = c->eigmin = c->eigmax = 0.0;
  if (!ensure_scratch(c)) { *status = TLO_ERR_NOMEM; tlo_chunk_free(c); return NULL; }
  return c;
}

void tlo_chunk_free(tlo_chunk *c) {
  if (!c) return;
  for (int f = 0; f < TLO_NFIELDS; ++f) free(c->f[f]);
  free(c->vertexx); free(c->vertexy); free(c->cellx); free(c->celly);
  free(c->cgalpha); free(c->cgbeta); free(c->chebyalpha); free(c->chebybeta);
  free(c);
}

double *tlo_field(tlo_chunk *c, int field) {
  if (!c || field < 0 || field >= TLO_NFIELDS) return NULL;
  return c->f[field];
}

/* setchunkstate! (chunk.jl:122-151).  Reference mode writes [j, k] with j the
 * y-vertex index on dimension 1 (chunk.jl:143-144) and applies the rectangle
 * test to every state: Match.jl 1.x treats the bare symbol `Rectangular` in
 * chunk.jl:132 as a binding pattern, so the first arm matches any geometry.
 * Tealeaf mode writes [k, j] and honours circular and point states. */
int tlo_set_chunk_state(tlo_chunk *c, const tlo_settings *s, const tlo_opts *o) {
  const int X = c->x, Y = c->y;
  const size_t n = (size_t)X * Y;
  if (s->nstates < 1) { set_msg("no states"); return TLO_ERR_ARG; }
  double *e0 = c->f[TLO_ENERGY0], *rho = c->f[TLO_DENSITY];
  for (size_t k = 0; k < n; ++k) { e0[k] = s->states[0].energy; rho[k] = s->states[0].density; }
  const int ref = (o->mode == TLO_MODE_REFERENCE);
  for (int si = 0; si < s->nstates; ++si) {
    const tlo_state *st = &s->states[si];
    double b[4];
    tlo_effective_bounds(s, st, o->mode, b);
    const double sxmin = b[0], symin = b[1], sxmax = b[2], symax = b[3];
    for (int j = 0; j < Y; ++j)
      for (int k = 0; k < X; ++k) {
        int apply;
        int geom = ref ? TLO_RECTANGULAR : st->geometry;
        if (geom == TLO_RECTANGULAR)
          apply = c->vertexx[k + 1] >= sxmin && c->vertexx[k] < sxmax &&
                  c->vertexy[j + 1] >= symin && c->vertexy[j] < symax;
        else if (geom == TLO_CIRCULAR) {
          double ddx = c->cellx[k] - sxmin, ddy = c->celly[j] - symin;
          apply = ddx * ddx + ddy * ddy <= st->radius * st->radius;
        } else
          apply = c->vertexx[k] == sxmin && c->vertexy[j] == symin;
        if (!apply) continue;
        size_t id = ref ? (size_t)j + (size_t)k * X : (size_t)k + (size_t)j * X;
        e0[id] = st->energy;
        rho[id] = st->density;
      }
  }
  /* u[halo(ch,1)] = energy0 * density (chunk.jl:148-150) */
  double *u = c->f[TLO_U];
  for (int j = 1; j < Y - 1; ++j)
    for (int i = 1; i < X - 1; ++i) u[IDX(i, j)] = e0[IDX(i, j)] * rho[IDX(i, j)];
  return TLO_OK;
}

/* ------------------------------------------------------------------------- */
/* Halo (kernels.jl:146-159, 191-210)                                          */
/* ------------------------------------------------------------------------- */

static const int EX_TO_FIELD[TLO_NEX] = {TLO_DENSITY, TLO_P, TLO_ENERGY0, TLO_ENERGY, TLO_U, TLO_SD};

/* updateface!.  Reference mode keeps the 1-based index math of the Julia
 * transcription (left: b[hd-kk] <- b[hd+kk], right: b[X-hd+kk] <- b[X-hd-1-kk],
 * kk = 1:depth), which is one cell off from a reflection.  Tealeaf mode
 * reflects: 0-based b[hd-1-kk] <- b[hd+kk], b[X-hd+kk] <- b[X-hd-1-kk].
 * Faces cover the interior range of the other axis; corners are untouched. */
static int update_face(tlo_chunk *c, int depth, double *b, int mode) {
  const int X = c->x, Y = c->y, hd = c->hd;
  if (mode == TLO_MODE_REFERENCE) {
    if (hd - depth - 1 < 0) {
      set_msg("BoundsError: halo index %d (1-based) in updateface! (src/kernels.jl:196)", hd - depth);
      return TLO_ERR_REFERENCE_THROWS;
    }
    for (int kk = 1; kk <= depth; ++kk)
      for (int j = hd; j < Y - hd; ++j) b[IDX(hd - kk - 1, j)] = b[IDX(hd + kk - 1, j)];
    for (int kk = 1; kk <= depth; ++kk)
      for (int j = hd; j < Y - hd; ++j) b[IDX(X - hd + kk - 1, j)] = b[IDX(X - hd - 2 - kk, j)];
    for (int jj = 1; jj <= depth; ++jj)
      for (int i = hd; i < X - hd; ++i) b[IDX(i, Y - hd + jj - 1)] = b[IDX(i, Y - hd - 2 - jj)];
    for (int jj = 1; jj <= depth; ++jj)
      for (int i = hd; i < X - hd; ++i) b[IDX(i, hd - jj - 1)] = b[IDX(i, hd + jj - 1)];
  } else {
    if (depth > hd) { set_msg("halo depth %d exceeds halo_depth %d", depth, hd); return TLO_ERR_ARG; }
    for (int kk = 0; kk < depth; ++kk)
      for (int j = hd; j < Y - hd; ++j) b[IDX(hd - 1 - kk, j)] = b[IDX(hd + kk, j)];
    for (int kk = 0; kk < depth; ++kk)
      for (int j = hd; j < Y - hd; ++j) b[IDX(X - hd + kk, j)] = b[IDX(X - hd - 1 - kk, j)];
    for (int jj = 0; jj < depth; ++jj)
      for (int i = hd; i < X - hd; ++i) b[IDX(i, Y - hd + jj)] = b[IDX(i, Y - hd - 1 - jj)];
    for (int jj = 0; jj < depth; ++jj)
      for (int i = hd; i < X - hd; ++i) b[IDX(i, hd - 1 - jj)] = b[IDX(i, hd + jj)];
  }
  return TLO_OK;
}

static void reset_to_exchange(tlo_settings *s) {  /* settings.jl:80 */
  for (int k = 0; k < TLO_NEX; ++k) s->toexchange[k] = 0;
}

/* haloupdate!(chunk, set, depth[, toex][, reset]); fields are EXCHANGE_FIELDS
 * indices; nfields < 0 means "use set.toexchange". */
int tlo_halo_update(tlo_chunk *c, tlo_settings *s, const tlo_opts *o, int depth, const int *fields, int nfields,
                    int reset) {
  int list[TLO_NEX], nl = 0;
  if (nfields >= 0) {
    if (reset) reset_to_exchange(s);
    for (int k = 0; k < nfields; ++k) {
      if (fields[k] < 0 || fields[k] >= TLO_NEX) return TLO_ERR_ARG;
      s->toexchange[fields[k]] = 1;
      list[nl++] = fields[k];
    }
  } else {
    for (int k = 0; k < TLO_NEX; ++k)
      if (s->toexchange[k]) list[nl++] = k;
  }
  for (int k = 0; k < nl; ++k) {
    int rc = update_face(c, depth, c->f[EX_TO_FIELD[list[k]]], o->mode);
    if (rc) return rc;
  }
  return TLO_OK;
}

/* ------------------------------------------------------------------------- */
/* Stencil (kernels.jl:178-184)                                                */
/* ------------------------------------------------------------------------- */

static inline double smvp(const tlo_chunk *c, const double *a, int i, int j, int mode) {
  const int X = c->x;
  const double *kx = c->f[TLO_KX], *ky = c->f[TLO_KY];
  const double kxr = kx[IDX(i + 1, j)], kxc = kx[IDX(i, j)], kyt = ky[IDX(i, j + 1)], kyc = ky[IDX(i, j)];
  double consum = 1.0 + kxr;   /* sum((1, kx[x+1,y], kx[x,y], ky[x,y+1], ky[x,y])): left fold */
  consum = consum + kxc;
  consum = consum + kyt;
  consum = consum + kyc;
  double v = consum * a[IDX(i, j)];
  if (mode == TLO_MODE_REFERENCE) return v;   /* kernels.jl:181 returns here */
  v = v - (kxr * a[IDX(i + 1, j)] + kxc * a[IDX(i - 1, j)]);
  v = v - (kyt * a[IDX(i, j + 1)] + kyc * a[IDX(i, j - 1)]);
  return v;
}

/* ------------------------------------------------------------------------- */
/* Elementwise kernels (kernels.jl:217-242)                                    */
/* ------------------------------------------------------------------------- */

void tlo_copy_u(tlo_chunk *c, const tlo_opts *o) {  /* kernels.jl:217-220 */
  const int X = c->x, Y = c->y, hd = c->hd;
  double *u0 = c->f[TLO_U0], *u = c->f[TLO_U];
#pragma omp parallel for num_threads(NT(o)) schedule(static)
  for (int j = hd; j < Y - hd; ++j)
    for (int i = hd; i < X - hd; ++i) u0[IDX(i, j)] = u[IDX(i, j)];
}

void tlo_residual(tlo_chunk *c, const tlo_opts *o) {  /* kernels.jl:227-232 */
  const int X = c->x, Y = c->y, hd = c->hd;
  double *r = c->f[TLO_R], *u0 = c->f[TLO_U0], *u = c->f[TLO_U];
#pragma omp parallel for num_threads(NT(o)) schedule(static)
  for (int j = hd; j < Y - hd; ++j)
    for (int i = hd; i < X - hd; ++i) r[IDX(i, j)] = u0[IDX(i, j)] - smvp(c, u, i, j, o->mode);
}

void tlo_finalise(tlo_chunk *c, const tlo_opts *o) {  /* kernels.jl:239-242 */
  const int X = c->x, Y = c->y, hd = c->hd;
  double *e = c->f[TLO_ENERGY], *u = c->f[TLO_U], *rho = c->f[TLO_DENSITY];
#pragma omp parallel for num_threads(NT(o)) schedule(static)
  for (int j = hd; j < Y - hd; ++j)
    for (int i = hd; i < X - hd; ++i) e[IDX(i, j)] = u[IDX(i, j)] / rho[IDX(i, j)];
}

int tlo_solve_finished(tlo_chunk *c, tlo_settings *s, const tlo_opts *o) {  /* kernels.jl:166-170 */
  if (s->checkresult) tlo_residual(c, o);
  tlo_finalise(c, o);
  int f = TLO_EX_ENERGY;
  return tlo_halo_update(c, s, o, 1, &f, 1, 0);
}

/* fieldsummary (kernels.jl:119-133) computes temp = sum(vol .* rho .* u) over
 * the interior; vol, mass and ie are the added field_summary quantities
 * (sum vol, sum vol*rho, sum vol*rho*energy), summed the same way. */
void tlo_field_summary(tlo_chunk *c, const tlo_opts *o, tlo_summary *out) {
  const int X = c->x, Y = c->y, hd = c->hd, nx = X - 2 * hd;
  const double *vol = c->f[TLO_VOLUME], *rho = c->f[TLO_DENSITY], *u = c->f[TLO_U], *e = c->f[TLO_ENERGY];
  double *sc = g_scr.interior;
  double res[4];
  for (int q = 0; q < 4; ++q) {
    if (o->order == TLO_ORDER_THREADS) {
      double acc = 0.0;
#pragma omp parallel for num_threads(NT(o)) schedule(static) reduction(+ : acc)
      for (int j = hd; j < Y - hd; ++j)
        for (int i = hd; i < X - hd; ++i) {
          size_t id = IDX(i, j);
          double v = q == 0 ? vol[id] : q == 1 ? vol[id] * rho[id] : q == 2 ? vol[id] * rho[id] * e[id] : vol[id] * rho[id] * u[id];
          acc += v;
        }
      res[q] = acc;
      continue;
    }
#pragma omp parallel for num_threads(NT(o)) schedule(static)
    for (int j = hd; j < Y - hd; ++j)
      for (int i = hd; i < X - hd; ++i) {
        size_t id = IDX(i, j);
        double v = q == 0 ? vol[id] : q == 1 ? vol[id] * rho[id] : q == 2 ? vol[id] * rho[id] * e[id] : vol[id] * rho[id] * u[id];
        sc[(size_t)(i - hd) + (size_t)(j - hd) * nx] = v;
      }
    res[q] = reduce_interior(c, o, PAIRWISE);
  }
  out->vol = res[0]; out->mass = res[1]; out->ie = res[2]; out->temp = res[3];
}

/* ------------------------------------------------------------------------- */
/* CG (src/solvers/CG.jl)                                                      */
/* ------------------------------------------------------------------------- */

/* init! = tea_leaf_init (CG.jl:47-79) */
int tlo_cg_init(tlo_chunk *c, int coefficient, double rx, double ry, const tlo_opts *o, double *rro) {
  if (coefficient != TLO_CONDUCTIVITY && coefficient != TLO_RECIP_CONDUCTIVITY) {
    set_msg("Coefficient %d is not valid (src/solvers/CG.jl:49)", coefficient);
    return TLO_ERR_COEF;
  }
  const int X = c->x, Y = c->y, hd = c->hd, nx = X - 2 * hd;
  const size_t n = (size_t)X * Y;
  double *u = c->f[TLO_U], *e = c->f[TLO_ENERGY], *rho = c->f[TLO_DENSITY], *p = c->f[TLO_P], *r = c->f[TLO_R],
         *w = c->f[TLO_W], *kx = c->f[TLO_KX], *ky = c->f[TLO_KY];
#pragma omp parallel for num_threads(NT(o)) schedule(static)
  for (size_t k = 0; k < n; ++k) { u[k] = e[k] * rho[k]; p[k] = 0.0; r[k] = 0.0; }
  /* CG.jl:57-60 computes w on 2:X-1 x 2:Y-1 only; with halo depth 1 the
   * outer halo layer then keeps w = 0 and Kx, Ky at the domain edge are
   * infinite.  Tealeaf mode computes w over the whole array (the density
   * halo is exchanged), which changes nothing for halo depth >= 2. */
  const int w0 = o->mode == TLO_MODE_TEALEAF ? 0 : 1;
#pragma omp parallel for num_threads(NT(o)) schedule(static)
  for (int j = w0; j < Y - w0; ++j)
    for (int i = w0; i < X - w0; ++i)
      w[IDX(i, j)] = coefficient == TLO_CONDUCTIVITY ? rho[IDX(i, j)] : 1.0 / rho[IDX(i, j)];
#pragma omp parallel for num_threads(NT(o)) schedule(static)
  for (int j = hd; j < Y - 1; ++j)
    for (int i = hd; i < X - 1; ++i) {
      const double wl = w[IDX(i - 1, j)], wc = w[IDX(i, j)], wd = w[IDX(i, j - 1)];
      kx[IDX(i, j)] = rx * (wl + wc) / (2 * wl * wc);
      ky[IDX(i, j)] = ry * (wd + wc) / (2 * wd * wc);
    }
  double acc = 0.0;
  const int store = o->order != TLO_ORDER_THREADS;
#pragma omp parallel for num_threads(NT(o)) schedule(static) reduction(+ : acc)
  for (int j = hd; j < Y - hd; ++j)
    for (int i = hd; i < X - hd; ++i) {
      const size_t id = IDX(i, j);
      const double wv = smvp(c, u, i, j, o->mode);
      w[id] = wv;
      r[id] = u[id] - wv;
      p[id] = r[id];
      const double v = r[id] * r[id];
      if (store) g_scr.interior[(size_t)(i - hd) + (size_t)(j - hd) * nx] = v; else acc += v;
    }
  *rro = store ? reduce_interior(c, o, SEQ) : acc;
  return TLO_OK;
}

/* w! (CG.jl:82-90): w = A p, returns p.w */
double tlo_cg_calc_w(tlo_chunk *c, const tlo_opts *o) {
  const int X = c->x, Y = c->y, hd = c->hd, nx = X - 2 * hd;
  double *w = c->f[TLO_W], *p = c->f[TLO_P];
  double acc = 0.0;
  const int store = o->order != TLO_ORDER_THREADS;
#pragma omp parallel for num_threads(NT(o)) schedule(static) reduction(+ : acc)
  for (int j = hd; j < Y - hd; ++j)
    for (int i = hd; i < X - hd; ++i) {
      const size_t id = IDX(i, j);
      const double wv = smvp(c, p, i, j, o->mode);
      w[id] = wv;
      const double v = wv * p[id];
      if (store) g_scr.interior[(size_t)(i - hd) + (size_t)(j - hd) * nx] = v; else acc += v;
    }
  return store ? reduce_interior(c, o, SEQ) : acc;
}

/* ur! (CG.jl:93-98): u += a p, r -= a w on the interior; returns
 * sum(x -> x^2, r) over the WHOLE array (halo r stays zero). */
double tlo_cg_calc_ur(tlo_chunk *c, double alpha, const tlo_opts *o) {
  const int X = c->x, Y = c->y, hd = c->hd, nx = X - 2 * hd;
  double *u = c->f[TLO_U], *p = c->f[TLO_P], *r = c->f[TLO_R], *w = c->f[TLO_W];
  double acc = 0.0;
  const int ord = o->order;
#pragma omp parallel for num_threads(NT(o)) schedule(static) reduction(+ : acc)
  for (int j = hd; j < Y - hd; ++j)
    for (int i = hd; i < X - hd; ++i) {
      const size_t id = IDX(i, j);
      u[id] = u[id] + alpha * p[id];
      r[id] = r[id] - alpha * w[id];
      const double v = r[id] * r[id];
      if (ord == TLO_ORDER_DEVICE) g_scr.interior[(size_t)(i - hd) + (size_t)(j - hd) * nx] = v;
      else if (ord == TLO_ORDER_THREADS) acc += v;
    }
  if (ord == TLO_ORDER_THREADS) return acc;
  if (ord == TLO_ORDER_DEVICE) return reduce_interior(c, o, PAIRWISE);
  const size_t n = (size_t)X * Y;
  for (size_t k = 0; k < n; ++k) g_scr.full[k] = r[k] * r[k];
  return tlo_pairwise_sum(g_scr.full, (long long)n);
}

/* p! (CG.jl:101-104) */
void tlo_cg_calc_p(tlo_chunk *c, double beta, const tlo_opts *o) {
  const int X = c->x, Y = c->y, hd = c->hd;
  double *p = c->f[TLO_P], *r = c->f[TLO_R];
#pragma omp parallel for num_threads(NT(o)) schedule(static)
  for (int j = hd; j < Y - hd; ++j)
    for (int i = hd; i < X - hd; ++i) p[IDX(i, j)] = beta * p[IDX(i, j)] + r[IDX(i, j)];
}

/* mainstep! (CG.jl:32-44) */
static double cg_mainstep(tlo_chunk *c, int tt, double rro, const tlo_opts *o) {
  const double pw = tlo_cg_calc_w(c, o);
  const double alpha = rro / pw;
  c->cgalpha[tt] = alpha;
  const double rrn = tlo_cg_calc_ur(c, alpha, o);
  const double beta = rrn / rro;
  c->cgbeta[tt] = beta;
  tlo_cg_calc_p(c, beta, o);
  return rrn;
}

/* a.a over the interior (the relative criterion's bb = u0.u0), summed in the
 * order the options select. */
static double interior_dot(tlo_chunk *c, const double *a, const tlo_opts *o) {
  const int X = c->x, Y = c->y, hd = c->hd, nx = X - 2 * hd;
  double acc = 0.0;
  const int store = o->order != TLO_ORDER_THREADS;
#pragma omp parallel for num_threads(NT(o)) schedule(static) reduction(+ : acc)
  for (int j = hd; j < Y - hd; ++j)
    for (int i = hd; i < X - hd; ++i) {
      const double v = a[IDX(i, j)] * a[IDX(i, j)];
      if (store) g_scr.interior[(size_t)(i - hd) + (size_t)(j - hd) * nx] = v; else acc += v;
    }
  return store ? reduce_interior(c, o, SEQ) : acc;
}

/* The true residual t = u0 - A u over the interior; returns t.t.  With
 * `write`, r = p = t (the restart of the relative criterion). */
static double true_residual(tlo_chunk *c, const tlo_opts *o, int write) {
  const int X = c->x, Y = c->y, hd = c->hd, nx = X - 2 * hd;
  double *u = c->f[TLO_U], *u0 = c->f[TLO_U0], *r = c->f[TLO_R], *p = c->f[TLO_P];
  double acc = 0.0;
  const int store = o->order != TLO_ORDER_THREADS;
#pragma omp parallel for num_threads(NT(o)) schedule(static) reduction(+ : acc)
  for (int j = hd; j < Y - hd; ++j)
    for (int i = hd; i < X - hd; ++i) {
      const size_t id = IDX(i, j);
      const double t = u0[id] - smvp(c, u, i, j, o->mode);
      if (write) r[id] = p[id] = t;
      const double v = t * t;
      if (store) g_scr.interior[(size_t)(i - hd) + (size_t)(j - hd) * nx] = v; else acc += v;
    }
  return store ? reduce_interior(c, o, SEQ) : acc;
}

/* solve! (CG.jl:7-29).  With o->criterion == 1 (not in the reference, which
 * tests sqrt|rr| < eps, CG.jl:24) the loop tests sqrt(|rr| / bb) < eps with
 * bb = u0.u0, including before the first iteration; once it holds, the true
 * residual u0 - A u is measured, and while its relative norm is above eps
 * (and iterations remain) CG restarts from it: r = p = u0 - A u. */
static int cg_solve(tlo_chunk *c, tlo_settings *s, const tlo_opts *o, double rx, double ry, tlo_result *res) {
  double rro;
  int rc = tlo_cg_init(c, s->coefficient, rx, ry, o, &rro);
  if (rc) return rc;
  const int up[2] = {TLO_EX_U, TLO_EX_P};
  if ((rc = tlo_halo_update(c, s, o, 1, up, 2, 1))) return rc;
  tlo_copy_u(c, o);
  const int rel = o->criterion == 1;
  const double bb = rel ? interior_dot(c, c->f[TLO_U0], o) : 0.0;
  double error = ERROR_START;
  int iters = 0;
  res->rel_residual = -1.0;
  if (rel) {
    const double rel0 = bb > 0 ? sqrt(rro / bb) : sqrt(rro);
    if (rel0 < s->eps) {
      res->iters = res->cg_iters = 0;
      res->error = rro;
      res->converged = 1;
      res->rel_residual = rel0;
      return TLO_OK;
    }
  }
  int converged = 0;
  for (int restart = 0; restart < 8; ++restart) {
    for (int tt = iters + 1; tt <= s->maxiters; ++tt) {
      iters = tt;
      rro = error = cg_mainstep(c, tt, rro, o);
      if ((rc = tlo_halo_update(c, s, o, 1, NULL, -1, 1))) return rc;
      if (rel ? sqrt(fabs(error) / bb) < s->eps : sqrt(fabs(error)) < s->eps) {
        converged = 1;
        break;
      }
    }
    if (!rel) break;
    const double tr = true_residual(c, o, 0);
    res->rel_residual = bb > 0 ? sqrt(tr / bb) : sqrt(tr);
    converged = res->rel_residual < s->eps;
    if (converged || o->mode == TLO_MODE_REFERENCE || iters >= s->maxiters) break;
    rro = true_residual(c, o, 1);
    if ((rc = tlo_halo_update(c, s, o, 1, up, 2, 1))) return rc;
  }
  res->iters = iters;
  res->cg_iters = iters;
  res->error = error;
  res->converged = converged;
  return TLO_OK;
}

/* ------------------------------------------------------------------------- */
/* Eigenvalue estimate (kernels.jl:19-51)                                      */
/* ------------------------------------------------------------------------- */

/* Number of eigenvalues of the symmetric tridiagonal (d, e) below x, by the
 * Sturm sequence of the LDL^T pivots (e[i] couples rows i-1 and i). */
static int sturm_count(const double *d, const double *e, int n, double x) {
  int count = 0;
  double q = 1.0;
  for (int i = 0; i < n; ++i) {
    double off = (i == 0) ? 0.0 : (e[i] * e[i]) / q;
    q = (d[i] - x) - off;
    if (q == 0.0) q = -DBL_MIN;
    if (q < 0.0) ++count;
  }
  return count;
}

/* k-th smallest eigenvalue (0-based) by bisection on the Gershgorin interval;
 * a fixed 200 halvings keep the host result identical on every machine. */
static double tri_eig_bisect(const double *d, const double *e, int n, int k) {
  double lo = d[0], hi = d[0];
  for (int i = 0; i < n; ++i) {
    double rad = (i > 0 ? fabs(e[i]) : 0.0) + (i + 1 < n ? fabs(e[i + 1]) : 0.0);
    if (d[i] - rad < lo) lo = d[i] - rad;
    if (d[i] + rad > hi) hi = d[i] + rad;
  }
  for (int it = 0; it < 200; ++it) {
    double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (sturm_count(d, e, n, mid) > k) hi = mid; else lo = mid;
  }
  return 0.5 * (lo + hi);
}

/* eigenvalues!: the Lanczos tridiagonal from the CG coefficients
 * (kernels.jl:20-31), its extreme eigenvalues, then the 0.95/1.05 margins
 * (kernels.jl:47-48).  The reference's tqli! (kernels.jl:60-112) is replaced
 * by Sturm bisection, and its one-argument minmax by the min and max. */
int tlo_eigenvalues(tlo_chunk *c, int cgiters, const tlo_opts *o) {
  (void)o;
  const int n = cgiters;
  if (n < 1) { set_msg("no CG iterations for the eigenvalue estimate"); return TLO_ERR_EIGEN; }
  double *d = (double *)malloc(sizeof(double) * n), *e = (double *)calloc((size_t)n + 1, sizeof(double));
  if (!d || !e) { free(d); free(e); return TLO_ERR_NOMEM; }
  /* cgalpha/cgbeta are indexed by the 1-based iteration number */
  for (int ii = 1; ii <= n; ++ii) {
    d[ii - 1] = 1.0 / c->cgalpha[ii];
    if (ii > 1) d[ii - 1] += c->cgbeta[ii - 1] / c->cgalpha[ii - 1];
    if (ii < n) e[ii] = sqrt(c->cgbeta[ii]) / c->cgalpha[ii];
  }
  double emin = tri_eig_bisect(d, e, n, 0), emax = tri_eig_bisect(d, e, n, n - 1);
  free(d); free(e);
  c->eigmin = emin;
  c->eigmax = emax;
  if (c->eigmin < 0 || c->eigmax < 0 || !(c->eigmin == c->eigmin) || !(c->eigmax == c->eigmax)) {
    set_msg("Negative eigenvalue found: (%g, %g) (src/kernels.jl:42)", c->eigmin, c->eigmax);
    return TLO_ERR_EIGEN;
  }
  c->eigmin *= 0.95;
  c->eigmax *= 1.05;
  return TLO_OK;
}

/* ------------------------------------------------------------------------- */
/* Chebyshev (src/solvers/Cheby.jl)                                            */
/* ------------------------------------------------------------------------- */

/* coef! (Cheby.jl:121-135); entries are stored 1-based. */
static void cheby_coef(tlo_chunk *c, int n) {
  c->theta = (c->eigmax + c->eigmin) / 2;
  const double delta = (c->eigmax - c->eigmin) / 2;
  const double sigma = c->theta / delta;
  double rho_o = 1 / sigma;
  if (n > c->maxiters + 1) n = c->maxiters + 1;
  for (int ii = 1; ii <= n; ++ii) {
    const double rho_n = 1 / (2 * sigma - rho_o);
    c->chebyalpha[ii] = rho_n * rho_o;
    c->chebybeta[ii] = 2 * rho_n / delta;
    rho_o = rho_n;
  }
}

/* calciter (Cheby.jl:109-118); a non-finite estimate becomes 0. */
static int cheby_calciter(const tlo_chunk *c, double error, double bb) {
  const double connum = c->eigmax / c->eigmin;
  const double ita = DBL_EPSILON * bb / (4 * error);
  const double gamma = (sqrt(connum) - 1) / (sqrt(connum) + 1);
  const double est = nearbyint((log(ita) / log(10.0)) / (2 * (log(gamma) / log(10.0))));
  if (!(est == est) || fabs(est) > 2147483647.0) return 0;
  return (int)est;
}

/* Cheby init! (Cheby.jl:64-81), tealeaf mode */
static int cheby_init(tlo_chunk *c, tlo_settings *s, const tlo_opts *o, int cgiters, double *bb_out) {
  int rc = tlo_eigenvalues(c, cgiters, o);
  if (rc) return rc;
  cheby_coef(c, s->maxiters - cgiters + 1);
  const int X = c->x, Y = c->y, hd = c->hd, nx = X - 2 * hd;
  double *u = c->f[TLO_U], *u0 = c->f[TLO_U0], *w = c->f[TLO_W], *r = c->f[TLO_R], *p = c->f[TLO_P];
  double acc = 0.0;
  const int store = o->order != TLO_ORDER_THREADS;
#pragma omp parallel for num_threads(NT(o)) schedule(static) reduction(+ : acc)
  for (int j = hd; j < Y - hd; ++j)
    for (int i = hd; i < X - hd; ++i) {
      const size_t id = IDX(i, j);
      const double v = u0[id] * u0[id];
      if (store) g_scr.interior[(size_t)(i - hd) + (size_t)(j - hd) * nx] = v; else acc += v;
    }
  *bb_out = store ? reduce_interior(c, o, PAIRWISE) : acc;
#pragma omp parallel for num_threads(NT(o)) schedule(static)
  for (int j = hd; j < Y - hd; ++j)
    for (int i = hd; i < X - hd; ++i) {
      const size_t id = IDX(i, j);
      const double wv = smvp(c, u, i, j, o->mode);
      w[id] = wv;
      r[id] = u0[id] - wv;
      p[id] = r[id] / c->theta;
    }
#pragma omp parallel for num_threads(NT(o)) schedule(static)
  for (int j = hd; j < Y - hd; ++j)
    for (int i = hd; i < X - hd; ++i) u[IDX(i, j)] = u[IDX(i, j)] + p[IDX(i, j)];
  const int fu = TLO_EX_U;
  return tlo_halo_update(c, s, o, 1, &fu, 1, 1);
}

/* Cheby mainstep! (Cheby.jl:84-106) */
static double cheby_mainstep(tlo_chunk *c, const tlo_opts *o, int chebyiters, int calc2norm, double error) {
  const int X = c->x, Y = c->y, hd = c->hd, nx = X - 2 * hd;
  double *u = c->f[TLO_U], *u0 = c->f[TLO_U0], *w = c->f[TLO_W], *r = c->f[TLO_R], *p = c->f[TLO_P];
  const double ca = c->chebyalpha[chebyiters + 1], cb = c->chebybeta[chebyiters + 1];
#pragma omp parallel for num_threads(NT(o)) schedule(static)
  for (int j = hd; j < Y - hd; ++j)
    for (int i = hd; i < X - hd; ++i) {
      const size_t id = IDX(i, j);
      const double wv = smvp(c, u, i, j, o->mode);
      w[id] = wv;
      r[id] = u0[id] - wv;
      p[id] = ca * p[id] + cb * r[id];
    }
  double acc = 0.0;
  const int store = o->order != TLO_ORDER_THREADS;
#pragma omp parallel for num_threads(NT(o)) schedule(static) reduction(+ : acc)
  for (int j = hd; j < Y - hd; ++j)
    for (int i = hd; i < X - hd; ++i) {
      const size_t id = IDX(i, j);
      u[id] = u[id] + p[id];
      if (calc2norm) {
        const double v = r[id] * r[id];
        if (store) g_scr.interior[(size_t)(i - hd) + (size_t)(j - hd) * nx] = v; else acc += v;
      }
    }
  if (calc2norm) error = store ? reduce_interior(c, o, PAIRWISE) : acc;
  return error;
}

/* Cheby solve! (Cheby.jl:10-61).  Tealeaf-mode fixes: rro is carried from
 * each CG prestep (the reference passes the stale init value, Cheby.jl:33);
 * the CG prologue halo-updates u, p and copies u0 like CG.solve!; the
 * eigen-estimate uses the tt-1 CG steps actually taken (the reference passes
 * tt, whose cgalpha entry is still 0). */
static int cheby_solve(tlo_chunk *c, tlo_settings *s, const tlo_opts *o, double rx, double ry, tlo_result *res) {
  const int ref = o->mode == TLO_MODE_REFERENCE;
  double error = ERROR_START, rro;
  int estiter = 0, chebyiters = 0, rc, iters = 0;
  if ((rc = tlo_cg_init(c, s->coefficient, rx, ry, o, &rro))) return rc;
  if (!ref) {
    const int up[2] = {TLO_EX_U, TLO_EX_P};
    if ((rc = tlo_halo_update(c, s, o, 1, up, 2, 1))) return rc;
    tlo_copy_u(c, o);
  }
  for (int tt = 1; tt <= s->maxiters; ++tt) {
    iters = tt;
    const int sw = chebyiters != 0 ||
                   (s->errorswitch ? (error < s->epslim) && (tt > CGEIGENITERS) : (tt > s->presteps) && (error < ERROR_SWITCH_MAX));
    if (!sw) {
      if (ref) error = cg_mainstep(c, tt, rro, o);
      else rro = error = cg_mainstep(c, tt, rro, o);
    } else {
      chebyiters++;
      if (chebyiters == 1) {
        if (ref) {
          set_msg("MethodError: no method matching minmax(::Vector{Float64}) (src/kernels.jl:39)");
          res->iters = tt; res->cg_iters = tt - 1; res->error = error;
          return TLO_ERR_REFERENCE_THROWS;
        }
        double bb;
        if ((rc = cheby_init(c, s, o, tt - 1, &bb))) return rc;
        error = cheby_mainstep(c, o, chebyiters, 1, error);
        estiter = cheby_calciter(c, error, bb);
      } else {
        const int calc2norm = (chebyiters >= estiter) && ((tt + 1) % 10 == 0);
        error = cheby_mainstep(c, o, chebyiters, calc2norm, error);
      }
    }
    if ((rc = tlo_halo_update(c, s, o, 1, NULL, -1, 1))) return rc;
    if (fabs(error) < s->eps) break;
  }
  res->iters = iters;
  res->cg_iters = iters - chebyiters;
  res->inner_iters = chebyiters;
  res->est_iters = estiter;
  res->error = error;
  res->eigmin = c->eigmin;
  res->eigmax = c->eigmax;
  return TLO_OK;
}

/* ------------------------------------------------------------------------- */
/* PPCG (src/solvers/PPCG.jl)                                                  */
/* ------------------------------------------------------------------------- */

static double interior_rr(tlo_chunk *c, const tlo_opts *o) {
  const int X = c->x, Y = c->y, hd = c->hd, nx = X - 2 * hd;
  const double *r = c->f[TLO_R];
  double acc = 0.0;
  const int store = o->order != TLO_ORDER_THREADS;
#pragma omp parallel for num_threads(NT(o)) schedule(static) reduction(+ : acc)
  for (int j = hd; j < Y - hd; ++j)
    for (int i = hd; i < X - hd; ++i) {
      const double v = r[IDX(i, j)] * r[IDX(i, j)];
      if (store) g_scr.interior[(size_t)(i - hd) + (size_t)(j - hd) * nx] = v; else acc += v;
    }
  return store ? reduce_interior(c, o, PAIRWISE) : acc;
}

/* PPCG mainstep! (PPCG.jl:64-94), tealeaf mode: sd = r/theta starts the inner
 * sweeps (the init!(chunk, hd) overload of PPCG.jl:97-100 that dispatch never
 * reaches); each inner sweep reads the old sd everywhere before sd is
 * updated; the closing r.r is taken over the interior. */
static double ppcg_mainstep(tlo_chunk *c, tlo_settings *s, const tlo_opts *o, double rro, int *rc) {
  const int X = c->x, Y = c->y, hd = c->hd;
  const double pw = tlo_cg_calc_w(c, o);
  const double alpha = rro / pw;
  (void)tlo_cg_calc_ur(c, alpha, o);
  double *u = c->f[TLO_U], *r = c->f[TLO_R], *sd = c->f[TLO_SD];
#pragma omp parallel for num_threads(NT(o)) schedule(static)
  for (int j = hd; j < Y - hd; ++j)
    for (int i = hd; i < X - hd; ++i) sd[IDX(i, j)] = r[IDX(i, j)] / c->theta;
  reset_to_exchange(s);
  s->toexchange[TLO_EX_SD] = 1;
  for (int pp = 1; pp <= s->ppcginnersteps; ++pp) {
    if ((*rc = tlo_halo_update(c, s, o, 1, NULL, -1, 1))) return 0.0;
    const double ca = c->chebyalpha[pp], cb = c->chebybeta[pp];
#pragma omp parallel for num_threads(NT(o)) schedule(static)
    for (int j = hd; j < Y - hd; ++j)
      for (int i = hd; i < X - hd; ++i) {
        const size_t id = IDX(i, j);
        r[id] = r[id] - smvp(c, sd, i, j, o->mode);
        u[id] = u[id] + sd[id];
      }
#pragma omp parallel for num_threads(NT(o)) schedule(static)
    for (int j = hd; j < Y - hd; ++j)
      for (int i = hd; i < X - hd; ++i) {
        const size_t id = IDX(i, j);
        sd[id] = ca * sd[id] + cb * r[id];
      }
  }
  reset_to_exchange(s);
  s->toexchange[TLO_EX_P] = 1;
  const double rrn = interior_rr(c, o);
  const double beta = rrn / rro;
  tlo_cg_calc_p(c, beta, o);
  *rc = TLO_OK;
  return rrn;
}

/* PPCG solve! (PPCG.jl:9-55).  Tealeaf-mode fixes: the CG prologue halo
 * update and copyu as in CG.solve!; eigenvalues from the tt-1 CG steps
 * taken; at the switch, init! (residual + halo p) also resets rro to the
 * true residual's r.r so that beta divides consistent norms. */
static int ppcg_solve(tlo_chunk *c, tlo_settings *s, const tlo_opts *o, double rx, double ry, tlo_result *res) {
  const int ref = o->mode == TLO_MODE_REFERENCE;
  int ppcgiters = 0, rc, iters = 0;
  double rro;
  if ((rc = tlo_cg_init(c, s->coefficient, rx, ry, o, &rro))) return rc;
  if (!ref) {
    const int up[2] = {TLO_EX_U, TLO_EX_P};
    if ((rc = tlo_halo_update(c, s, o, 1, up, 2, 1))) return rc;
    tlo_copy_u(c, o);
  }
  double error = ERROR_START;
  for (int tt = 1; tt <= s->maxiters; ++tt) {
    iters = tt;
    const int sw = ppcgiters != 0 ||
                   (s->errorswitch ? (error < s->epslim) && (tt > CGEIGENITERS) : (tt > s->presteps) && (error < ERROR_SWITCH_MAX));
    if (!sw) {
      rro = error = cg_mainstep(c, tt, rro, o);
    } else {
      if (ref) {
        set_msg("UndefVarError: ++ not defined (src/solvers/PPCG.jl:36)");
        res->iters = tt; res->cg_iters = tt - 1; res->error = error;
        return TLO_ERR_REFERENCE_THROWS;
      }
      ppcgiters++;
      if (ppcgiters == 1) {
        if ((rc = tlo_eigenvalues(c, tt - 1, o))) return rc;
        cheby_coef(c, s->ppcginnersteps);
        tlo_residual(c, o);
        rro = interior_rr(c, o);
        const int fp = TLO_EX_P;
        if ((rc = tlo_halo_update(c, s, o, 1, &fp, 1, 1))) return rc;
      }
      rro = error = ppcg_mainstep(c, s, o, rro, &rc);
      if (rc) return rc;
    }
    if ((rc = tlo_halo_update(c, s, o, 1, NULL, -1, 1))) return rc;
    if (fabs(error) < s->eps) break;
  }
  res->iters = iters;
  res->cg_iters = iters - ppcgiters;
  res->inner_iters = ppcgiters;
  res->error = error;
  res->eigmin = c->eigmin;
  res->eigmax = c->eigmax;
  return TLO_OK;
}

/* ------------------------------------------------------------------------- */
/* Jacobi (src/solvers/Jacobi.jl)                                              */
/* ------------------------------------------------------------------------- */

/* init! (Jacobi.jl:33-57) */
static int jacobi_init(tlo_chunk *c, tlo_settings *s, const tlo_opts *o, double rx, double ry) {
  if (s->coefficient < TLO_CONDUCTIVITY) {
    set_msg("Coefficient %d is not valid. (src/solvers/Jacobi.jl:35)", s->coefficient);
    return TLO_ERR_COEF;
  }
  const int X = c->x, Y = c->y, hd = c->hd;
  const size_t n = (size_t)X * Y;
  double *u = c->f[TLO_U], *u0 = c->f[TLO_U0], *e = c->f[TLO_ENERGY], *rho = c->f[TLO_DENSITY], *kx = c->f[TLO_KX],
         *ky = c->f[TLO_KY];
#pragma omp parallel for num_threads(NT(o)) schedule(static)
  for (size_t k = 0; k < n; ++k) { const double t = e[k] * rho[k]; u0[k] = t; u[k] = t; }
  const int recip = s->coefficient != TLO_CONDUCTIVITY;
#pragma omp parallel for num_threads(NT(o)) schedule(static)
  for (int j = hd; j < Y - 1; ++j)
    for (int i = hd; i < X - 1; ++i) {
      const double densc = recip ? 1.0 / rho[IDX(i, j)] : rho[IDX(i, j)];
      const double densl = recip ? 1.0 / rho[IDX(i - 1, j)] : rho[IDX(i - 1, j)];
      const double densd = recip ? 1.0 / rho[IDX(i, j - 1)] : rho[IDX(i, j - 1)];
      kx[IDX(i, j)] = rx * (densl + densc) / (2 * densl * densc);
      ky[IDX(i, j)] = ry * (densd + densc) / (2 * densd * densc);
    }
  tlo_copy_u(c, o);
  reset_to_exchange(s);
  s->toexchange[TLO_EX_U] = 1;
  return TLO_OK;
}

/* iterate! (Jacobi.jl:59-80): returns sum(abs.(u .- r)) over the whole array */
static double jacobi_iterate(tlo_chunk *c, const tlo_opts *o) {
  const int X = c->x, Y = c->y, hd = c->hd, nx = X - 2 * hd;
  const size_t n = (size_t)X * Y;
  double *u = c->f[TLO_U], *u0 = c->f[TLO_U0], *r = c->f[TLO_R], *kx = c->f[TLO_KX], *ky = c->f[TLO_KY];
  memcpy(r, u, n * sizeof(double));
#pragma omp parallel for num_threads(NT(o)) schedule(static)
  for (int j = hd; j < Y - hd; ++j)
    for (int i = hd; i < X - hd; ++i) {
      const size_t id = IDX(i, j);
      const double num = u0[id] + kx[IDX(i + 1, j)] * r[IDX(i + 1, j)] + kx[id] * r[IDX(i - 1, j)] +
                         ky[IDX(i, j + 1)] * r[IDX(i, j + 1)] + ky[id] * r[IDX(i, j - 1)];
      const double den = 1 + kx[id] + kx[IDX(i + 1, j)] + ky[id] + ky[IDX(i, j + 1)];
      u[id] = num / den;
    }
  if (o->order == TLO_ORDER_REFERENCE) {
    for (size_t k = 0; k < n; ++k) g_scr.full[k] = fabs(u[k] - r[k]);
    return tlo_pairwise_sum(g_scr.full, (long long)n);
  }
  double acc = 0.0;
  const int store = o->order == TLO_ORDER_DEVICE;
#pragma omp parallel for num_threads(NT(o)) schedule(static) reduction(+ : acc)
  for (int j = hd; j < Y - hd; ++j)
    for (int i = hd; i < X - hd; ++i) {
      const double v = fabs(u[IDX(i, j)] - r[IDX(i, j)]);
      if (store) g_scr.interior[(size_t)(i - hd) + (size_t)(j - hd) * nx] = v; else acc += v;
    }
  return store ? reduce_interior(c, o, PAIRWISE) : acc;
}

/* driver! (Jacobi.jl:7-30), tealeaf mode.  The reference never reaches it
 * (it defines driver!, not the solve! that diffuse! calls); the fix resets
 * the error to each sweep's sum|u - r| instead of adding it to ERROR_START. */
static int jacobi_solve(tlo_chunk *c, tlo_settings *s, const tlo_opts *o, double rx, double ry, tlo_result *res) {
  if (o->mode == TLO_MODE_REFERENCE) {
    set_msg("UndefVarError: solve! not defined in module Jacobi (src/TeaLeaf.jl:74, src/solvers/Jacobi.jl:7)");
    res->iters = 0;
    return TLO_ERR_REFERENCE_THROWS;
  }
  int rc = jacobi_init(c, s, o, rx, ry), iters = 0;
  if (rc) return rc;
  double error = ERROR_START;
  for (int tt = 1; tt <= s->maxiters; ++tt) {
    error = jacobi_iterate(c, o);
    if (tt % 50 == 0) {
      if ((rc = tlo_halo_update(c, s, o, 1, NULL, -1, 1))) return rc;
      tlo_residual(c, o);
      error += interior_rr(c, o);
    }
    if ((rc = tlo_halo_update(c, s, o, 1, NULL, -1, 1))) return rc;
    iters = tt;
    if (fabs(error) < s->eps) break;
  }
  res->iters = iters;
  res->error = error;
  return TLO_OK;
}

/* ------------------------------------------------------------------------- */
/* Driver (src/TeaLeaf.jl)                                                     */
/* ------------------------------------------------------------------------- */

int tlo_solve(tlo_chunk *c, tlo_settings *s, const tlo_opts *o, double rx, double ry, tlo_result *res) {
  memset(res, 0, sizeof *res);
  res->rel_residual = -1.0;
  if (!ensure_scratch(c)) return TLO_ERR_NOMEM;
  int rc;
  switch (s->solver) {
    case TLO_CG: rc = cg_solve(c, s, o, rx, ry, res); break;
    case TLO_CHEBY: rc = cheby_solve(c, s, o, rx, ry, res); break;
    case TLO_PPCG: rc = ppcg_solve(c, s, o, rx, ry, res); break;
    case TLO_JACOBI: rc = jacobi_solve(c, s, o, rx, ry, res); break;
    default: rc = TLO_ERR_ARG;
  }
  res->status = rc;
  return rc;
}

/* initialiseapp! (TeaLeaf.jl:35-44) on an already created chunk */
int tlo_initialise_app(tlo_chunk *c, tlo_settings *s, const tlo_opts *o) {
  int rc = tlo_set_chunk_state(c, s, o);
  if (rc) return rc;
  const int ex[3] = {TLO_EX_DENSITY, TLO_EX_ENERGY0, TLO_EX_ENERGY};
  if ((rc = tlo_halo_update(c, s, o, 1, ex, 3, 1))) return rc;
  memcpy(c->f[TLO_ENERGY], c->f[TLO_ENERGY0], sizeof(double) * (size_t)c->x * c->y);
  return TLO_OK;
}

int tlo_diffuse(tlo_chunk *c, tlo_settings *s, const tlo_opts *o, tlo_result *steps, int maxsteps,
                tlo_summary *summaries, int maxsummaries, int *nsummaries) {
  *nsummaries = 0;
  if (s->endstep > maxsteps) { set_msg("endstep %lld exceeds the step record capacity", s->endstep); return TLO_ERR_ARG; }
  for (long long tt = 1; tt <= s->endstep; ++tt) {
    const double rx = s->dtinit / (s->dx * s->dx);   /* TeaLeaf.jl:69-70: dt/dx^2 */
    const double ry = s->dtinit / (s->dy * s->dy);
    const int ex[2] = {TLO_EX_ENERGY, TLO_EX_DENSITY};
    int rc = tlo_halo_update(c, s, o, 1, ex, 2, 1);
    if (rc) return rc;
    rc = tlo_solve(c, s, o, rx, ry, &steps[tt - 1]);
    if (rc) return rc;
    if ((rc = tlo_solve_finished(c, s, o))) return rc;
    if (tt % s->summaryfrequency == 0 && s->checkresult && *nsummaries < maxsummaries)
      tlo_field_summary(c, o, &summaries[(*nsummaries)++]);
  }
  if (s->checkresult && *nsummaries < maxsummaries) tlo_field_summary(c, o, &summaries[(*nsummaries)++]);
  return TLO_OK;
}
