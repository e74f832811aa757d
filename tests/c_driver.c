/* A plain C driver of the library (test infrastructure): reads a tea.in deck
 * with tl_parse_deck, runs diffuse! on the device with tl_diffuse and prints
 * the field summaries, one line each: "summary <vol> <mass> <ie> <temp>" in
 * %.17g, then "iters <n1> <n2> ...".
 *
 * usage: c_driver <deck> <mode 0|1> <precision 0|1> <criterion 0|1> <exact 0|1>
 */
#include <stdio.h>
#include <stdlib.h>

#include "tealeaf_gb300.h"

int main(int argc, char **argv) {
  if (argc < 6) {
    fprintf(stderr, "usage: %s deck mode precision criterion exact\n", argv[0]);
    return 2;
  }
  FILE *f = fopen(argv[1], "rb");
  if (!f) {
    perror(argv[1]);
    return 2;
  }
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  rewind(f);
  char *text = (char *)calloc((size_t)n + 1, 1);
  if (fread(text, 1, (size_t)n, f) != (size_t)n) {
    fclose(f);
    return 2;
  }
  fclose(f);
  const int mode = atoi(argv[2]);
  tl_deck d;
  tl_state st[64];
  char err[256];
  if (tl_parse_deck(text, mode, &d, st, 64, err, (int)sizeof err)) {
    fprintf(stderr, "deck: %s\n", err);
    return 1;
  }
  tl_config cfg = {d.xcells, d.ycells, d.halodepth, d.maxiters, d.xmin, d.ymin, d.dx, d.dy, mode};
  tl_ctx *ctx = NULL;
  if (tl_create(&ctx, &cfg) || tl_initialise(ctx, st, d.nstates < 64 ? d.nstates : 64)) {
    fprintf(stderr, "create: %s\n", ctx ? tl_last_error(ctx) : "no context");
    return 1;
  }
  tl_params p = {d.solver, d.coefficient, d.maxiters, d.presteps, d.ppcginnersteps, d.errorswitch, d.eps,
                 d.epslim, atoi(argv[4]), atoi(argv[3]), atoi(argv[5]), TL_WARM_OFF};
  const int steps = (int)d.endstep;
  tl_result *res = (tl_result *)calloc((size_t)steps, sizeof *res);
  double sums[4 * 64];
  int ns = 0;
  if (tl_diffuse(ctx, &p, d.dtinit, steps, d.summaryfrequency, d.checkresult, res, sums, 64, &ns)) {
    fprintf(stderr, "diffuse: %s\n", tl_last_error(ctx));
    return 1;
  }
  for (int k = 0; k < ns; ++k)
    printf("summary %.17g %.17g %.17g %.17g\n", sums[4 * k], sums[4 * k + 1], sums[4 * k + 2], sums[4 * k + 3]);
  printf("iters");
  for (int k = 0; k < steps; ++k) printf(" %d", res[k].iters);
  printf("\n");
  tl_destroy(ctx);
  free(res);
  free(text);
  return 0;
}
