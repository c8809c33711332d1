/*
 * oracle_cli -- command-line driver of the CPU ORACLE (TEST INFRASTRUCTURE).
 *
 *   oracle_cli file.inp [--order reference|jacobi|redblack] [--slabs P]
 *              [--threads T] [--sweeps N] [--log path]
 *
 * Reads the reference's fixed-order .inp (read_problem_params.cc:75-91) and
 * .raw geometry, then either runs the calc_flow loop (default) or exactly N
 * iterations (--sweeps, used as the bounded CPU-baseline sample).  Prints one
 * JSON line with the result and the wall time of the sweep loop.
 */
#define _POSIX_C_SOURCE 200809L
#include "pm_oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: oracle_cli file.inp [--order o] [--slabs P] [--threads T] [--sweeps N]\n");
    return 2;
  }
  int order = OR_ORDER_REFERENCE, slabs = 1, threads = 1, sweeps = -1;
  const char* log_override = NULL;
  for (int a = 2; a < argc; ++a) {
    if (!strcmp(argv[a], "--order") && a + 1 < argc) {
      ++a;
      order = !strcmp(argv[a], "jacobi") ? OR_ORDER_JACOBI
              : !strcmp(argv[a], "redblack") ? OR_ORDER_REDBLACK : OR_ORDER_REFERENCE;
    } else if (!strcmp(argv[a], "--slabs") && a + 1 < argc) slabs = atoi(argv[++a]);
    else if (!strcmp(argv[a], "--threads") && a + 1 < argc) threads = atoi(argv[++a]);
    else if (!strcmp(argv[a], "--sweeps") && a + 1 < argc) sweeps = atoi(argv[++a]);
    else if (!strcmp(argv[a], "--log") && a + 1 < argc) log_override = argv[++a];
  }
  FILE* f = fopen(argv[1], "r");
  if (!f) { fprintf(stderr, "cannot open %s\n", argv[1]); return 1; }
  int dd[3], bc, size[3], max_iter, it_eval, it_write, di[6], wo[4];
  unsigned solver;
  double dx, eps, porosity;
  char geom[400], logf[400];
  int n = 0;
  n += fscanf(f, "dom_decomposition %d %d %d \n", &dd[0], &dd[1], &dd[2]);
  n += fscanf(f, "boundary_method %d \n", &bc);
  n += fscanf(f, "geometry_file_name %399s \n", geom);
  n += fscanf(f, "size_x_y_z %d %d %d \n", &size[0], &size[1], &size[2]);
  n += fscanf(f, "voxel_size  %lf \n", &dx);
  n += fscanf(f, "max_iter %d \n", &max_iter);
  n += fscanf(f, "it_eval %d \n", &it_eval);
  n += fscanf(f, "it_write %d \n", &it_write);
  n += fscanf(f, "log_file_name %399s \n", logf);
  n += fscanf(f, "solving_algorithm %u \n", &solver);
  n += fscanf(f, "eps %lf \n", &eps);
  n += fscanf(f, "porosity %lf \n", &porosity);
  n += fscanf(f, "dom_interest %d %d %d %d %d %d \n", &di[0], &di[1], &di[2], &di[3], &di[4], &di[5]);
  n += fscanf(f, "write_output %d %d %d %d \n", &wo[0], &wo[1], &wo[2], &wo[3]);
  fclose(f);
  if (n != 26) { fprintf(stderr, "malformed input file (%d fields)\n", n); return 1; }
  long nvox = (long)size[0] * size[1] * size[2];
  unsigned char* g = (unsigned char*)malloc(nvox);
  FILE* gf = fopen(geom, "rb");
  if (!gf || (long)fread(g, 1, nvox, gf) != nvox) { fprintf(stderr, "cannot read %s\n", geom); return 1; }
  fclose(gf);
  or_problem* pr = or_create(size, bc, solver, slabs, g, dx, porosity, di);
  if (!pr) { fprintf(stderr, "bad decomposition\n"); return 1; }
  or_threads(pr, threads);
  or_result res;
  memset(&res, 0, sizeof(res));
  double t0 = now_s();
  if (sweeps >= 0) {
    or_iterate(pr, order, sweeps);
    res.sweeps = sweeps;
  } else {
    or_calc_flow(pr, order, max_iter, it_eval, it_write, eps, log_override ? log_override : logf, &res);
  }
  double el = now_s() - t0;
  if (sweeps >= 0) {
    double perm = 0.0;
    res.conv = or_convergence(pr, &perm);
    res.permeability = perm;
    or_permeability(pr, &res);
  }
  printf("{\"sweeps\": %d, \"iterations\": %d, \"seconds\": %.6f, \"mlups\": %.3f, \"conv\": %.17g, "
         "\"wk13\": %.17g, \"wk23\": %.17g, \"wk33\": %.17g, \"porosity\": %.17g, \"slabs\": %d, "
         "\"threads\": %d}\n",
         res.sweeps, res.iterations, el, el > 0 ? (double)nvox * res.sweeps / el / 1e6 : 0.0,
         res.conv, res.wk13, res.wk23, res.wk33, res.porosity, slabs, threads);
  or_destroy(pr);
  free(g);
  return 0;
}
