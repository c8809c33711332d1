// poremaps_gpu -- drop-in for the reference program on one GB300:
//
//   poremaps_gpu [file.inp] [--order reference|jacobi|redblack]
//                [--precision fp64|mixed] [--arith exact|fast]
//                [--eps-fixed-point X]
//
// Reads the same .inp (default input_param.inp, main_stokes_solver.cc:146-147)
// and .raw geometry, appends the same permeability log rows and writes the
// same velx_/vely_/velz_/press_/voxel_neighborhood_/domain_decomp_ files.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/poremaps.h"

int main(int argc, char** argv) {
  const char* inp = "input_param.inp";
  pm_params ov;
  pm_params_default(&ov);
  for (int a = 1; a < argc; ++a) {
    if (!strcmp(argv[a], "--order") && a + 1 < argc) {
      const char* o = argv[++a];
      ov.order = !strcmp(o, "reference") ? PM_ORDER_REFERENCE
                 : !strcmp(o, "jacobi")  ? PM_ORDER_JACOBI
                 : !strcmp(o, "redblack") ? PM_ORDER_REDBLACK
                                          : PM_ORDER_DEFAULT;
    } else if (!strcmp(argv[a], "--precision") && a + 1 < argc) {
      ov.precision = !strcmp(argv[++a], "mixed") ? PM_PREC_MIXED : PM_PREC_FP64;
    } else if (!strcmp(argv[a], "--arith") && a + 1 < argc) {
      ov.arith = !strcmp(argv[++a], "exact") ? PM_ARITH_EXACT : PM_ARITH_FAST;
    } else if (!strcmp(argv[a], "--eps-fixed-point") && a + 1 < argc) {
      ov.eps_fixed_point = strtod(argv[++a], nullptr);
    } else if (argv[a][0] != '-') {
      inp = argv[a];
    } else {
      fprintf(stderr, "unknown option %s\n", argv[a]);
      return 2;
    }
  }
  if (argc == 1) printf("No input file specified. Using input_param.inp\n");
  else printf("Input file: %s\n", inp);
  if (ov.order == PM_ORDER_REFERENCE) ov.arith = PM_ARITH_EXACT;
  pm_result r;
  memset(&r, 0, sizeof r);
  printf("START MAIN COMPUTATION\n");
  pm_status s = pm_run_inp(inp, &ov, &r);
  if (s != PM_OK && s != PM_ERR_NONFINITE) {
    fprintf(stderr, "poremaps_gpu: %s\n", pm_last_error());
    return 1;
  }
  printf("Iterations: %d (sweeps %d)  Convergence: %e  wk33: %e m^2  GLUP/s: %.3f\n",
         r.iterations, r.sweeps, r.conv, r.wk33, r.glups);
  printf("Writing output to file\n");
  return s == PM_OK ? 0 : 3;
}
