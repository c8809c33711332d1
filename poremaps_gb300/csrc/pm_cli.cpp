// poremaps_gpu -- drop-in for the reference program on one GB300:
//
//   poremaps_gpu [file.inp] [--order reference|jacobi|redblack]
//                [--precision fp64|mixed] [--arith exact|fast]
//                [--eps-fixed-point X] [--tensor] [--report out.json]
//
// Reads the same .inp (default input_param.inp, main_stokes_solver.cc:146-147)
// and .raw geometry, appends the same permeability log rows and writes the
// same velx_/vely_/velz_/press_/voxel_neighborhood_/domain_decomp_ files.
//
// --tensor runs the three axis-rotated solves of the full permeability
// tensor (README.md:215-227 of the reference describes doing this by hand
// with rotated geometry files) and prints the 3x3 tensor; no log rows or
// field files are written in that mode.
// --report writes a machine-readable summary (iterations, every permeability
// component at full precision, the tensor when computed, GLUP/s, device and
// wall time) as one JSON object; the reference's log keeps its 7 digits.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <vector>

#include "../../include/poremaps.h"

namespace {

void json_result(FILE* f, const pm_result& r) {
  fprintf(f,
          "{\"iterations\": %d, \"sweeps\": %d, \"converged\": %d, \"conv\": %.17g, "
          "\"permeability\": %.17g, \"k13\": %.17g, \"k23\": %.17g, \"k33\": %.17g, "
          "\"wk13\": %.17g, \"wk23\": %.17g, \"wk33\": %.17g, \"wmax_velz\": %.17g, "
          "\"wmean_velz\": %.17g, \"porosity\": %.17g, \"device_ms\": %.6f, "
          "\"wall_ms\": %.6f, \"glups\": %.6f}",
          r.iterations, r.sweeps, r.converged, r.conv, r.permeability, r.k13, r.k23, r.k33,
          r.wk13, r.wk23, r.wk33, r.wmax_velz, r.wmean_velz, r.porosity, r.device_ms,
          r.wall_ms, r.glups);
}

const char* status_name(pm_status s) {
  switch (s) {
    case PM_OK: return "ok";
    case PM_ERR_NONFINITE: return "nonfinite";
    default: return "error";
  }
}

// One JSON object: the single solve (tensor == nullptr) or the three rotated
// solves and the tensor.
bool write_report(const char* path, const char* inp, const pm_params& p, pm_status s,
                  const pm_result* r, int nres, const double* K, double wall_ms) {
  FILE* f = fopen(path, "w");
  if (!f) return false;
  fprintf(f, "{\"input\": \"%s\", \"geometry\": \"%s\", \"size\": [%d, %d, %d], "
             "\"solving_algorithm\": %u, \"boundary_method\": %d, \"eps\": %.17g, "
             "\"order\": %d, \"precision\": \"%s\", \"status\": \"%s\", \"wall_ms\": %.3f",
          inp, p.geometry_file_name, p.size[0], p.size[1], p.size[2], p.solving_algorithm,
          p.boundary_method, p.eps, p.order, p.precision == PM_PREC_MIXED ? "mixed" : "fp64",
          status_name(s), wall_ms);
  if (K) {
    fprintf(f, ", \"tensor_m2\": [");
    for (int i = 0; i < 9; ++i) fprintf(f, "%s%.17g", i ? ", " : "", K[i]);
    fprintf(f, "], \"solves\": [");
    for (int a = 0; a < nres; ++a) {
      if (a) fprintf(f, ", ");
      json_result(f, r[a]);
    }
    fprintf(f, "]");
  } else {
    fprintf(f, ", \"result\": ");
    json_result(f, r[0]);
  }
  fprintf(f, "}\n");
  return fclose(f) == 0;
}

int run_tensor(const char* inp, const pm_params& ov, const char* report) {
  pm_params p;
  if (pm_read_params(inp, &p) != PM_OK) {
    fprintf(stderr, "poremaps_gpu: %s\n", pm_last_error());
    return 1;
  }
  p.order = ov.order;
  p.precision = ov.precision;
  p.arith = ov.arith;
  p.mixed_inner = ov.mixed_inner;
  p.eps_fixed_point = ov.eps_fixed_point;
  std::vector<uint8_t> geom((size_t)p.size[0] * p.size[1] * p.size[2]);
  if (pm_read_geometry(p.geometry_file_name, p.size, geom.data()) != PM_OK) {
    fprintf(stderr, "poremaps_gpu: %s\n", pm_last_error());
    return 1;
  }
  double K[9];
  pm_result r3[3];
  memset(r3, 0, sizeof r3);
  auto t0 = std::chrono::steady_clock::now();
  pm_status s = pm_solve_tensor(&p, geom.data(), K, r3);
  double wall =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (s != PM_OK && s != PM_ERR_NONFINITE) {
    fprintf(stderr, "poremaps_gpu: %s\n", pm_last_error());
    return 1;
  }
  printf("Permeability tensor [m^2] (row i: response along axis i; column j: pressure "
         "drop along axis j)\n");
  for (int i = 0; i < 3; ++i) printf("  %e %e %e\n", K[3 * i], K[3 * i + 1], K[3 * i + 2]);
  const char* ax = "xyz";
  for (int a = 0; a < 3; ++a)
    printf("Flow along %c: iterations %d, converged %d, conv %e\n", ax[a], r3[a].iterations,
           r3[a].converged, r3[a].conv);
  if (report && !write_report(report, inp, p, s, r3, 3, K, wall)) {
    fprintf(stderr, "poremaps_gpu: cannot write %s\n", report);
    return 1;
  }
  return s == PM_OK ? 0 : 3;
}

}  // namespace

int main(int argc, char** argv) {
  const char* inp = "input_param.inp";
  const char* report = nullptr;
  bool tensor = false;
  bool given = false;
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
    } else if (!strcmp(argv[a], "--report") && a + 1 < argc) {
      report = argv[++a];
    } else if (!strcmp(argv[a], "--tensor")) {
      tensor = true;
    } else if (argv[a][0] != '-') {
      inp = argv[a];
      given = true;
    } else {
      fprintf(stderr, "unknown option %s\n", argv[a]);
      return 2;
    }
  }
  if (!given) printf("No input file specified. Using input_param.inp\n");
  else printf("Input file: %s\n", inp);
  if (ov.order == PM_ORDER_REFERENCE) ov.arith = PM_ARITH_EXACT;
  printf("START MAIN COMPUTATION\n");
  if (tensor) return run_tensor(inp, ov, report);
  pm_result r;
  memset(&r, 0, sizeof r);
  auto t0 = std::chrono::steady_clock::now();
  pm_status s = pm_run_inp(inp, &ov, &r);
  double wall =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (s != PM_OK && s != PM_ERR_NONFINITE) {
    fprintf(stderr, "poremaps_gpu: %s\n", pm_last_error());
    return 1;
  }
  printf("Iterations: %d (sweeps %d)  Convergence: %e  wk33: %e m^2  GLUP/s: %.3f\n",
         r.iterations, r.sweeps, r.conv, r.wk33, r.glups);
  printf("Writing output to file\n");
  if (report) {
    pm_params p;
    if (pm_read_params(inp, &p) != PM_OK) p = ov;
    p.order = ov.order;
    p.precision = ov.precision;
    if (!write_report(report, inp, p, s, &r, 1, nullptr, wall)) {
      fprintf(stderr, "poremaps_gpu: cannot write %s\n", report);
      return 1;
    }
  }
  return s == PM_OK ? 0 : 3;
}
