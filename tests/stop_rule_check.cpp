// Replays a convergence trace through the library's stop rule
// (pm_api_internal.h: stop_record / stop_met / stop_converged) on the host.
//
//   stop_rule_check EPS EPS_FIXED_POINT < trace
//
// The trace is one conv value per line ("nan" allowed).  Prints the 0-based
// index of the evaluation after which the loop ends and whether the result
// counts as converged, or "none" when the trace runs out first.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../poremaps_gb300/csrc/pm_api_internal.h"

int main(int argc, char** argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: stop_rule_check EPS EPS_FIXED_POINT < trace\n");
    return 2;
  }
  pm_params p;
  memset(&p, 0, sizeof p);
  p.eps = strtod(argv[1], nullptr);
  p.eps_fixed_point = strtod(argv[2], nullptr);
  pm::StopState st;
  char line[128];
  int i = 0;
  while (fgets(line, sizeof line, stdin)) {
    const double conv = strtod(line, nullptr);
    pm::stop_record(p, conv, st);
    if (pm::stop_met(p, conv, st)) {
      printf("stop %d converged %d\n", i, pm::stop_converged(p, conv, st) ? 1 : 0);
      return 0;
    }
    ++i;
  }
  printf("none\n");
  return 0;
}
