/*
 * CPU ORACLE for the POREMAPS pseudo-time Stokes sweep (TEST INFRASTRUCTURE).
 *
 * A plain-C restatement of the reference algorithm, used only by tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker.
 * The product (poremaps_gb300) never links or calls it.
 *
 * Parity pin: the restatement is checked bit-for-bit against the reference's
 * own sources built here unmodified (oracle/Makefile target `ref`), see
 * tests/golden/make_golden.py and tests/test_oracle_golden.py.
 *
 * Domain model: one global domain split into `nslabs` z-slabs, each a padded
 * [NZ][NY][NX] array with 2-voxel halos, exactly like the reference run with
 * dom_decomposition 1 1 nslabs (geometry.cc:129-171).  nslabs = 1 is the
 * single-rank run that the GPU product reproduces.
 */
#ifndef PM_ORACLE_H
#define PM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { OR_ORDER_REFERENCE = 0, OR_ORDER_JACOBI = 1, OR_ORDER_REDBLACK = 2 };

typedef struct or_problem or_problem;

typedef struct {
  int iterations;      /* last iteration index evaluated (log row) */
  int sweeps;          /* number of sweeps done */
  double conv;
  double permeability; /* mean(w)/Re, voxel units (compute_convergence) */
  double k13, k23, k33, wk13, wk23, wk33, wmax_velz, wmean_velz;
  double porosity;
} or_result;

/* geom_raw: nx*ny*nz bytes, x fastest, 0 = fluid, nonzero = solid. */
or_problem* or_create(const int size[3], int bc_method, unsigned solver, int nslabs,
                      const unsigned char* geom_raw, double voxel_size, double porosity,
                      const int dom_interest[6]);
void or_destroy(or_problem* pr);

/* n full iterations: [reapply if first] sweep, halo exchange p,u,v,w, reapply. */
void or_iterate(or_problem* pr, int order, int n);

/* The calc_flow loop (calc_flow.cc:53-169). log_path may be NULL. */
void or_calc_flow(or_problem* pr, int order, int max_iter, int it_eval, int it_write, double eps,
                  const char* log_path, or_result* res);

double or_convergence(or_problem* pr, double* permeability);
void or_permeability(or_problem* pr, or_result* res);
double or_porosity(or_problem* pr);

/* Interior fields, x fastest (nx*ny*nz doubles each); any may be NULL. */
void or_get_fields(const or_problem* pr, double* u, double* v, double* w, double* p);
/* Interior neighbourhood codes (100cx+10cy+cz, -1 solid), x fastest. */
void or_get_nhood(const or_problem* pr, int* out);
/* Test hooks: set interior fields; the stencil helpers on their own. */
void or_set_fields(or_problem* pr, const double* u, const double* v, const double* w,
                   const double* p);
double or_second_derivative(int cs, double ll, double l, double m, double r, double rr);
void or_split_code(int code, int out[3]);
/* Full padded arrays of slab s (for halo checks). */
void or_get_padded(const or_problem* pr, int s, int dims_out[3], double* u, double* v, double* w,
                   double* p);
int or_threads(or_problem* pr, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
