/*
 * poremaps_gb300 -- C ABI of the GB300 (sm_103a) POREMAPS permeability solver.
 *
 * One process, one GPU, one device-resident domain per problem.  Every entry
 * point is extern "C", takes plain pointers and sizes, returns pm_status and
 * never aborts or prints.  The library owns all device memory it allocates;
 * host buffers passed in are owned by the caller.  Calls on distinct problems
 * are thread-safe (each problem has its own CUDA stream); calls on one
 * problem must not overlap.
 *
 * Reference interfaces replaced (paths inside the krachdd/poremaps project):
 *   pm_read_params        read_problem_params / read_parallel_params
 *                         (src/read_problem_params.cc:50-156)
 *   pm_read_geometry      read_geometry (src/geometry.cc:58-126)
 *   pm_problem_create     get_dom_limits + eval_geometry + allocate_initial_field
 *                         + set_halos_initial (src/geometry.cc:129-302,
 *                         src/initialize.cc:69-289, src/main_stokes_solver.cc:161-276)
 *   pm_solve              calc_flow (src/calc_flow.cc:53-169; declared in
 *                         src/calc_flow.h:36-61)
 *   pm_iterate            one calc_flow iteration body: central_diff5
 *                         (src/solver.cc:112-224) + communicate_halos
 *                         (src/parallelization.cc:193-318) +
 *                         reapply_pressure_gradient (src/boundary_conditions.cc:46-79)
 *   pm_compute_convergence compute_convergence (src/evaluation.cc:216-262)
 *   pm_compute_permeability compute_permeability (src/evaluation.cc:54-211)
 *   pm_get_porosity       get_porosity (src/geometry.cc:335-364)
 *   pm_get_fields / pm_write_outputs / pm_write_log_row
 *                         write_output_raw, write_domain_decomposition,
 *                         write_logfile (src/output.cc:53-230)
 *   pm_run_inp            the POREMAPS program (src/main_stokes_solver.cc:57-416)
 */
#ifndef POREMAPS_GB300_H
#define POREMAPS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  PM_OK = 0,
  PM_ERR_INVALID = 1,   /* bad argument or parameter value */
  PM_ERR_IO = 2,        /* file missing, short or unwritable */
  PM_ERR_CUDA = 3,      /* CUDA runtime error (message in pm_last_error) */
  PM_ERR_NOMEM = 4,     /* device or host allocation failed / over budget */
  PM_ERR_NONFINITE = 5, /* NaN/Inf detected in a reduction */
  PM_ERR_BUSY = 6,      /* server full / request not finished */
  PM_ERR_NOT_FOUND = 7,
  PM_ERR_CANCELLED = 8  /* server request withdrawn by pm_server_cancel */
} pm_status;

/* sweep ordering on the device */
typedef enum {
  PM_ORDER_DEFAULT = -1,  /* REDBLACK for every solver */
  PM_ORDER_REFERENCE = 0, /* the reference's in-place lexicographic order, run as an exact
                             hyperplane wavefront: bit-identical to the reference */
  PM_ORDER_JACOBI = 1,    /* ping-pong: every neighbour from the previous iterate
                             (diverges for solver 1, whose pressure update uses the
                             pre-update velocities; solvers 2 and 3 are stable) */
  PM_ORDER_REDBLACK = 2   /* red then black half-sweeps, +-2 same-colour reads old */
} pm_order;

typedef enum {
  PM_PREC_FP64 = 0,  /* fields stored and swept in FP64 */
  PM_PREC_MIXED = 1  /* FP32 correction sweeps + FP64 residual/defect correction
                        (Jacobi ordering; solvers 2 and 3) */
} pm_precision;

typedef enum {
  PM_ARITH_EXACT = 0, /* the reference's operation order, no FMA contraction */
  PM_ARITH_FAST = 1   /* coefficient form with FMA (a few ulp from EXACT per sweep) */
} pm_arith;

/* The 14 keys of the reference .inp file (input_template.inp, README.md:86-101), in order,
 * plus GPU extensions. */
typedef struct {
  int dom_decomposition[3];     /* parsed and ignored: one device-resident domain */
  int boundary_method;          /* 0..4 */
  char geometry_file_name[400];
  int size[3];                  /* nx, ny, nz */
  double voxel_size;            /* m */
  int max_iter;
  int it_eval;
  int it_write;
  char log_file_name[400];
  unsigned solving_algorithm;   /* 1 Jacobi, 2 Gauss-Seidel, 3 SOR (update formula) */
  double eps;
  double porosity;              /* -1: computed from the geometry */
  int dom_interest[6];          /* xmin xmax ymin ymax zmin zmax (inclusive), all 0 = off */
  int write_output[4];          /* vel, press, neighbourhood, domain decomposition */
  /* ---- GPU extensions (pm_params_default sets them) ---- */
  int order;                    /* pm_order */
  int precision;                /* pm_precision */
  int arith;                    /* pm_arith (FP64 sweeps) */
  int write_log;                /* 1: append the reference log rows to log_file_name */
  int mixed_inner;              /* FP32 sweeps per FP64 correction (0 = it_eval) */
  int kernel;                   /* correction sweep of the mixed form: -1 autotune
                                   (default: time the kernels 10, 9, 8, 6, 5, 7, 2 on
                                   the problem; the first is kept unless another is
                                   at least 5 % faster),
                                   0 TMA z-march 32x16 tiles, 3 TMA
                                   z-march 32x8 tiles, 1 fluid-list gather, 2 fluid-list
                                   gather at four blocks per SM, 4 TMA bricks (one
                                   brick + halo per CTA in shared memory), 5 / 6 / 7
                                   persistent fluid-list gather, list prefetched, at
                                   four / three / two blocks per SM, 8 / 9 / 10
                                   persistent sweep over a compact store (correction
                                   and residual of fluid voxels only, in fluid-list
                                   order, six neighbour positions per voxel) at
                                   three / four blocks per SM with the next
                                   positions prefetched, five blocks per SM without,
                                   11 / 12 the same with each chunk's positions
                                   staged in shared memory by bulk copies at five /
                                   four blocks per SM, 13 the same with the six
                                   positions and the metadata in one 16-byte packed
                                   record per voxel (16-bit offsets) at five blocks
                                   per SM */
  int brick[3];                 /* fluid-list order when kernel >= 0: brick extents
                                   x y z (voxels), 0 0 0 = lexicographic; kernel 4 takes
                                   32 8 8 (default), 32 8 4 or 32 4 4 */
  double eps_fixed_point;       /* 0 (default): stop at conv < eps as the reference does.
                                   > 0: stop at conv < eps_fixed_point instead, or when
                                   conv stagnates at its rounding floor: the largest conv
                                   of a window of 10 evaluations is below 1e-13 and no
                                   smaller than the previous window's.  Both count as
                                   converged.  Runs the fast orders and the mixed form to
                                   the fixed point, where their permeability agrees with
                                   the reference order's to far below eps */
} pm_params;

typedef struct {
  int iterations;     /* iteration index of the last convergence evaluation */
  int sweeps;         /* sweeps performed (iterations + 1 when stopped by eps) */
  int converged;      /* 1 if the stop rule (conv < eps, or eps_fixed_point's) ended the loop */
  double conv;
  double permeability; /* mean(w)/Re in voxel units (compute_convergence) */
  double k13, k23, k33;        /* dom_interest box (0 if off) */
  double wk13, wk23, wk33;     /* whole domain, m^2 */
  double wmax_velz, wmean_velz; /* m/s (velocity x voxel size) */
  double porosity;
  double device_ms;   /* device time of the sweep loop (CUDA events on the problem stream) */
  double wall_ms;     /* host wall time of pm_solve */
  double glups;       /* nx*ny*nz*sweeps / device time, 1e9/s */
} pm_result;

typedef struct pm_problem pm_problem;

/* The calling thread's last error message (thread-local; valid until that
 * thread's next failing call). */
const char* pm_last_error(void);
/* The same message copied into a caller-owned buffer, NUL-terminated and
 * truncated to size - 1 bytes (nothing is written when size is 0); returns
 * the full message length.  For bindings that cannot hold a pointer into the
 * library (cgo, JNI). */
size_t pm_last_error_copy(char* buf, size_t size);
const char* pm_version(void);
pm_status pm_params_default(pm_params* p);

pm_status pm_read_params(const char* inp_path, pm_params* out);
pm_status pm_read_geometry(const char* raw_path, const int size[3], uint8_t* out);

/* geom: nx*ny*nz bytes, x fastest, 0 = fluid, nonzero = solid (copied to the device). */
pm_status pm_problem_create(const pm_params* p, const uint8_t* geom, pm_problem** out);
pm_status pm_problem_destroy(pm_problem* pr);

/* Full calc_flow loop; fills res.  Re-entrant: a second call continues iterating. */
pm_status pm_solve(pm_problem* pr, pm_result* res);
/* n iterations (sweep + halo exchange + pressure reapply) without convergence checks. */
pm_status pm_iterate(pm_problem* pr, int n);
pm_status pm_compute_convergence(pm_problem* pr, double* permeability, double* conv);
pm_status pm_compute_permeability(pm_problem* pr, pm_result* res);
pm_status pm_get_porosity(pm_problem* pr, double* porosity);
pm_status pm_get_iteration(pm_problem* pr, int* iteration);

/* Interior fields, x fastest, nx*ny*nz doubles each; any pointer may be NULL.
 * Unscaled (the writers multiply velocities by voxel_size). */
pm_status pm_get_fields(pm_problem* pr, double* u, double* v, double* w, double* p);
/* Restart from interior fields (the inverse of pm_get_fields): replaces the
 * state, refreshes the periodic halos, reapplies the pressure planes and sets
 * the iteration counter.  The next convergence check compares against k = 0,
 * as the first check of a fresh run does.  No counterpart in the reference
 * (it has no restart); it is the resume half of checkpointing through the
 * field dumps. */
pm_status pm_set_fields(pm_problem* pr, const double* u, const double* v, const double* w,
                        const double* p, int iteration);
/* Reads velx_/vely_/velz_/press_<geometry_file_name> from the working
 * directory as pm_write_outputs wrote them (velocities divided by voxel_size)
 * and calls pm_set_fields.  No counterpart in the reference. */
pm_status pm_resume_outputs(pm_problem* pr, int iteration);
/* Interior neighbourhood codes 100*cx + 10*cy + cz (-1 solid), x fastest. */
pm_status pm_get_neighborhood(pm_problem* pr, int32_t* out);
/* Writes velx_/vely_/velz_/press_/voxel_neighborhood_/domain_decomp_ + geometry name per
 * write_output, byte-compatible with the reference writers. */
pm_status pm_write_outputs(pm_problem* pr);

/* The whole POREMAPS program on one .inp file (log + field files); res may be NULL.
 * overrides (may be NULL) supplies the GPU extensions order, precision, arith,
 * mixed_inner and eps_fixed_point; the .inp supplies everything else. */
pm_status pm_run_inp(const char* inp_path, const pm_params* overrides, pm_result* res);

/* Full permeability tensor from three axis-rotated solves of one geometry
 * (README.md:215-227).  K is row-major 3x3 in m^2, K[3*i+j] = k_(i+1)(j+1): the
 * response along axis i to a unit pressure drop along axis j.  res3 (may be NULL)
 * receives the three solves (flow along x, y, z). */
pm_status pm_solve_tensor(const pm_params* p, const uint8_t* geom, double K[9],
                          pm_result res3[3]);

/* ---- device selection, timing and re-use (bench and serving support) ---- */
/* Select the CUDA device for problems created afterwards by this thread. */
pm_status pm_set_device(int device);
/* Back to the initial state (iteration 0, fields as after pm_problem_create). */
pm_status pm_problem_reset(pm_problem* pr);
/* n iterations, then (if check) the convergence evaluation of
 * compute_convergence; *device_ms = CUDA-event time on the problem's stream
 * from before the first sweep to after the reduction's read-back. */
pm_status pm_block_timed(pm_problem* pr, int n, int check, double* permeability, double* conv,
                         double* device_ms);
/* pm_block_timed for `count` problems at once: each problem's n iterations
 * (and check) are issued on its own stream so the blocks run concurrently;
 * *device_ms = CUDA-event time from a start event every stream waits on to an
 * end event that waits on every stream.  permeability/conv: arrays of count.
 * No counterpart in the reference. */
pm_status pm_block_group_timed(pm_problem** prs, int count, int n, int check,
                               double* permeability, double* conv, double* device_ms);
/* Average device time of one launch of a sweep kernel of this problem's form,
 * measured with CUDA events over n back-to-back launches on its stream
 * (kernel 0: the form's main sweep -- the FP32 correction sweep of the mixed
 * form, the Jacobi/red-black FP64 sweep otherwise).  The state is restored. */
pm_status pm_kernel_time(pm_problem* pr, int kernel, int n, double* avg_ms);
/* The correction-sweep kernel a mixed-precision problem uses (pm_params.kernel
 * values; the autotuned choice when it was created with kernel = -1). */
pm_status pm_get_kernel(pm_problem* pr, int* kernel);
/* Brick order of the problem's fluid list (x, y, z extents; 0 0 0 = lexicographic
 * rows): the autotuner's choice for the mixed form. */
pm_status pm_get_brick(pm_problem* pr, int brick[3]);
/* Number of kernels this library has launched in this process. */
uint64_t pm_kernel_launches(void);

/* ---- allocation-free sums (no counterpart in the reference) ----
 * For callers that cannot let a library allocate device memory: a serving
 * process whose HBM is reserved up front by its own admission control, or a
 * host framework that owns every device allocation (a cudaMalloc/cudaFree
 * inside its stream work would also synchronise the device).  Computes, over
 * device buffers the caller owns, the nine sums behind compute_permeability /
 * compute_convergence, over fluid voxels (geom == 0) only:
 *   sums[0..3] = sum u, sum v, sum w, max(0, max w)
 *   sums[4..8] = dom_interest box: sum u, sum v, sum w, sum p on its zmin plane,
 *                sum p on its zmax plane (zeros when dom_interest is all 0 / NULL)
 * geom, u, v, w, p: device arrays of nx*ny*nz elements, x fastest; sums: 9
 * doubles in device memory.  Launches on `stream` (a cudaStream_t; NULL = the
 * default stream) and returns without synchronising.  No cudaMalloc, cudaFree
 * or allocating library call: the only scratch is a fixed device array of the
 * library (ny*nz <= 16384 rows, 1.18 MB, held by every GPU that loads the
 * library until exit); larger sizes return PM_ERR_INVALID.  All calls share that
 * array, so calls that overlap on the GPU race.  The first call on a device
 * looks up the array's address with that device current; make it before any
 * stream capture.  The address is kept for the life of the process: do not
 * call this after cudaDeviceReset on that device.  The fluid-voxel counts that
 * turn the sums into permeabilities (all fluid voxels, those in the box and on
 * its zmin / zmax planes; evaluation.cc:192-210) are not returned: the caller
 * counts them from its geometry. */
pm_status pm_reduce_fields_noalloc(const int size[3], const uint8_t* geom, const double* u,
                                   const double* v, const double* w, const double* p,
                                   const int dom_interest[6], double* sums, void* stream);

/* Device bytes pm_problem_create will hold for these parameters (fields,
 * lists, codes, scratch): the footprint the server admits requests by.  No
 * counterpart in the reference. */
pm_status pm_problem_footprint(const pm_params* p, size_t* bytes);

/* ---- batched / serving form: many uneven samples resident at once ---- */
typedef struct {
  size_t hbm_budget_bytes;  /* admission budget for resident problems (0 = 80% of free) */
  int max_resident;         /* slot limit (0 = 1024) */
  int precision;            /* pm_precision for all requests */
  int use_graphs;           /* capture each it_eval block of sweeps in a CUDA graph */
  int autotune;             /* pick the launch shape (pm_server_launch_shape) per size
                               class of the resident set by timing */
  int max_bypass;           /* backfill: when the request at the head of the queue does
                               not fit the free budget, later requests that fit are
                               admitted past it, at most max_bypass times before the
                               head is admitted (0 = 64; negative = strict first come,
                               first served).  A request larger than the whole budget
                               completes at once with PM_ERR_NOMEM. */
  int relaunch_sweeps;      /* mixed form: 0 (default) runs a round's FP32 sweeps as one
                               persistent kernel walking a device tile queue; 1 launches
                               every sweep separately (same results bit for bit) */
} pm_server_config;

typedef struct pm_server pm_server;

typedef struct {
  uint64_t ticket;
  pm_status status;
  pm_result result;
  double submit_ms, admit_ms, finish_ms; /* server clock */
} pm_completion;

pm_status pm_server_create(const pm_server_config* cfg, pm_server** out);
pm_status pm_server_destroy(pm_server* s);
/* Queue one request (geometry copied).  Never blocks. */
pm_status pm_server_submit(pm_server* s, const pm_params* p, const uint8_t* geom,
                           uint64_t* ticket);
/* Advance the device by one scheduling round (admit, one it_eval block for every
 * resident request, retire converged ones).  *active = resident + queued after the round. */
pm_status pm_server_step(pm_server* s, int* active);
/* Move up to max finished requests into out; *n = number written. */
pm_status pm_server_poll(pm_server* s, pm_completion* out, int max, int* n);
pm_status pm_server_stats(pm_server* s, double* busy_ms, double* wall_ms, uint64_t* lups);
double pm_server_clock_ms(pm_server* s);
/* Withdraw a request: a queued one is removed, a resident one is retired at
 * once (between scheduling rounds; its device memory is freed and the others
 * continue).  Either way its completion carries PM_ERR_CANCELLED and no
 * result.  PM_ERR_NOT_FOUND when the ticket has already completed or was never
 * issued.  No counterpart in the reference (one run per process). */
pm_status pm_server_cancel(pm_server* s, uint64_t ticket);
/* Device bytes the server would admit this request by (its footprint with the
 * server's precision and kernels), to plan budgets.  No counterpart in the
 * reference. */
pm_status pm_server_request_bytes(pm_server* s, const pm_params* p, size_t* bytes);
/* Launch shape of the batched sweeps: shape[0] voxels per work item (the tile
 * of the device queue; cut smaller when the resident set is small), shape[1]
 * CTAs per SM and shape[2] threads per block of the mixed form's persistent
 * round, shape[3] threads per block of the other batched kernels.  With
 * cfg.autotune the server picks them per size class of the resident set; the
 * getter reports the current choice.  The setter pins a shape (autotuning
 * stops; 128 threads with 1-8 CTAs or 256 with 1-4, threads 128 / 256 / 512)
 * from the next round on; call it between rounds.  Every shape gives the same
 * results bit for bit.  No counterpart in the reference. */
pm_status pm_server_launch_shape(pm_server* s, int shape[4]);
pm_status pm_server_set_launch_shape(pm_server* s, const int shape[4]);

/* ---- test hook (no counterpart in the reference) ----
 * Makes the nth device allocation of problem set-up from now on (1 = the next
 * one) fail as an out-of-memory error would, so that callers can exercise
 * their PM_ERR_NOMEM handling on the host without exhausting a GPU; 0 clears
 * it.  Process-wide. */
pm_status pm_debug_fail_alloc(int nth);
/* Makes the waits of the server's persistent sweep kernel (mixed form) wait
 * for `extra` more finished items than exist, with at most `polls` polls
 * (0 = the kernel's own limit of a few seconds), so a test can see a wait run
 * out: the kernel sets its error flag and returns, pm_server_step reports
 * PM_ERR_CUDA, and the device stays usable.  Takes effect for rounds captured
 * after the call; 0, 0 restores normal operation.  Process-wide. */
pm_status pm_debug_round_wait(unsigned extra, int polls);
/* While on, every launch of the TMA z-march correction sweep (kernels 0 and 3)
 * and of the bulk-staged compact sweep (kernels 11 and 12) reports its first
 * pipeline wait as timed out without waiting: each CTA sets
 * the error flag, waits (bounded) for its copies in flight and returns, and
 * the sweep's caller gets PM_ERR_CUDA with the device still usable.  0 turns
 * it off.  Process-wide. */
pm_status pm_debug_tma_fail(int on);

#ifdef __cplusplus
}
#endif

#endif
