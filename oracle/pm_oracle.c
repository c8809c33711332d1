/*
 * CPU ORACLE for the POREMAPS pseudo-time Stokes sweep -- TEST INFRASTRUCTURE.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
 * this file, as the checker.  The poremaps_gb300 product never links it.
 *
 * Each function restates one reference routine (file:line in the reference
 * project krachdd/poremaps) in single-process C.  The "ranks" of the
 * reference become z-slabs of one process (the reference run with
 * dom_decomposition 1 1 P), which lets the CPU baseline use P host cores with
 * the reference's own per-rank semantics; nslabs = 1 is the single-rank run.
 *
 * Floating-point expressions keep the reference's operand order and are built
 * with -ffp-contract=off, so results are bitwise identical to the reference
 * binary (pinned by tests/test_oracle_golden.py).
 */
#define _POSIX_C_SOURCE 200809L
#include "pm_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* constants.h:46-64 */
#define OMEGA_SOR 1.2
#define RE 0.01
#define C2 1.5e6
#define DT 1.0e-4
#define LIM 2

typedef struct {
  int NX, NY, NZ; /* padded sizes of this slab */
  int lnz, z0;    /* interior z extent and global z start */
  unsigned char* g;
  int* nh;
  double *u, *v, *w, *p;
  double *u2, *v2, *w2, *p2;
  double* p3; /* swept (pre-reapply) pressure of the last interior plane */
  unsigned short* ck; /* neighbourhood cases of nh decoded once: cx | cy << 4 | cz << 8 */
  double* stage;      /* z-exchange send planes: 4 fields x (low 2 + high 2) planes */
} slab;

struct or_problem {
  int nx, ny, nz;
  int bc;
  unsigned solver;
  int ns;
  int periods[3];
  double dx, porosity_in, phi;
  int di[6];
  slab* s;
  int iteration;
  int nthreads;
};

static inline long IDX(const slab* S, int z, int y, int x) {
  return ((long)z * S->NY + y) * S->NX + x;
}

/* ---------------------------------------------------------------------- */
/* halo exchange: parallelization.cc:67-190 (geometry) and :193-318 (fields).
 * X then Y then Z, 2-deep faces over the full extent of the other axes.  In
 * x and y the only neighbour is the slab itself (periodic) or none; in z the
 * neighbours are the adjacent slabs (wrapping when periodic). */
#define DEF_EXCHANGE(NAME, T)                                                          \
  static void NAME(or_problem* pr, T** arr) {                                          \
    for (int c = 0; c < pr->ns; ++c) {                                                 \
      slab* S = &pr->s[c];                                                             \
      T* a = arr[c];                                                                   \
      int nx = S->NX, ny = S->NY, nz = S->NZ;                                          \
      if (pr->periods[0])                                                              \
        for (int i = 0; i < nz; i++)                                                   \
          for (int j = 0; j < ny; j++) {                                               \
            T s2 = a[IDX(S, i, j, 2)], s3 = a[IDX(S, i, j, 3)];                        \
            T r0 = a[IDX(S, i, j, nx - 4)], r1 = a[IDX(S, i, j, nx - 3)];              \
            a[IDX(S, i, j, nx - 2)] = s2; a[IDX(S, i, j, nx - 1)] = s3;                 \
            a[IDX(S, i, j, 0)] = r0; a[IDX(S, i, j, 1)] = r1;                           \
          }                                                                            \
      if (pr->periods[1])                                                              \
        for (int i = 0; i < nz; i++)                                                   \
          for (int k = 0; k < nx; k++) {                                               \
            T s2 = a[IDX(S, i, 2, k)], s3 = a[IDX(S, i, 3, k)];                        \
            T r0 = a[IDX(S, i, ny - 4, k)], r1 = a[IDX(S, i, ny - 3, k)];              \
            a[IDX(S, i, ny - 2, k)] = s2; a[IDX(S, i, ny - 1, k)] = s3;                 \
            a[IDX(S, i, 0, k)] = r0; a[IDX(S, i, 1, k)] = r1;                           \
          }                                                                            \
    }                                                                                  \
    /* z: pack every slab's send planes first (MPI_Sendrecv semantics) */              \
    int ns = pr->ns;                                                                   \
    T** lo = (T**)malloc(sizeof(T*) * ns);                                             \
    T** hi = (T**)malloc(sizeof(T*) * ns);                                             \
    for (int c = 0; c < ns; ++c) {                                                     \
      slab* S = &pr->s[c];                                                             \
      long plane = (long)S->NX * S->NY;                                                \
      lo[c] = (T*)malloc(sizeof(T) * 2 * plane);                                       \
      hi[c] = (T*)malloc(sizeof(T) * 2 * plane);                                       \
      memcpy(lo[c], arr[c] + 2 * plane, sizeof(T) * 2 * plane);                        \
      memcpy(hi[c], arr[c] + (long)(S->NZ - 4) * plane, sizeof(T) * 2 * plane);         \
    }                                                                                  \
    for (int c = 0; c < ns; ++c) {                                                     \
      slab* S = &pr->s[c];                                                             \
      long plane = (long)S->NX * S->NY;                                                \
      int up = c + 1, dn = c - 1;                                                      \
      if (up == ns) up = pr->periods[2] ? 0 : -1;                                       \
      if (dn < 0) dn = pr->periods[2] ? ns - 1 : -1;                                    \
      if (up >= 0) memcpy(arr[c] + (long)(S->NZ - 2) * plane, lo[up], sizeof(T) * 2 * plane); \
      if (dn >= 0) memcpy(arr[c], hi[dn], sizeof(T) * 2 * plane);                       \
    }                                                                                  \
    for (int c = 0; c < ns; ++c) { free(lo[c]); free(hi[c]); }                         \
    free(lo); free(hi);                                                                \
  }

DEF_EXCHANGE(exchange_u8, unsigned char)
DEF_EXCHANGE(exchange_f64, double)

static void exchange_field(or_problem* pr, int which) {
  double** arr = (double**)malloc(sizeof(double*) * pr->ns);
  for (int c = 0; c < pr->ns; ++c) {
    slab* S = &pr->s[c];
    arr[c] = which == 0 ? S->p : which == 1 ? S->u : which == 2 ? S->v : S->w;
  }
  exchange_f64(pr, arr);
  free(arr);
}

/* ---------------------------------------------------------------------- */
/* eval_geometry: geometry.cc:174-302 (Bentz et al. 2007 neighbourhood). */
static void eval_geometry(slab* S) {
  long n = (long)S->NX * S->NY * S->NZ;
  for (long c = 0; c < n; ++c) S->nh[c] = S->g[c] == 0 ? 0 : -1;
  const long st[3] = {1, S->NX, (long)S->NX * S->NY};
  const int shift[3] = {100, 10, 1};
  for (int d = 0; d < 3; ++d)
    for (int i = LIM; i < S->NZ - LIM; i++)
      for (int j = LIM; j < S->NY - LIM; j++)
        for (int k = LIM; k < S->NX - LIM; k++) {
          long c = IDX(S, i, j, k);
          if (S->g[c] != 0) continue;
          int l = S->g[c - st[d]] != 0, r = S->g[c + st[d]] != 0;
          int ll = -1, rr = -1;
          if (!l) ll = S->g[c - 2 * st[d]] != 0;
          if (!r) rr = S->g[c + 2 * st[d]] != 0;
          int cs = 0;
          if (l == 1 && r == 1) cs = 1;
          else if (l == 1 && r == 0 && rr == 1) cs = 2;
          else if (ll == 1 && l == 0 && r == 1) cs = 3;
          else if (l == 1 && r == 0 && rr == 0) cs = 4;
          else if (ll == 0 && l == 0 && r == 1) cs = 5;
          else if (l == 0 && r == 0) cs = 6;
          S->nh[c] += cs * shift[d];
        }
  /* split_number (solver.cc:94-109) of every fluid code, done here once
   * instead of per voxel and sweep (the same integer digits) */
  for (long c = 0; c < n; ++c) {
    int code = S->nh[c];
    if (code <= 0) { S->ck[c] = 0; continue; }
    int cz = code % 10; code /= 10;
    int cy = code % 10; code /= 10;
    int cx = code % 10;
    S->ck[c] = (unsigned short)(cx | (cy << 4) | (cz << 8));
  }
}

/* ---------------------------------------------------------------------- */
/* reapply_pressure_gradient: boundary_conditions.cc:46-79 */
static void reapply(or_problem* pr) {
  slab* S = &pr->s[0];
  for (int j = LIM; j < S->NY - LIM; j++)
    for (int k = LIM; k < S->NX - LIM; k++)
      if (S->g[IDX(S, 1, j, k)] == 0) S->p[IDX(S, 1, j, k)] = pr->nz + 2;
  S = &pr->s[pr->ns - 1];
  for (int j = LIM; j < S->NY - LIM; j++)
    for (int k = LIM; k < S->NX - LIM; k++) {
      if (S->g[IDX(S, S->NZ - 2, j, k)] == 0) S->p[IDX(S, S->NZ - 2, j, k)] = 2.0;
      if (S->g[IDX(S, S->NZ - 3, j, k)] == 0) S->p[IDX(S, S->NZ - 3, j, k)] = 3.0;
    }
}

/* ---------------------------------------------------------------------- */
/* get_2nd_derivation: solver.cc:57-91 (six wall-aware 1-D stencils). */
static inline double d2(int cs, double ll, double l, double m, double r, double rr) {
  switch (cs) {
    case 1: return -8.0 * m;
    case 2: return 8.0 / 3.0 * r - 16.0 / 3.0 * m;
    case 3: return 8.0 / 3.0 * l - 16.0 / 3.0 * m;
    case 4: return 2.0 * r - 5.0 * m - 1.0 / 5.0 * rr;
    case 5: return 2.0 * l - 1.0 / 5.0 * ll - 5.0 * m;
    case 6: return l - 2.0 * m + r;
  }
  return 0.0;
}

/* One fluid voxel of central_diff5 (solver.cc:136-220).  Reads the source
 * arrays s*, writes the destination d*.  In-place (reference order): s == d.
 * Ping-pong Jacobi: s = old state.  Red-black: see sweep_redblack. */
static inline void voxel(const slab* S, long c, unsigned solver, const double* su,
                         const double* sv, const double* sw, const double* sp, double* du,
                         double* dv, double* dw, double* dpr, const double* p3) {
  const long sx = 1, sy = S->NX, sz = (long)S->NX * S->NY;
  const unsigned char* g = S->g;
  double pxm = sp[c - sx], pym = sp[c - sy];
  if (p3) {
    /* Voxel on the last interior plane: in the reference's in-place order its
     * -x / -y neighbours on the same plane were already swept in this
     * iteration and hold their pre-reapply pressure (the reapply to 3 runs
     * after the sweep), so an out-of-place ordering reads the swept values. */
    long q = c % sz;
    int k = (int)(q % S->NX), j = (int)(q / S->NX);
    if (k - 1 >= LIM) pxm = p3[q - sx];
    if (j - 1 >= LIM) pym = p3[q - sy];
  }
  double dp_dz = g[c - sz] == 0 ? -sp[c - sz] + sp[c] : 0.;
  double dp_dy = g[c - sy] == 0 ? -pym + sp[c] : 0.;
  double dp_dx = g[c - sx] == 0 ? -pxm + sp[c] : 0.;
  const unsigned ck = S->ck[c];
  const int cx = ck & 15, cy = (ck >> 4) & 15, cz = ck >> 8;
  double uxx = (su[c - sx] - 2 * su[c] + su[c + sx]);
  double vyy = (sv[c - sy] - 2 * sv[c] + sv[c + sy]);
  double wzz = (sw[c - sz] - 2 * sw[c] + sw[c + sz]);
  double vxx = d2(cx, sv[c - 2 * sx], sv[c - sx], sv[c], sv[c + sx], sv[c + 2 * sx]);
  double wxx = d2(cx, sw[c - 2 * sx], sw[c - sx], sw[c], sw[c + sx], sw[c + 2 * sx]);
  double uyy = d2(cy, su[c - 2 * sy], su[c - sy], su[c], su[c + sy], su[c + 2 * sy]);
  double wyy = d2(cy, sw[c - 2 * sy], sw[c - sy], sw[c], sw[c + sy], sw[c + 2 * sy]);
  double uzz = d2(cz, su[c - 2 * sz], su[c - sz], su[c], su[c + sz], su[c + 2 * sz]);
  double vzz = d2(cz, sv[c - 2 * sz], sv[c - sz], sv[c], sv[c + sz], sv[c + 2 * sz]);
  double fu = uxx + uyy + uzz;
  double fv = vyy + vzz + vxx;
  double fw = wzz + wxx + wyy;
  double v_sum = 0.0;
  double un = su[c], vn = sv[c], wn = sw[c];
  if (solver == 1)
    v_sum = (sw[c + sz] - sw[c] + sv[c + sy] - sv[c] + su[c + sx] - su[c]);
  if (solver == 1 || solver == 2) {
    un = g[c - sx] != 0 ? 0.0 : su[c] + (-dp_dx + fu / RE) * DT;
    vn = g[c - sy] != 0 ? 0.0 : sv[c] + (-dp_dy + fv / RE) * DT;
    wn = g[c - sz] != 0 ? 0.0 : sw[c] + (-dp_dz + fw / RE) * DT;
  } else if (solver == 3) {
    un = (1.0 - OMEGA_SOR) * su[c] + OMEGA_SOR * (-dp_dx + fu / RE) * DT;
    vn = (1.0 - OMEGA_SOR) * sv[c] + OMEGA_SOR * (-dp_dy + fv / RE) * DT;
    wn = (1.0 - OMEGA_SOR) * sw[c] + OMEGA_SOR * (-dp_dz + fw / RE) * DT;
  }
  if (solver == 2 || solver == 3)
    v_sum = (sw[c + sz] - wn + sv[c + sy] - vn + su[c + sx] - un);
  du[c] = un;
  dv[c] = vn;
  dw[c] = wn;
  dpr[c] = sp[c] - C2 * v_sum * DT;
}

/* central_diff5 (solver.cc:112-224): in-place lexicographic sweep of one
 * slab (one rank of the reference run). */
static void sweep_reference(or_problem* pr, slab* S) {
  for (int i = LIM; i < S->NZ - LIM; i++)
    for (int j = LIM; j < S->NY - LIM; j++)
      for (int k = LIM; k < S->NX - LIM; k++) {
        long c = IDX(S, i, j, k);
        if (S->g[c] == 0)
          voxel(S, c, pr->solver, S->u, S->v, S->w, S->p, S->u, S->v, S->w, S->p, NULL);
      }
}

static void swap_state(slab* S) {
  double* t;
  t = S->u; S->u = S->u2; S->u2 = t;
  t = S->v; S->v = S->v2; S->v2 = t;
  t = S->w; S->w = S->w2; S->w2 = t;
  t = S->p; S->p = S->p2; S->p2 = t;
}

/* record the swept pressure of the last interior plane before the reapply */
static void save_p3(slab* S) {
  long plane = (long)S->NX * S->NY;
  memcpy(S->p3, S->p + (long)(S->NZ - 3) * plane, sizeof(double) * plane);
}

/* state2 := state on padded planes [z0, z1) */
static void copy_planes(slab* S, int z0, int z1) {
  if (z1 <= z0) return;
  long plane = (long)S->NX * S->NY, o = (long)z0 * plane;
  size_t n = sizeof(double) * plane * (z1 - z0);
  memcpy(S->u2 + o, S->u + o, n); memcpy(S->v2 + o, S->v + o, n);
  memcpy(S->w2 + o, S->w + o, n); memcpy(S->p2 + o, S->p + o, n);
}

/* Ping-pong Jacobi ordering of the same update on interior planes [i0, i1):
 * every neighbour is read from the previous iterate; solvers 2/3 use the
 * voxel's own new velocity in the divergence exactly as solver.cc:216-218
 * does. */
static void jacobi_planes(or_problem* pr, slab* S, int i0, int i1) {
  for (int i = i0; i < i1; i++)
    for (int j = LIM; j < S->NY - LIM; j++)
      for (int k = LIM; k < S->NX - LIM; k++) {
        long c = IDX(S, i, j, k);
        if (S->g[c] == 0)
          voxel(S, c, pr->solver, S->u, S->v, S->w, S->p, S->u2, S->v2, S->w2, S->p2,
                i == S->NZ - 3 ? S->p3 : NULL);
      }
}

/* Red-black ordering: colour = parity of the global interior coordinates.
 * Red voxels update from the previous iterate (state -> state2); black
 * voxels then update from state2, which holds the new red values and the old
 * black values (so the same-colour +-2 reads of the wall stencils see old
 * values and the result does not depend on the order inside a colour), into
 * state; finally the new red values are merged into state. */
static void colour_planes(or_problem* pr, slab* S, int colour, int i0, int i1) {
  for (int i = i0; i < i1; i++)
    for (int j = LIM; j < S->NY - LIM; j++)
      for (int k = LIM; k < S->NX - LIM; k++) {
        if ((((k - LIM) + (j - LIM) + (S->z0 + i - LIM)) & 1) != colour) continue;
        long c = IDX(S, i, j, k);
        if (S->g[c] != 0) continue;
        if (colour == 0) /* red: old state -> state2; black neighbours' swept p */
          voxel(S, c, pr->solver, S->u, S->v, S->w, S->p, S->u2, S->v2, S->w2, S->p2,
                i == S->NZ - 3 ? S->p3 : NULL);
        else /* black: state2 (new red, old black) -> state */
          voxel(S, c, pr->solver, S->u2, S->v2, S->w2, S->p2, S->u, S->v, S->w, S->p, NULL);
      }
}

static void merge_red_planes(slab* S, int i0, int i1) {
  for (int i = i0; i < i1; i++)
    for (int j = LIM; j < S->NY - LIM; j++)
      for (int k = LIM; k < S->NX - LIM; k++) {
        if (((k - LIM) + (j - LIM) + (S->z0 + i - LIM)) & 1) continue;
        long c = IDX(S, i, j, k);
        if (S->g[c] != 0) continue;
        S->u[c] = S->u2[c]; S->v[c] = S->v2[c]; S->w[c] = S->w2[c]; S->p[c] = S->p2[c];
      }
}

static double* field_of(slab* S, int f) {
  return f == 0 ? S->p : f == 1 ? S->u : f == 2 ? S->v : S->w;
}

/* communicate_halos (parallelization.cc:193-318), x and y part, on padded
 * planes [z0, z1) of one field: on one rank in x/y the neighbour is the
 * slab itself (periodic) or none.  x then y per plane, as the reference's
 * X-then-Y order leaves them (the y copies carry the x halos). */
static void exchange_xy_planes(or_problem* pr, slab* S, double* a, int z0, int z1) {
  int nx = S->NX, ny = S->NY;
  for (int i = z0; i < z1; i++) {
    if (pr->periods[0])
      for (int j = 0; j < ny; j++) {
        double s2 = a[IDX(S, i, j, 2)], s3 = a[IDX(S, i, j, 3)];
        double r0 = a[IDX(S, i, j, nx - 4)], r1 = a[IDX(S, i, j, nx - 3)];
        a[IDX(S, i, j, nx - 2)] = s2; a[IDX(S, i, j, nx - 1)] = s3;
        a[IDX(S, i, j, 0)] = r0; a[IDX(S, i, j, 1)] = r1;
      }
    if (pr->periods[1])
      for (int k = 0; k < nx; k++) {
        double s2 = a[IDX(S, i, 2, k)], s3 = a[IDX(S, i, 3, k)];
        double r0 = a[IDX(S, i, ny - 4, k)], r1 = a[IDX(S, i, ny - 3, k)];
        a[IDX(S, i, ny - 2, k)] = s2; a[IDX(S, i, ny - 1, k)] = s3;
        a[IDX(S, i, 0, k)] = r0; a[IDX(S, i, 1, k)] = r1;
      }
  }
}

/* z part: every slab first packs its send planes (2, 3 down; NZ-4, NZ-3 up)
 * for all four fields (MPI_Sendrecv semantics), then receives the adjacent
 * slabs' planes into its halos (wrapping when z is periodic). */
static void exchange_z_pack(slab* S) {
  long plane = (long)S->NX * S->NY;
  for (int f = 0; f < 4; ++f) {
    double* a = field_of(S, f);
    memcpy(S->stage + (long)(4 * f) * plane, a + 2 * plane, sizeof(double) * 2 * plane);
    memcpy(S->stage + (long)(4 * f + 2) * plane, a + (long)(S->NZ - 4) * plane,
           sizeof(double) * 2 * plane);
  }
}

static void exchange_z_unpack(or_problem* pr, int c) {
  slab* S = &pr->s[c];
  long plane = (long)S->NX * S->NY;
  int ns = pr->ns, up = c + 1, dn = c - 1;
  if (up == ns) up = pr->periods[2] ? 0 : -1;
  if (dn < 0) dn = pr->periods[2] ? ns - 1 : -1;
  for (int f = 0; f < 4; ++f) {
    double* a = field_of(S, f);
    if (up >= 0)
      memcpy(a + (long)(S->NZ - 2) * plane, pr->s[up].stage + (long)(4 * f) * plane,
             sizeof(double) * 2 * plane);
    if (dn >= 0)
      memcpy(a, pr->s[dn].stage + (long)(4 * f + 2) * plane, sizeof(double) * 2 * plane);
  }
}

/* ---------------------------------------------------------------------- */
/* Iteration engine.  One calc_flow iteration (calc_flow.cc:101-118) is
 * [reapply before the first] -> sweep -> halo exchange of p, u, v, w ->
 * reapply.  nthreads workers run a block of iterations with a barrier after
 * every phase:
 *   - reference order: each worker sweeps whole slabs (a slab is a rank of
 *     the reference run, its in-place sweep is sequential);
 *   - Jacobi / red-black: each pass reads only the other buffer, so the
 *     workers split every slab's z planes;
 *   - exchange: x/y copies split by planes, z copies by slab.
 * Every phase completes before the next starts, so the values are bitwise
 * those of one worker. */
typedef struct {
  or_problem* pr;
  int order, n, tid, nt;
  pthread_barrier_t* bar;
} pool_job;

static void pool_wait(pool_job* jb) {
  if (jb->nt > 1) pthread_barrier_wait(jb->bar);
}

static inline void part(int lo, int hi, int t, int nt, int* a, int* b) {
  long n = hi - lo;
  *a = lo + (int)(n * t / nt);
  *b = lo + (int)(n * (t + 1) / nt);
}

static void* pool_worker(void* arg) {
  pool_job* jb = (pool_job*)arg;
  or_problem* pr = jb->pr;
  const int t = jb->tid, nt = jb->nt, ns = pr->ns;
  int a, b;
  for (int it = 0; it < jb->n; ++it) {
    if (pr->iteration == 0) {
      if (t == 0) reapply(pr);
      pool_wait(jb);
    }
    if (jb->order == OR_ORDER_REFERENCE) {
      for (int c = t; c < ns; c += nt) sweep_reference(pr, &pr->s[c]);
      pool_wait(jb);
    } else {
      for (int c = 0; c < ns; ++c) {
        part(0, pr->s[c].NZ, t, nt, &a, &b);
        copy_planes(&pr->s[c], a, b);
      }
      pool_wait(jb);
      if (jb->order == OR_ORDER_JACOBI) {
        for (int c = 0; c < ns; ++c) {
          slab* S = &pr->s[c];
          part(LIM, S->NZ - LIM, t, nt, &a, &b);
          jacobi_planes(pr, S, a, b);
        }
        pool_wait(jb);
        if (t == 0)
          for (int c = 0; c < ns; ++c) swap_state(&pr->s[c]);
      } else {
        for (int colour = 0; colour < 2; ++colour) {
          for (int c = 0; c < ns; ++c) {
            slab* S = &pr->s[c];
            part(LIM, S->NZ - LIM, t, nt, &a, &b);
            colour_planes(pr, S, colour, a, b);
          }
          pool_wait(jb);
        }
        for (int c = 0; c < ns; ++c) {
          slab* S = &pr->s[c];
          part(LIM, S->NZ - LIM, t, nt, &a, &b);
          merge_red_planes(S, a, b);
        }
      }
      pool_wait(jb);
      if (t == 0)
        for (int c = 0; c < ns; ++c) save_p3(&pr->s[c]);
      pool_wait(jb);
    }
    for (int c = 0; c < ns; ++c) {
      slab* S = &pr->s[c];
      part(0, S->NZ, t, nt, &a, &b);
      for (int f = 0; f < 4; ++f) exchange_xy_planes(pr, S, field_of(S, f), a, b);
    }
    pool_wait(jb);
    for (int c = t; c < ns; c += nt) exchange_z_pack(&pr->s[c]);
    pool_wait(jb);
    for (int c = t; c < ns; c += nt) exchange_z_unpack(pr, c);
    pool_wait(jb);
    if (t == 0) {
      reapply(pr);
      pr->iteration++;
    }
    pool_wait(jb);
  }
  return NULL;
}

/* n iterations on the worker pool (the calling thread is worker 0). */
static void run_iterations(or_problem* pr, int order, int n) {
  if (n <= 0) return;
  int nt = pr->nthreads;
  if (nt > 256) nt = 256;
  if (nt <= 1) {
    pool_job jb = {pr, order, n, 0, 1, NULL};
    pool_worker(&jb);
    return;
  }
  pthread_barrier_t bar;
  pthread_barrier_init(&bar, NULL, (unsigned)nt);
  pthread_t th[256];
  pool_job jobs[256];
  for (int t = 0; t < nt; ++t) jobs[t] = (pool_job){pr, order, n, t, nt, &bar};
  for (int t = 1; t < nt; ++t) pthread_create(&th[t], NULL, pool_worker, &jobs[t]);
  pool_worker(&jobs[0]);
  for (int t = 1; t < nt; ++t) pthread_join(th[t], NULL);
  pthread_barrier_destroy(&bar);
}

/* ---------------------------------------------------------------------- */
/* set-up: get_dom_limits (geometry.cc:129-171), read_geometry (:58-126),
 * eval_geometry, allocate_initial_field (initialize.cc:69-121) and the
 * periods of main_stokes_solver.cc:163-165. */
or_problem* or_create(const int size[3], int bc_method, unsigned solver, int nslabs,
                      const unsigned char* geom_raw, double voxel_size, double porosity,
                      const int dom_interest[6]) {
  if (nslabs < 1 || nslabs > size[2]) return NULL;
  or_problem* pr = (or_problem*)calloc(1, sizeof(or_problem));
  pr->nx = size[0]; pr->ny = size[1]; pr->nz = size[2];
  pr->bc = bc_method; pr->solver = solver; pr->ns = nslabs;
  pr->periods[0] = pr->periods[1] = (bc_method == 0);
  pr->periods[2] = (bc_method <= 2);
  pr->dx = voxel_size; pr->porosity_in = porosity;
  for (int i = 0; i < 6; ++i) pr->di[i] = dom_interest ? dom_interest[i] : 0;
  pr->nthreads = 1;
  pr->s = (slab*)calloc(nslabs, sizeof(slab));
  int base = size[2] / nslabs, add = size[2] - nslabs * base;
  for (int c = 0; c < nslabs; ++c) {
    slab* S = &pr->s[c];
    int cum = c == 0 ? 0 : (c <= add ? c : add);
    S->z0 = c * base + cum;
    S->lnz = base + (c < add ? 1 : 0);
    S->NX = size[0] + 4; S->NY = size[1] + 4; S->NZ = S->lnz + 4;
    long n = (long)S->NX * S->NY * S->NZ;
    S->g = (unsigned char*)calloc(n, 1);
    S->nh = (int*)calloc(n, sizeof(int));
    S->u = (double*)calloc(n, 8); S->v = (double*)calloc(n, 8);
    S->w = (double*)calloc(n, 8); S->p = (double*)calloc(n, 8);
    S->u2 = (double*)calloc(n, 8); S->v2 = (double*)calloc(n, 8);
    S->w2 = (double*)calloc(n, 8); S->p2 = (double*)calloc(n, 8);
    S->p3 = (double*)calloc((long)S->NX * S->NY, 8);
    S->ck = (unsigned short*)calloc(n, sizeof(unsigned short));
    S->stage = (double*)calloc((long)16 * S->NX * S->NY, 8);
    for (int i = 0; i < S->lnz; ++i)
      for (int j = 0; j < size[1]; ++j)
        for (int k = 0; k < size[0]; ++k)
          S->g[IDX(S, i + 2, j + 2, k + 2)] =
              geom_raw[((long)(S->z0 + i) * size[1] + j) * size[0] + k] != 0;
  }
  unsigned char** ga = (unsigned char**)malloc(sizeof(void*) * nslabs);
  for (int c = 0; c < nslabs; ++c) ga[c] = pr->s[c].g;
  exchange_u8(pr, ga);
  free(ga);
  for (int c = 0; c < nslabs; ++c) {
    slab* S = &pr->s[c];
    eval_geometry(S);
    long n = (long)S->NX * S->NY * S->NZ;
    for (long q = 0; q < n; ++q) S->p[q] = -1.0;
    for (int i = LIM; i < S->NZ - LIM; i++)
      for (int j = LIM; j < S->NY - LIM; j++)
        for (int k = LIM; k < S->NX - LIM; k++) {
          long q = IDX(S, i, j, k);
          S->p[q] = S->g[q] == 0 ? (double)((size[2] - S->z0 - i) + LIM + 2) : 0.0;
        }
  }
  exchange_field(pr, 0);
  for (int c = 0; c < nslabs; ++c) save_p3(&pr->s[c]);
  /* set_halos_initial (initialize.cc:240-289) zeroes velocity halos that
   * are already zero. */
  pr->phi = porosity == -1.0 ? or_porosity(pr) : porosity;
  pr->iteration = 0;
  return pr;
}

void or_destroy(or_problem* pr) {
  if (!pr) return;
  for (int c = 0; c < pr->ns; ++c) {
    slab* S = &pr->s[c];
    free(S->g); free(S->nh);
    free(S->u); free(S->v); free(S->w); free(S->p);
    free(S->u2); free(S->v2); free(S->w2); free(S->p2);
    free(S->p3); free(S->ck); free(S->stage);
  }
  free(pr->s);
  free(pr);
}

int or_threads(or_problem* pr, int nthreads) {
  pr->nthreads = nthreads < 1 ? 1 : nthreads;
  return pr->nthreads;
}

/* get_porosity: geometry.cc:335-364 */
double or_porosity(or_problem* pr) {
  double fl = 0.0, vc = 0.0;
  for (int c = 0; c < pr->ns; ++c) {
    slab* S = &pr->s[c];
    double f = 0.0;
    double v = (S->NX - 2 * LIM) * (S->NY - 2 * LIM) * (S->NZ - 2 * LIM);
    for (int i = LIM; i < S->NZ - LIM; i++)
      for (int j = LIM; j < S->NY - LIM; j++)
        for (int k = LIM; k < S->NX - LIM; k++)
          if (S->g[IDX(S, i, j, k)] == 0) f += 1.0;
    fl = c == 0 ? f : fl + f;
    vc = c == 0 ? v : vc + v;
  }
  return fl / vc;
}

/* compute_convergence: evaluation.cc:216-262 */
double or_convergence(or_problem* pr, double* permeability) {
  double sum = 0.0, cnt = 0.0;
  for (int c = 0; c < pr->ns; ++c) {
    slab* S = &pr->s[c];
    double vs = 0.0;
    int fl = 0;
    for (int i = LIM; i < S->NZ - LIM; i++)
      for (int j = LIM; j < S->NY - LIM; j++)
        for (int k = LIM; k < S->NX - LIM; k++) {
          long q = IDX(S, i, j, k);
          if (S->g[q] == 0) { fl += 1; vs += S->w[q]; }
        }
    if (fl == 0) vs = 0.0;
    if (c == 0) { sum = vs; cnt = (double)fl; }
    else { sum = sum + vs; cnt = cnt + (double)fl; }
  }
  int flcount = (int)cnt;
  double mean = sum / flcount;
  double cur = mean / RE;
  double conv = fabs(cur - *permeability) / cur;
  *permeability = cur;
  return conv;
}

/* compute_permeability: evaluation.cc:54-211 */
void or_permeability(or_problem* pr, or_result* res) {
  double W[3] = {0, 0, 0}, wmax = 0.0;
  int wfl = 0;
  double D[5] = {0, 0, 0, 0, 0};
  int I[3] = {0, 0, 0};
  const int* di = pr->di;
  int dofi = !(di[0] == 0 && di[1] == 0 && di[2] == 0 && di[3] == 0 && di[4] == 0 && di[5] == 0);
  for (int c = 0; c < pr->ns; ++c) {
    slab* S = &pr->s[c];
    double wx = 0, wy = 0, wz = 0, wm = 0.0, vx = 0, vy = 0, vz = 0, p0 = 0, pe = 0;
    int wf = 0, fl = 0, p0f = 0, pef = 0;
    for (int i = LIM; i < S->NZ - LIM; i++)
      for (int j = LIM; j < S->NY - LIM; j++)
        for (int k = LIM; k < S->NX - LIM; k++) {
          long q = IDX(S, i, j, k);
          if (S->g[q] == 0) {
            wf += 1; wx += S->u[q]; wy += S->v[q]; wz += S->w[q];
            if (S->w[q] > wm) wm = S->w[q];
          }
        }
    if (dofi)
      for (int i = LIM; i < S->NZ - LIM; i++)
        for (int j = LIM; j < S->NY - LIM; j++)
          for (int k = LIM; k < S->NX - LIM; k++) {
            int gi = S->z0 + i - LIM, gj = j - LIM, gk = k - LIM;
            if (gk < di[0] || gk > di[1] || gj < di[2] || gj > di[3] || gi < di[4] || gi > di[5])
              continue;
            long q = IDX(S, i, j, k);
            if (S->g[q] == 0) { fl += 1; vx += S->u[q]; vy += S->v[q]; vz += S->w[q]; }
            if (gi == di[4] && S->g[q] == 0) { p0f += 1; p0 += S->p[q]; }
            if (gi == di[5] && S->g[q] == 0) { pef += 1; pe += S->p[q]; }
          }
    if (wf == 0) { wx = wy = wz = 0.0; wm = 0.0; }
    if (fl == 0) { vx = vy = vz = 0.0; }
    if (p0f == 0) p0 = 0.0;
    if (pef == 0) pe = 0.0;
    double d5[5] = {vx, vy, vz, p0, pe};
    int i3[3] = {fl, p0f, pef};
    for (int t = 0; t < 5; ++t) D[t] = c == 0 ? d5[t] : D[t] + d5[t];
    for (int t = 0; t < 3; ++t) I[t] = c == 0 ? i3[t] : I[t] + i3[t];
    double w3[3] = {wx, wy, wz};
    for (int t = 0; t < 3; ++t) W[t] = c == 0 ? w3[t] : W[t] + w3[t];
    wfl = c == 0 ? wf : wfl + wf;
    wmax = c == 0 ? wm : (wm > wmax ? wm : wmax);
  }
  double phi = pr->phi, dx = pr->dx;
  if (dofi) {
    double pgrad = ((D[4] / I[2]) - (D[3] / I[1])) / (di[5] - di[4]);
    res->k13 = (D[0] / I[0]) * (1.0 / RE) * phi * (1.0 / pgrad) * (dx * dx);
    res->k23 = (D[1] / I[0]) * (1.0 / RE) * phi * (1.0 / pgrad) * (dx * dx);
    res->k33 = (D[2] / I[0]) * (1.0 / RE) * phi * (1.0 / pgrad) * (dx * dx);
  } else {
    res->k13 = res->k23 = res->k33 = 0.0;
  }
  res->wk13 = (W[0] / wfl) * (1.0 / RE) * phi * (dx * dx);
  res->wk23 = (W[1] / wfl) * (1.0 / RE) * phi * (dx * dx);
  res->wk33 = (W[2] / wfl) * (1.0 / RE) * phi * (dx * dx);
  res->wmean_velz = W[2] / wfl * dx;
  res->wmax_velz = wmax * dx;
  res->porosity = phi;
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

void or_iterate(or_problem* pr, int order, int n) { run_iterations(pr, order, n); }

/* The next iteration index >= it at which calc_flow evaluates convergence
 * (it % it_eval == 0 && it > 1000, calc_flow.cc:120). */
static int next_eval(int it, int it_eval) {
  if (it_eval <= 0) return 2147483647;
  int e = it <= 1001 ? 1001 : it;
  int r = e % it_eval;
  if (r) {
    long q = (long)e + (it_eval - r);
    e = q > 2147483647 ? 2147483647 : (int)q;
  }
  return e;
}

/* calc_flow: calc_flow.cc:53-169, including the log rows of output.cc:193-230.
 * Iterations between two convergence evaluations run as one block on the
 * worker pool; the stop rule is only consulted at the evaluations, as in the
 * reference loop, so the trajectory and the stop iteration are the same.
 * The log's TPS column is the block's mean rate (it is wall-clock time). */
void or_calc_flow(or_problem* pr, int order, int max_iter, int it_eval, int it_write, double eps,
                  const char* log_path, or_result* res) {
  double conv = 1.0 + eps, perm = 0.0;
  int first = 1;
  memset(res, 0, sizeof(*res));
  while (pr->iteration < max_iter && conv >= eps) {
    int it = pr->iteration;
    int e = next_eval(it, it_eval);
    int last = e < max_iter - 1 ? e : max_iter - 1;
    double t0 = now_s();
    run_iterations(pr, order, last - it + 1);
    if (last != e) break; /* max_iter reached before the next evaluation */
    conv = or_convergence(pr, &perm);
    if (e % it_write == 0) {
      or_permeability(pr, res);
      if (log_path) {
        double tps = (last - it + 1) / (now_s() - t0);
        FILE* f = fopen(log_path, "a");
        if (f) {
          if (first)
            fprintf(f, "# iteration, conv, TPS [1/s], wmax_velz [m/s], wmean_velz [m/s], k13 "
                       "[m^2], k23 [m^2], k33 [m^2], wk13 [m^2], wk23 [m^2], wk33 [m^2]\n");
          fprintf(f, "%i, %e, %e, %e, %e, %e, %e, %e, %e, %e, %e\n", e, conv, tps,
                  res->wmax_velz, res->wmean_velz, res->k13, res->k23, res->k33, res->wk13,
                  res->wk23, res->wk33);
          fclose(f);
        }
      }
      first = 0;
    }
    res->iterations = e;
  }
  /* the result reports the permeability of the final state (the log rows keep
   * the values of their own iterations) */
  int last = res->iterations;
  or_permeability(pr, res);
  res->iterations = last;
  res->sweeps = pr->iteration;
  res->conv = conv;
  res->permeability = perm;
  res->porosity = pr->phi;
}

void or_get_fields(const or_problem* pr, double* u, double* v, double* w, double* p) {
  for (int c = 0; c < pr->ns; ++c) {
    const slab* S = &pr->s[c];
    for (int i = 0; i < S->lnz; ++i)
      for (int j = 0; j < pr->ny; ++j)
        for (int k = 0; k < pr->nx; ++k) {
          long o = ((long)(S->z0 + i) * pr->ny + j) * pr->nx + k;
          long q = IDX(S, i + 2, j + 2, k + 2);
          if (u) u[o] = S->u[q];
          if (v) v[o] = S->v[q];
          if (w) w[o] = S->w[q];
          if (p) p[o] = S->p[q];
        }
  }
}

/* Test hooks: interior fields set directly (the evaluation routines on
 * prescribed velocities, as the reference's tests/test_evaluation.py does),
 * and the stencil helpers on their own (tests/test_solver.py). */
void or_set_fields(or_problem* pr, const double* u, const double* v, const double* w,
                   const double* p) {
  for (int c = 0; c < pr->ns; ++c) {
    slab* S = &pr->s[c];
    for (int i = 0; i < S->lnz; ++i)
      for (int j = 0; j < pr->ny; ++j)
        for (int k = 0; k < pr->nx; ++k) {
          long o = ((long)(S->z0 + i) * pr->ny + j) * pr->nx + k;
          long q = IDX(S, i + 2, j + 2, k + 2);
          if (u) S->u[q] = u[o];
          if (v) S->v[q] = v[o];
          if (w) S->w[q] = w[o];
          if (p) S->p[q] = p[o];
        }
  }
}

double or_second_derivative(int cs, double ll, double l, double m, double r, double rr) {
  return d2(cs, ll, l, m, r, rr);
}

void or_split_code(int code, int out[3]) {
  /* split_number (solver.cc:94-109): 100 cx + 10 cy + cz */
  out[2] = code % 10;
  code /= 10;
  out[1] = code % 10;
  code /= 10;
  out[0] = code % 10;
}

void or_get_nhood(const or_problem* pr, int* out) {
  for (int c = 0; c < pr->ns; ++c) {
    const slab* S = &pr->s[c];
    for (int i = 0; i < S->lnz; ++i)
      for (int j = 0; j < pr->ny; ++j)
        for (int k = 0; k < pr->nx; ++k)
          out[((long)(S->z0 + i) * pr->ny + j) * pr->nx + k] = S->nh[IDX(S, i + 2, j + 2, k + 2)];
  }
}

void or_get_padded(const or_problem* pr, int s, int dims_out[3], double* u, double* v, double* w,
                   double* p) {
  const slab* S = &pr->s[s];
  dims_out[0] = S->NX; dims_out[1] = S->NY; dims_out[2] = S->NZ;
  size_t n = sizeof(double) * S->NX * S->NY * S->NZ;
  if (u) memcpy(u, S->u, n);
  if (v) memcpy(v, S->v, n);
  if (w) memcpy(w, S->w, n);
  if (p) memcpy(p, S->p, n);
}
