// Internal declarations shared by the CUDA kernels and the host runtime of
// poremaps_gb300.  Not part of the public C ABI (include/poremaps.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pm {

// Physics constants of the reference (src/constants.h:46-64).
constexpr double kOmega = 1.2;
constexpr double kRe = 0.01;
constexpr double kC2 = 1.5e6;
constexpr double kDt = 1.0e-4;

// Padded device layout.  A field element (x, y, z) of the padded domain
// (x in [0, NX), NX = nx + 4, halo 2 on each side as in the reference) lives at
// f[(z * NY + y) * px + x], where f points XOFF elements past the 256-byte
// aligned allocation so that the first interior column x = 2 starts on a
// 128-byte boundary; px (row pitch) is a multiple of 128 bytes.
constexpr int kXoff64 = 14;
constexpr int kXoff32 = 30;
constexpr int kXoffC = 14;
// The mixed form stores its FP32 correction and residual interleaved, one
// float4 (u, v, w, p) per voxel: a stencil point is one 128-bit load.
constexpr int kXoff4 = 6;

struct Grid {
  int nx, ny, nz;
  int NX, NY, NZ;
  int per[3];          // periodic axes (x, y, z) from boundary_method
  int px64, px32, pxc, px4; // row pitches in elements
  long long pl64, pl32, plc, pl4; // plane strides in elements
  long long alloc64, alloc32, allocc, alloc4; // elements to allocate (including XOFF)
  long long nvox;      // nx*ny*nz
  // n / nx and n / ny for 0 <= n < 2^31 as (n * m) >> (32 + s) (round-up magic)
  unsigned long long mnx, mny;
  int snx, sny;
};

Grid make_grid(int nx, int ny, int nz, int boundary_method);

template <typename T>
struct Fields {
  T* u;
  T* v;
  T* w;
  T* p;
};

// Voxel code byte: 0 solid; 1..216 interior fluid with neighbourhood cases
// (cx, cy, cz) in 1..6 as 1 + (cx-1)*36 + (cy-1)*6 + (cz-1); 255 fluid halo.
constexpr uint8_t kHaloFluid = 255;

// Reduction partials: fixed grid so the summation order never changes.
constexpr int kRedBlocks = 592;  // 4 x 148; fixed independent of the device
constexpr int kRedThreads = 256;
constexpr int kRedVals = 9;      // sum u, v, w, max w, box u, v, w, p(zmin), p(zmax)

struct Counts {
  long long fluid;       // interior fluid voxels
  long long box_fluid;   // fluid voxels inside dom_interest
  long long p0_fluid;    // fluid voxels on the dom_interest zmin plane
  long long pend_fluid;  // fluid voxels on the dom_interest zmax plane
};

// Kernel launch counter (all launch wrappers add the kernels they start).
void count_launches(int n);
// Multiprocessors of the current device (queried once; problem creation
// calls it first, so no launcher queries the device inside a graph capture).
int sm_count();
unsigned long long launches_total();

// ---------------------------------------------------------------- launchers
// All launchers are asynchronous on `st` and return the launch error.
cudaError_t launch_codes(const uint8_t* raw, uint8_t* codes, const Grid& g, cudaStream_t st);
// The geometry of an axis-rotated tensor solve from the unrotated one (sizes
// nx, ny, nz of the source): axis 0 -> sizes (ny, nz, nx), axis 1 -> (nz, nx, ny).
cudaError_t launch_rotate_geom(const uint8_t* src, uint8_t* dst, int axis, int nx, int ny, int nz,
                               cudaStream_t st);
// Fluid list in brick order (bx x by x bz bricks; bx <= 0: whole rows,
// by/bz <= 0: 1, i.e. lexicographic order); parity 0 / 1 keeps only the
// voxels with (x + y + z) of that parity, < 0 all of them.
cudaError_t launch_fluid_list(const uint8_t* codes, const Grid& g, int* list, int* count,
                              cudaStream_t st, int bx = 0, int by = 0, int bz = 0,
                              int parity = -1);
cudaError_t launch_counts(const uint8_t* codes, const Grid& g, const int di[6],
                          unsigned long long* out4, cudaStream_t st);
cudaError_t launch_init64(Fields<double> f, const uint8_t* codes, const Grid& g,
                          cudaStream_t st);
cudaError_t launch_copy_fields64(Fields<double> dst, Fields<double> src, const Grid& g,
                                 cudaStream_t st);
cudaError_t launch_halo64(Fields<double> f, const Grid& g, cudaStream_t st);
cudaError_t launch_reapply64(double* p, const uint8_t* codes, const Grid& g, cudaStream_t st);

// Reference order: in-place lexicographic sweep as an exact hyperplane
// wavefront, then halo exchange and reapply, n_iter times (cooperative launch).
cudaError_t launch_wavefront(Fields<double> f, const uint8_t* codes, const Grid& g,
                             int solver, int n_iter, int threads, int* coop_blocks,
                             cudaStream_t st);

// Ping-pong Jacobi (phase 0) and red (1) / black (2) half-sweeps from A into B
// over the fluid list; periodic halo copies and the pressure reapply fused.
// persistent: one wave of 2 CTAs per SM walking the list (else one voxel per
// thread); both give identical fields.
cudaError_t launch_sweep64(Fields<double> A, Fields<double> B, const uint8_t* codes,
                           const int* list, int nlist, const Grid& g, int solver, int exact,
                           int phase, cudaStream_t st, int persistent = 1);

// Mixed precision (defect correction).  x: FP64 state, e: FP32 correction
// (ping-pong), r: FP32 residual; e and r interleaved (float4 u, v, w, p).
// x += e over the fluid list and the halo copies its sweeps write (the only
// places where e is non-zero).
cudaError_t launch_dc_correct_list(Fields<double> x, const float4* e, const int* list, int nlist,
                                   const Grid& g, cudaStream_t st);
cudaError_t launch_dc_residual(Fields<double> x, float4* r, float4* e, const uint8_t* codes,
                               const int* list, int nlist, const Grid& g, int solver,
                               cudaStream_t st);
cudaError_t launch_dc_inner(const float4* e, float4* e2, const float4* r, const uint8_t* codes,
                            const int* list, int nlist, const Grid& g, int solver,
                            cudaStream_t st);
// Persistent fluid-list sweep (one wave of minb CTAs per SM, list entries
// prefetched one iteration ahead); minb 4, 3 or 2.
cudaError_t launch_dc_inner_pf(const float4* e, float4* e2, const float4* r,
                               const uint8_t* codes, const int* list, int nlist, const Grid& g,
                               int solver, int minb, cudaStream_t st);
cudaError_t launch_dc_inner_occ(const float4* e, float4* e2, const float4* r,
                                const uint8_t* codes, const int* list, int nlist, const Grid& g,
                                int solver, cudaStream_t st);
cudaError_t launch_zero4(float4* e, const Grid& g, cudaStream_t st);

// Reductions.  mode 0: FP64 fields; mode 1: FP64 x + FP32 e.  full = 0 only
// sums w.  partials: kRedBlocks*kRedVals doubles; out: kRedVals doubles.
// implied3: the state stores swept pressure on the last interior plane and the
// reapplied 3 is implied there (out-of-place orderings).
// The convergence check's sum (value 2: sum of w, + e.z in mode 1) over the
// fluid list; the other values of out are 0.  compact: e is the compact store
// (one float4 per list position) instead of the padded one.
cudaError_t launch_reduce_check(Fields<double> x, const float4* e, int mode, const int* list,
                                int nlist, const Grid& g, double* partials, double* out,
                                cudaStream_t st, int compact = 0);
// words (non-null): e is the compact store, located through these fluid-mask
// words (pm_compact.h).
cudaError_t launch_reduce(Fields<double> x, const float4* e, int mode, int full, int implied3,
                          const uint8_t* codes, const Grid& g, const int di[6],
                          double* partials, double* out, cudaStream_t st,
                          const uint2* words = nullptr);

// The same sums in the reference's serial lexicographic order (bitwise equal
// to the reference's reductions; used by the reference order).
cudaError_t launch_reduce_serial(Fields<double> x, int full, const uint8_t* codes, const Grid& g,
                                 const int di[6], double* out, cudaStream_t st);

cudaError_t launch_pack64(const double* f, const uint8_t* codes, int implied3, const Grid& g,
                          double* out, cudaStream_t st);
cudaError_t launch_unpack64(const double* in, const Grid& g, double* f, cudaStream_t st);
cudaError_t launch_pack_codes(const uint8_t* codes, const Grid& g, int* out, cudaStream_t st);


}  // namespace pm
