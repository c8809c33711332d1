// Coefficient-form (FMA) sweeps: the FP64 fast sweeps and the kernels of the
// mixed-precision defect-correction form.
//
// Mixed precision.  One iteration of the solver is an affine map x -> F(x) of
// the padded state.  Writing the iterate as x + e with x a fixed FP64 state,
// e evolves by e -> L(e) + r, where L is the linear part of F (same stencil,
// homogeneous boundary values) and r = F(x) - x.  The correction e and the
// residual r are stored in FP32 (half the bytes of a sweep); every block of
// sweeps ends with the FP64 update x += e and a fresh FP64 residual, so FP32
// rounding only ever touches the (shrinking) correction and the iterate
// converges to the FP64 fixed point.
#include "pm_internal.h"
#include "pm_stencil.cuh"

namespace pm {

// ------------------------------------------------------------------ FP64 fast sweeps
template <int SOLVER, int PHASE>
__global__ void __launch_bounds__(256) k_sweep64_fast(Fields<double> A, Fields<double> B,
                                                      const uint8_t* codes, const int* list,
                                                      int nlist, Grid g) {
  __shared__ double ctab[16];
  fill_centre_table<SOLVER>(ctab);
  __syncthreads();
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nlist; q += gridDim.x * blockDim.x)
    sweep64_voxel<SOLVER, PHASE, false>(A, B, codes, g, list[q], ctab);
}

cudaError_t sweep64_exact(Fields<double> A, Fields<double> B, const uint8_t* codes,
                          const int* list, int nlist, const Grid& g, int solver, int phase,
                          cudaStream_t st);

// Persistent form: one wave of two CTAs per SM walks the list with a grid
// stride, each thread loading its next list entry before it computes the
// current voxel (the FP64 stencil needs ~110 registers: two CTAs fit).
template <int SOLVER, int PHASE>
__global__ void __launch_bounds__(256, 2) k_sweep64_pf(Fields<double> A, Fields<double> B,
                                                      const uint8_t* codes, const int* list,
                                                      int nlist, Grid g) {
  __shared__ double ctab[16];
  fill_centre_table<SOLVER>(ctab);
  __syncthreads();
  const int stride = gridDim.x * blockDim.x;
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  int lin = q < nlist ? __ldg(list + q) : 0;
  for (; q < nlist; q += stride) {
    const int qn = q + stride;
    const int next = qn < nlist ? __ldg(list + qn) : 0;
    sweep64_voxel<SOLVER, PHASE, false>(A, B, codes, g, lin, ctab);
    lin = next;
  }
}

template <int SOLVER>
static cudaError_t sweep_fast_s(Fields<double> A, Fields<double> B, const uint8_t* codes,
                                const int* list, int nlist, const Grid& g, int phase,
                                int persistent, cudaStream_t st) {
  int blocks = (nlist + 255) / 256;
  if (blocks < 1) return cudaSuccess;
  if (persistent) {
    const int sms = sm_count();
    if (blocks > 2 * sms) blocks = 2 * sms;
    if (phase == 0) k_sweep64_pf<SOLVER, 0><<<blocks, 256, 0, st>>>(A, B, codes, list, nlist, g);
    else if (phase == 1) k_sweep64_pf<SOLVER, 1><<<blocks, 256, 0, st>>>(A, B, codes, list, nlist, g);
    else k_sweep64_pf<SOLVER, 2><<<blocks, 256, 0, st>>>(A, B, codes, list, nlist, g);
  } else {
    if (phase == 0) k_sweep64_fast<SOLVER, 0><<<blocks, 256, 0, st>>>(A, B, codes, list, nlist, g);
    else if (phase == 1) k_sweep64_fast<SOLVER, 1><<<blocks, 256, 0, st>>>(A, B, codes, list, nlist, g);
    else k_sweep64_fast<SOLVER, 2><<<blocks, 256, 0, st>>>(A, B, codes, list, nlist, g);
  }
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_sweep64(Fields<double> A, Fields<double> B, const uint8_t* codes,
                           const int* list, int nlist, const Grid& g, int solver, int exact,
                           int phase, cudaStream_t st, int persistent) {
  if (exact) return sweep64_exact(A, B, codes, list, nlist, g, solver, phase, st);
  if (solver == 1) return sweep_fast_s<1>(A, B, codes, list, nlist, g, phase, persistent, st);
  if (solver == 2) return sweep_fast_s<2>(A, B, codes, list, nlist, g, phase, persistent, st);
  return sweep_fast_s<3>(A, B, codes, list, nlist, g, phase, persistent, st);
}

// ------------------------------------------------------------------ mixed precision
// x += e over the fluid list and the periodic halo copies its sweeps write:
// the only places where e is non-zero (residual and correction sweeps write a
// fluid voxel and its copies), so the state equals that of the dense form
// while solid regions are never touched.
__global__ void k_dc_correct_list(Fields<double> x, const float4* e, const int* list, int nlist,
                                  Grid g) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nlist; q += gridDim.x * blockDim.x)
    dc_correct_voxel(x, e, g, __ldg(list + q));
}

cudaError_t launch_dc_correct_list(Fields<double> x, const float4* e, const int* list, int nlist,
                                   const Grid& g, cudaStream_t st) {
  int blocks = (nlist + 255) / 256;
  if (blocks < 1) return cudaSuccess;
  k_dc_correct_list<<<blocks, 256, 0, st>>>(x, e, list, nlist, g);
  count_launches(1);
  return cudaGetLastError();
}


// r = F(x) - x in FP64 (stored FP32) and the first correction e1 = r.
template <int SOLVER>
__global__ void __launch_bounds__(256, 2) k_dc_residual(Fields<double> X, float4* R, float4* E,
                                                      const uint8_t* codes, const int* list,
                                                      int nlist, Grid g) {
  // persistent, next list entry prefetched (as the FP64 sweeps)
  __shared__ double ctab[16];
  fill_centre_table<SOLVER>(ctab);
  __syncthreads();
  const int stride = gridDim.x * blockDim.x;
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  int lin = q < nlist ? __ldg(list + q) : 0;
  for (; q < nlist; q += stride) {
    const int qn = q + stride;
    const int next = qn < nlist ? __ldg(list + qn) : 0;
    dc_residual_voxel<SOLVER>(X, R, E, codes, g, lin, ctab);
    lin = next;
  }
}

cudaError_t launch_dc_residual(Fields<double> x, float4* r, float4* e, const uint8_t* codes,
                               const int* list, int nlist, const Grid& g, int solver,
                               cudaStream_t st) {
  const int sms = sm_count();
  int blocks = (nlist + 255) / 256;
  if (blocks < 1) return cudaSuccess;
  if (blocks > 2 * sms) blocks = 2 * sms;
  if (solver == 1) k_dc_residual<1><<<blocks, 256, 0, st>>>(x, r, e, codes, list, nlist, g);
  else if (solver == 2) k_dc_residual<2><<<blocks, 256, 0, st>>>(x, r, e, codes, list, nlist, g);
  else k_dc_residual<3><<<blocks, 256, 0, st>>>(x, r, e, codes, list, nlist, g);
  count_launches(1);
  return cudaGetLastError();
}

// e2 = L(e) + r over the fluid list (FP32, interleaved fields).
template <int SOLVER>
__global__ void __launch_bounds__(256) k_dc_inner(const float4* E, float4* E2, const float4* R,
                                                  const uint8_t* codes, const int* list,
                                                  int nlist, Grid g) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nlist; q += gridDim.x * blockDim.x)
    dc_inner_voxel<SOLVER>(E, E2, R, codes, g, list[q]);
}

// The same sweep compiled for four resident blocks per SM (at most 64
// registers per thread): more warps in flight to hide the gather latency.
template <int SOLVER>
__global__ void __launch_bounds__(256, 4) k_dc_inner_occ(const float4* E, float4* E2,
                                                         const float4* R, const uint8_t* codes,
                                                         const int* list, int nlist, Grid g) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nlist; q += gridDim.x * blockDim.x)
    dc_inner_voxel<SOLVER>(E, E2, R, codes, g, list[q]);
}

// Persistent form of the fluid-list sweep: one wave of CTAs (MINB per SM)
// walks the list with a grid stride, and every thread loads its next list
// entry before it computes the current voxel, so the list read's latency
// overlaps the stencil instead of preceding it.  MINB 3 leaves each thread
// ~80 registers: all 13 float4 gathers of a voxel stay in flight at once
// (at 64 registers the compiler splits them and spills), which is worth more
// than the extra warps of MINB 4.
template <int SOLVER, int MINB>
__global__ void __launch_bounds__(256, MINB) k_dc_inner_pf(const float4* E, float4* E2,
                                                          const float4* R, const uint8_t* codes,
                                                          const int* list, int nlist, Grid g) {
  const int stride = gridDim.x * blockDim.x;
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  int lin = q < nlist ? __ldg(list + q) : 0;
  for (; q < nlist; q += stride) {
    const int qn = q + stride;
    const int next = qn < nlist ? __ldg(list + qn) : 0;
    dc_inner_voxel<SOLVER>(E, E2, R, codes, g, lin);
    lin = next;
  }
}

template <int MINB>
static cudaError_t launch_pf(const float4* e, float4* e2, const float4* r, const uint8_t* codes,
                             const int* list, int nlist, const Grid& g, int solver,
                             cudaStream_t st) {
  const int sms = sm_count();
  int blocks = (nlist + 255) / 256;
  if (blocks < 1) return cudaSuccess;
  if (blocks > MINB * sms) blocks = MINB * sms;
  if (solver == 1) k_dc_inner_pf<1, MINB><<<blocks, 256, 0, st>>>(e, e2, r, codes, list, nlist, g);
  else if (solver == 2) k_dc_inner_pf<2, MINB><<<blocks, 256, 0, st>>>(e, e2, r, codes, list, nlist, g);
  else k_dc_inner_pf<3, MINB><<<blocks, 256, 0, st>>>(e, e2, r, codes, list, nlist, g);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_dc_inner_pf(const float4* e, float4* e2, const float4* r,
                               const uint8_t* codes, const int* list, int nlist, const Grid& g,
                               int solver, int minb, cudaStream_t st) {
  if (minb <= 2) return launch_pf<2>(e, e2, r, codes, list, nlist, g, solver, st);
  if (minb == 3) return launch_pf<3>(e, e2, r, codes, list, nlist, g, solver, st);
  return launch_pf<4>(e, e2, r, codes, list, nlist, g, solver, st);
}

cudaError_t launch_dc_inner_occ(const float4* e, float4* e2, const float4* r,
                                const uint8_t* codes, const int* list, int nlist, const Grid& g,
                                int solver, cudaStream_t st) {
  int blocks = (nlist + 255) / 256;
  if (blocks < 1) return cudaSuccess;
  if (solver == 1) k_dc_inner_occ<1><<<blocks, 256, 0, st>>>(e, e2, r, codes, list, nlist, g);
  else if (solver == 2) k_dc_inner_occ<2><<<blocks, 256, 0, st>>>(e, e2, r, codes, list, nlist, g);
  else k_dc_inner_occ<3><<<blocks, 256, 0, st>>>(e, e2, r, codes, list, nlist, g);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_dc_inner(const float4* e, float4* e2, const float4* r, const uint8_t* codes,
                            const int* list, int nlist, const Grid& g, int solver,
                            cudaStream_t st) {
  int blocks = (nlist + 255) / 256;
  if (blocks < 1) return cudaSuccess;
  if (solver == 1) k_dc_inner<1><<<blocks, 256, 0, st>>>(e, e2, r, codes, list, nlist, g);
  else if (solver == 2) k_dc_inner<2><<<blocks, 256, 0, st>>>(e, e2, r, codes, list, nlist, g);
  else k_dc_inner<3><<<blocks, 256, 0, st>>>(e, e2, r, codes, list, nlist, g);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_zero4(float4* e, const Grid& g, cudaStream_t st) {
  return cudaMemsetAsync(e, 0, sizeof(float4) * (size_t)g.pl4 * g.NZ, st);
}

}  // namespace pm
