// Batched sweeps: one launch advances every resident sample by one sweep.
//
// The work is a table of items (sample, first fluid voxel, count) built from
// the samples' fluid lists; thread blocks walk the table with a grid stride,
// so samples of very different sizes share one launch and the device stays
// full while small samples finish and new ones arrive.  Each voxel runs the
// same device function as the single-problem kernels (pm_stencil.cuh), so a
// sample's fields are identical whether it is solved alone or in a batch.
// The mixed form's correction and residual are the compact store of
// pm_compact.cu (one float4 per fluid-list position), as the single-problem
// kernel 8 uses them.
#include "pm_batch.h"
#include "pm_compact.cuh"

namespace pm {

namespace {

__device__ __forceinline__ const SampleDesc& desc_of(const SampleDesc* d, int s) { return d[s]; }

// Every thread block walks work items with a grid stride.  The item's sample
// descriptor is staged in shared memory once per item (the voxel loop then
// reads it with broadcast loads instead of re-reading global memory per
// voxel), and each thread loads its next fluid-list entry before it computes
// the current voxel.
template <typename F>
__device__ __forceinline__ void walk_items(const SampleDesc* d, const WorkItem* items, int nitems,
                                           F f) {
  __shared__ __align__(16) SampleDesc sd;
  static_assert(sizeof(SampleDesc) % 4 == 0, "descriptor copied as words");
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const WorkItem w = items[it];
    __syncthreads();  // every reader of the previous item's descriptor is done
    const int* src = reinterpret_cast<const int*>(d + w.sample);
    for (int i = threadIdx.x; i < (int)(sizeof(SampleDesc) / 4); i += blockDim.x)
      reinterpret_cast<int*>(&sd)[i] = src[i];
    __syncthreads();
    const int* list = sd.list + w.start;
    int q = threadIdx.x;
    int lin = q < w.count ? __ldg(list + q) : 0;
    for (; q < w.count; q += blockDim.x) {
      const int qn = q + blockDim.x;
      const int next = qn < w.count ? __ldg(list + qn) : 0;
      f(sd, w.start + q, lin);
      lin = next;
    }
  }
}

// S: the solver every sample of the launch uses (1..3), or 0 when they differ
// (then each voxel dispatches on its sample's solver).
template <int S>
__global__ void k_batch_residual(const SampleDesc* d, const WorkItem* items, int nitems) {
  walk_items(d, items, nitems, [&](const SampleDesc& sd, int q, int lin) {
    float4* E = sd.ecur0 ? sd.E1 : sd.E0;
    const int sv = S ? S : sd.solver;
    if (sv == 3) residual_c_voxel<3>(sd.X0, sd.R, E, sd.codes, sd.g, q, lin);
    else if (sv == 2) residual_c_voxel<2>(sd.X0, sd.R, E, sd.codes, sd.g, q, lin);
    else residual_c_voxel<1>(sd.X0, sd.R, E, sd.codes, sd.g, q, lin);
  });
}

// At most 64 registers (1024 resident threads per SM at any block size the
// server tunes): measured faster here than three blocks of 256 threads at
// ~80 registers (54.2k against 50.8k solves/h on 32 uneven samples).
template <int S>
__global__ void __launch_bounds__(512, 2)
    k_batch_inner(const SampleDesc* d, const WorkItem* items, int nitems, int round) {
  walk_items(d, items, nitems, [&](const SampleDesc& sd, int q, int lin) {
    const int a = (sd.ecur0 + round - 1) & 1;
    const float4* Ein = a ? sd.E1 : sd.E0;
    float4* Eout = a ? sd.E0 : sd.E1;
    const int sv = S ? S : sd.solver;
    if (sv == 3) inner_c_voxel<3>(Ein, Eout, sd.R, sd.meta, sd.sa, sd.sb, q);
    else if (sv == 2) inner_c_voxel<2>(Ein, Eout, sd.R, sd.meta, sd.sa, sd.sb, q);
    else inner_c_voxel<1>(Ein, Eout, sd.R, sd.meta, sd.sa, sd.sb, q);
  });
}

__global__ void k_batch_correct(const SampleDesc* d, const WorkItem* items, int nitems,
                                int rounds) {
  walk_items(d, items, nitems, [&](const SampleDesc& sd, int q, int lin) {
    const int a = (sd.ecur0 + rounds - 1) & 1;
    correct_c_voxel(sd.X0, __ldg((a ? sd.E1 : sd.E0) + q), sd.g, lin);
  });
}

template <int S>
__global__ void k_batch_sweep64(const SampleDesc* d, const WorkItem* items, int nitems,
                                int round) {
  walk_items(d, items, nitems, [&](const SampleDesc& sd, int, int lin) {
    const int a = (sd.xcur0 + round) & 1;
    const Fields<double>& A = a ? sd.X1 : sd.X0;
    const Fields<double>& B = a ? sd.X0 : sd.X1;
    const int sv = S ? S : sd.solver;
    if (sv == 3) sweep64_voxel<3, 0, false>(A, B, sd.codes, sd.g, lin);
    else if (sv == 2) sweep64_voxel<2, 0, false>(A, B, sd.codes, sd.g, lin);
    else sweep64_voxel<1, 0, false>(A, B, sd.codes, sd.g, lin);
  });
}

// Per item: sum of w over its fluid voxels (fixed order: strided per thread,
// then a fixed tree), from the FP64 state selected by `round` parity.
__global__ void k_batch_sumw(const SampleDesc* d, const WorkItem* items, int nitems, int round,
                             double* out) {
  __shared__ double sh[1024];
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const WorkItem w = items[it];
    const SampleDesc& sd = desc_of(d, w.sample);
    const Fields<double>& X = ((sd.xcur0 + round) & 1) ? sd.X1 : sd.X0;
    double acc = 0.0;
    for (int q = threadIdx.x; q < w.count; q += blockDim.x) {
      int x, y, z;
      lin_to_xyz(sd.list[w.start + q], sd.g, x, y, z);
      acc += X.w[(long long)z * sd.g.pl64 + (long long)y * sd.g.px64 + x];
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if (threadIdx.x < (unsigned)o) sh[threadIdx.x] += sh[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[it] = sh[0];
    __syncthreads();
  }
}

// Acquire-load polls of a counter until it reaches target, bounded: about
// 2^24 polls of >= 128 ns each (seconds, against a sweep of one round that
// takes microseconds to a millisecond).
constexpr int kMaxPolls = 1 << 24;

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ bool wait_at_least(const unsigned* p, unsigned target, int polls) {
  for (int i = 0; i < polls; ++i) {
    if (ld_acquire(p) >= target) return true;
    __nanosleep(128);
  }
  return false;
}

// Persistent round of FP32 correction sweeps (see launch_batch_round).
// Progress: a ticket waits only on tickets of the previous sweep, which were
// handed out before it to CTAs that are running, so the smallest unfinished
// ticket never waits and no CTA needs another to be co-resident.  A sample's
// items are at most one sweep apart, so sweep k (reading buffer k - 1,
// writing the buffer sweep k - 2 wrote) never overwrites a value that a
// sweep-(k - 1) item still reads.  Corrections and residuals are read with
// L1-bypassing loads: other CTAs wrote them in this launch.
template <int S>
__global__ void __launch_bounds__(256, 4)
    k_batch_inner_round(const SampleDesc* d, const WorkItem* items, int nitems, int sweeps,
                        unsigned* sync, unsigned extra, int polls) {
  __shared__ __align__(16) SampleDesc sd;
  __shared__ unsigned sh_t;
  __shared__ int sh_ok;
  const unsigned total = (unsigned)sweeps * (unsigned)nitems;
  for (;;) {
    __syncthreads();  // the previous ticket's readers of sd are done
    if (threadIdx.x == 0) sh_t = atomicAdd(sync, 1u);
    __syncthreads();
    const unsigned t = sh_t;
    if (t >= total) break;
    const int k = (int)(t / (unsigned)nitems) + 1;  // sweep 1 .. sweeps
    const WorkItem w = items[t % (unsigned)nitems];
    const int* src = reinterpret_cast<const int*>(d + w.sample);
    for (int i = threadIdx.x; i < (int)(sizeof(SampleDesc) / 4); i += blockDim.x)
      reinterpret_cast<int*>(&sd)[i] = src[i];
    if (threadIdx.x == 0)
      sh_ok = wait_at_least(sync + 2 + w.sample,
                            (unsigned)(k - 1) * (unsigned)w.sample_items + extra, polls);
    __syncthreads();
    if (!sh_ok) {
      if (threadIdx.x == 0) atomicExch(sync + 1, 1u);
      break;
    }
    const int a = (sd.ecur0 + k - 1) & 1;
    const float4* Ein = a ? sd.E1 : sd.E0;
    float4* Eout = a ? sd.E0 : sd.E1;
    const int sv = S ? S : sd.solver;
    for (int q = threadIdx.x; q < w.count; q += blockDim.x) {
      const int i = w.start + q;
      if (sv == 3) inner_c_voxel<3, true>(Ein, Eout, sd.R, sd.meta, sd.sa, sd.sb, i);
      else if (sv == 2) inner_c_voxel<2, true>(Ein, Eout, sd.R, sd.meta, sd.sa, sd.sb, i);
      else inner_c_voxel<1, true>(Ein, Eout, sd.R, sd.meta, sd.sa, sd.sb, i);
    }
    __syncthreads();  // every store of the item is issued before the release
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(sync + 2 + w.sample, 1u);
    }
  }
}

template <int S>
void launch_solver_kind(int kind, int grid, int threads, const SampleDesc* d,
                        const WorkItem* items, int nitems, int round, cudaStream_t st) {
  if (kind == kBatchResidual) k_batch_residual<S><<<grid, threads, 0, st>>>(d, items, nitems);
  else if (kind == kBatchInner) k_batch_inner<S><<<grid, threads, 0, st>>>(d, items, nitems, round);
  else k_batch_sweep64<S><<<grid, threads, 0, st>>>(d, items, nitems, round);
}

}  // namespace

cudaError_t launch_batch_round(const SampleDesc* d, const WorkItem* items, int nitems,
                               int nsamples, int sweeps, unsigned* sync, cudaStream_t st,
                               int solver, unsigned extra, int polls, int ctas_per_sm,
                               int threads) {
  if (polls <= 0) polls = kMaxPolls;
  threads = threads == 128 ? 128 : 256;  // the kernel's 64 registers: 8 / 4 CTAs per SM
  const int max_ctas = threads == 128 ? 8 : 4;
  if (ctas_per_sm < 1) ctas_per_sm = 1;
  if (ctas_per_sm > max_ctas) ctas_per_sm = max_ctas;
  cudaError_t e = cudaMemsetAsync(sync, 0, sizeof(unsigned) * (2 + (size_t)nsamples), st);
  if (e != cudaSuccess) return e;
  if (nitems <= 0 || sweeps <= 0) return cudaSuccess;
  const long long tickets = (long long)sweeps * nitems;
  int grid = ctas_per_sm * sm_count();
  if (tickets < grid) grid = (int)tickets;
  if (solver == 1)
    k_batch_inner_round<1><<<grid, threads, 0, st>>>(d, items, nitems, sweeps, sync, extra, polls);
  else if (solver == 2)
    k_batch_inner_round<2><<<grid, threads, 0, st>>>(d, items, nitems, sweeps, sync, extra, polls);
  else if (solver == 3)
    k_batch_inner_round<3><<<grid, threads, 0, st>>>(d, items, nitems, sweeps, sync, extra, polls);
  else
    k_batch_inner_round<0><<<grid, threads, 0, st>>>(d, items, nitems, sweeps, sync, extra, polls);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_batch(int kind, const SampleDesc* d, const WorkItem* items, int nitems,
                         int round, int threads, int blocks, double* out, cudaStream_t st,
                         int solver) {
  if (nitems <= 0) return cudaSuccess;
  int grid = blocks > 0 ? (blocks < nitems ? blocks : nitems) : nitems;
  switch (kind) {
    case kBatchResidual:
    case kBatchInner:
    case kBatchSweep64:
      if (solver == 1) launch_solver_kind<1>(kind, grid, threads, d, items, nitems, round, st);
      else if (solver == 2) launch_solver_kind<2>(kind, grid, threads, d, items, nitems, round, st);
      else if (solver == 3) launch_solver_kind<3>(kind, grid, threads, d, items, nitems, round, st);
      else launch_solver_kind<0>(kind, grid, threads, d, items, nitems, round, st);
      break;
    case kBatchCorrect: k_batch_correct<<<grid, threads, 0, st>>>(d, items, nitems, round); break;
    case kBatchSumW: k_batch_sumw<<<grid, threads, 0, st>>>(d, items, nitems, round, out); break;
    default: return cudaErrorInvalidValue;
  }
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace pm
