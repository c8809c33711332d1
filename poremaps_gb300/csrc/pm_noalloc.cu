// Allocation-free variant of the permeability / convergence sums.
//
// Some callers cannot let a library allocate device memory: a serving process
// whose HBM is carved up ahead of time by its own admission control, or a host
// framework that owns every device allocation (and for which a cudaMalloc or
// cudaFree in the middle of its stream work would also synchronise the
// device).  pm_reduce_fields_noalloc gives them the sums behind
// compute_permeability / compute_convergence over buffers they already own,
// with the only scratch memory in a fixed-size array of this file.
//
// Scratch: g_noalloc_rows, one row of partial sums per (y, z) row of the
// domain, at most kNoallocMaxRows rows (ny * nz <= 16384, 1.18 MB).  Every GPU
// that loads the library holds the array until the process exits.  All calls
// share it and it keeps the last call's contents; each call overwrites every
// row it later reads, so nothing in it has to start at zero.  Calls that
// overlap on the GPU (different streams, or different host threads) race on
// the array.  The first call on a device looks up the array's device address
// with that device current (cudaGetSymbolAddress); make that first call before
// any stream capture.
#include <mutex>

#include "../../include/poremaps.h"
#include "pm_api_internal.h"
#include "pm_internal.h"

namespace pm {
namespace {

constexpr int kNoallocMaxRows = 16384;
constexpr int kNoallocMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_rows[kNoallocMaxRows * kRedVals];

std::mutex g_noalloc_mu;
double* g_noalloc_ptr[kNoallocMaxDevices] = {nullptr};

// One block per (y, z) row, x summed in a fixed order (per-thread strided
// sums, then a fixed shuffle tree): bitwise reproducible.
__global__ void k_noalloc_rows(const uint8_t* geom, const double* u, const double* v,
                               const double* w, const double* p, int nx, int ny, int d0, int d1,
                               int d2, int d3, int d4, int d5, double* rows) {
  const int row = blockIdx.x;
  const int y = row % ny, z = row / ny;
  const bool dofi = d0 | d1 | d2 | d3 | d4 | d5;
  const bool row_in_box = dofi && y >= d2 && y <= d3 && z >= d4 && z <= d5;
  double acc[kRedVals];
  for (int i = 0; i < kRedVals; ++i) acc[i] = 0.0;
  const long long base = (long long)row * nx;
  for (int x = threadIdx.x; x < nx; x += blockDim.x) {
    long long q = base + x;
    if (geom[q] != 0) continue;
    double uu = u[q], vv = v[q], ww = w[q];
    acc[0] += uu;
    acc[1] += vv;
    acc[2] += ww;
    if (ww > acc[3]) acc[3] = ww;
    if (row_in_box && x >= d0 && x <= d1) {
      acc[4] += uu;
      acc[5] += vv;
      acc[6] += ww;
      if (z == d4) acc[7] += p[q];
      if (z == d5) acc[8] += p[q];
    }
  }
  __shared__ double sh[kRedVals][32];
  for (int i = 0; i < kRedVals; ++i) {
    double a = acc[i];
    for (int o = 16; o > 0; o >>= 1) {
      double b = __shfl_down_sync(0xffffffffu, a, o);
      a = (i == 3) ? (b > a ? b : a) : a + b;
    }
    if ((threadIdx.x & 31) == 0) sh[i][threadIdx.x >> 5] = a;
  }
  __syncthreads();
  if (threadIdx.x < kRedVals) {
    const int i = threadIdx.x;
    double a = sh[i][0];
    for (int wi = 1; wi < (int)(blockDim.x >> 5); ++wi)
      a = (i == 3) ? (sh[i][wi] > a ? sh[i][wi] : a) : a + sh[i][wi];
    rows[(long long)row * kRedVals + i] = a;
  }
}

__global__ void k_noalloc_final(const double* rows, int nrows, double* out) {
  __shared__ double sh[1024];
  for (int i = 0; i < kRedVals; ++i) {
    double a = 0.0;
    for (int r = threadIdx.x; r < nrows; r += blockDim.x) {
      double b = rows[(long long)r * kRedVals + i];
      a = (i == 3) ? (b > a ? b : a) : a + b;
    }
    sh[threadIdx.x] = a;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if (threadIdx.x < (unsigned)o) {
        double x = sh[threadIdx.x], y = sh[threadIdx.x + o];
        sh[threadIdx.x] = (i == 3) ? (y > x ? y : x) : x + y;
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) out[i] = sh[0];
    __syncthreads();
  }
}

// Device address of the scratch array for the current device, looked up once.
pm_status scratch_for_current_device(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
  if (dev < 0 || dev >= kNoallocMaxDevices)
    return set_error(PM_ERR_INVALID, "device %d beyond the %d supported", dev, kNoallocMaxDevices);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    double* ptr = nullptr;
    e = cudaGetSymbolAddress((void**)&ptr, g_noalloc_rows);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(g_noalloc_rows)");
    g_noalloc_ptr[dev] = ptr;
  }
  *out = g_noalloc_ptr[dev];
  return PM_OK;
}

}  // namespace
}  // namespace pm

using namespace pm;

extern "C" pm_status pm_reduce_fields_noalloc(const int size[3], const uint8_t* geom,
                                              const double* u, const double* v, const double* w,
                                              const double* p, const int dom_interest[6],
                                              double* sums, void* stream) {
  if (!size || !geom || !u || !v || !w || !p || !sums)
    return set_error(PM_ERR_INVALID, "pm_reduce_fields_noalloc: NULL argument");
  const int nx = size[0], ny = size[1], nz = size[2];
  if (nx < 1 || ny < 1 || nz < 1)
    return set_error(PM_ERR_INVALID, "pm_reduce_fields_noalloc: size must be positive");
  const long long nrows = (long long)ny * nz;
  if (nrows > kNoallocMaxRows)
    return set_error(PM_ERR_INVALID,
                     "pm_reduce_fields_noalloc: ny*nz = %lld rows exceeds the fixed scratch of "
                     "%d rows", nrows, kNoallocMaxRows);
  int di[6] = {0, 0, 0, 0, 0, 0};
  if (dom_interest)
    for (int i = 0; i < 6; ++i) di[i] = dom_interest[i];
  double* rows = nullptr;
  pm_status s = scratch_for_current_device(&rows);
  if (s != PM_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  k_noalloc_rows<<<(unsigned)nrows, 128, 0, st>>>(geom, u, v, w, p, nx, ny, di[0], di[1], di[2],
                                                  di[3], di[4], di[5], rows);
  k_noalloc_final<<<1, 1024, 0, st>>>(rows, (int)nrows, sums);
  count_launches(2);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "pm_reduce_fields_noalloc launch");
  return PM_OK;
}
