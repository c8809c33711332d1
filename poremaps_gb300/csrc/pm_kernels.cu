// Set-up, boundary, reduction and exact-arithmetic sweep kernels.
// This translation unit is compiled with -fmad=false so that every
// floating-point expression rounds exactly as the reference CPU program's
// (which is built for x86-64 without FMA contraction).
#include <cooperative_groups.h>

#include <algorithm>
#include <atomic>

#include "pm_internal.h"
#include "pm_stencil.cuh"

namespace cg = cooperative_groups;

namespace pm {

static std::atomic<unsigned long long> g_launches{0};
void count_launches(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }
unsigned long long launches_total() { return g_launches.load(std::memory_order_relaxed); }

int sm_count() {
  static std::atomic<int> sms{0};
  int v = sms.load(std::memory_order_relaxed);
  if (v > 0) return v;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
  if (v <= 0) v = 1;
  sms.store(v, std::memory_order_relaxed);
  return v;
}

Grid make_grid(int nx, int ny, int nz, int bm) {
  Grid g;
  g.nx = nx; g.ny = ny; g.nz = nz;
  g.NX = nx + 4; g.NY = ny + 4; g.NZ = nz + 4;
  // main_stokes_solver.cc:163-165: periods from boundary_method
  g.per[0] = g.per[1] = (bm == 0);
  g.per[2] = (bm <= 2);
  auto up = [](long long a, long long b) { return (a + b - 1) / b * b; };
  g.px64 = (int)up(kXoff64 + g.NX, 16);
  g.px32 = (int)up(kXoff32 + g.NX, 32);
  g.pxc = (int)up(kXoffC + g.NX, 16);
  g.px4 = (int)up(kXoff4 + g.NX, 8);
  g.pl4 = (long long)g.px4 * g.NY;
  g.alloc4 = g.pl4 * g.NZ + 16;
  g.pl64 = (long long)g.px64 * g.NY;
  g.pl32 = (long long)g.px32 * g.NY;
  g.plc = (long long)g.pxc * g.NY;
  g.alloc64 = g.pl64 * g.NZ + 64;
  g.alloc32 = g.pl32 * g.NZ + 64;
  g.allocc = g.plc * g.NZ + 256;
  g.nvox = (long long)nx * ny * nz;
  // s = ceil(log2 d), m = ceil(2^(32+s) / d): (n m) >> (32+s) == n / d for all
  // n < 2^31, since the rounding error n (m - 2^(32+s)/d) / 2^(32+s) < 1/(2d).
  auto magic = [](unsigned d, unsigned long long& m, int& s) {
    s = 0;
    while ((1ULL << s) < d) ++s;
    m = ((1ULL << (32 + s)) + d - 1) / d;
  };
  magic((unsigned)nx, g.mnx, g.snx);
  magic((unsigned)ny, g.mny, g.sny);
  return g;
}

// ------------------------------------------------------------------ geometry
// Fluid status of padded voxel (x, y, z): interior from the raw file, halo
// coordinates on periodic axes wrap (communicate_geom_halos with the rank as
// its own neighbour), on non-periodic axes the halo is fluid (geometry halos
// start at 0 and are never received, geometry.cc:98-106).
__device__ __forceinline__ bool raw_solid(const uint8_t* raw, const Grid& g, int x, int y, int z) {
  // An axis of length 1 has no image one period away for its outer halo
  // cells: the reference's self-exchange copies a halo cell that still holds
  // its initial fluid value there, so they are fluid too.
  auto fold = [](int c, int n, int per, bool& outside) {
    int i = c - 2;
    if (i < 0 || i >= n) {
      if (!per) { outside = true; return 0; }
      i = i < 0 ? i + n : i - n;
      if (i < 0 || i >= n) { outside = true; return 0; }
    }
    return i;
  };
  bool outside = false;
  int i = fold(x, g.nx, g.per[0], outside);
  int j = fold(y, g.ny, g.per[1], outside);
  int k = fold(z, g.nz, g.per[2], outside);
  if (outside) return false;
  return raw[((long long)k * g.ny + j) * g.nx + i] != 0;
}

// eval_geometry (geometry.cc:174-302) for every padded voxel.
__global__ void k_codes(const uint8_t* raw, uint8_t* codes, Grid g) {
  long long n = (long long)g.NX * g.NY * g.NZ;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    int x = (int)(q % g.NX);
    long long r = q / g.NX;
    int y = (int)(r % g.NY);
    int z = (int)(r / g.NY);
    uint8_t code;
    if (raw_solid(raw, g, x, y, z)) {
      code = 0;
    } else if (x < 2 || y < 2 || z < 2 || x >= g.NX - 2 || y >= g.NY - 2 || z >= g.NZ - 2) {
      code = kHaloFluid;
    } else {
      int cs[3];
      for (int d = 0; d < 3; ++d) {
        int dx = d == 0, dy = d == 1, dz = d == 2;
        bool l = raw_solid(raw, g, x - dx, y - dy, z - dz);
        bool r = raw_solid(raw, g, x + dx, y + dy, z + dz);
        int c;
        if (l && r) c = 1;
        else if (l && !r) c = raw_solid(raw, g, x + 2 * dx, y + 2 * dy, z + 2 * dz) ? 2 : 4;
        else if (!l && r) c = raw_solid(raw, g, x - 2 * dx, y - 2 * dy, z - 2 * dz) ? 3 : 5;
        else c = 6;
        cs[d] = c;
      }
      code = (uint8_t)(1 + (cs[0] - 1) * 36 + (cs[1] - 1) * 6 + (cs[2] - 1));
    }
    codes[((long long)z * g.NY + y) * g.pxc + x] = code;
  }
}

cudaError_t launch_codes(const uint8_t* raw, uint8_t* codes, const Grid& g, cudaStream_t st) {
  k_codes<<<1184, 256, 0, st>>>(raw, codes, g);
  count_launches(1);
  return cudaGetLastError();
}

// Geometry of an axis-rotated solve of the permeability tensor (the flow
// axis becomes z, as the reference's README.md:221-225 rotates the sample for
// the x and y runs): src is the x-fastest uint8 volume of sizes (nx, ny, nz);
// axis 0 writes the volume of sizes (ny, nz, nx) with (x', y', z') =
// (y, z, x), axis 1 the volume of sizes (nz, nx, ny) with (x', y', z') =
// (z, x, y).  Coalesced writes, gathered reads.
__global__ void k_rotate_geom(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst,
                              int axis, int nx, int ny, int nz) {
  const long long n = (long long)nx * ny * nz;
  for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < n;
       o += (long long)gridDim.x * blockDim.x) {
    long long x, y, z;
    if (axis == 0) {  // o = (x * nz + z) * ny + y
      y = o % ny;
      const long long r = o / ny;
      z = r % nz;
      x = r / nz;
    } else {  // o = (y * nx + x) * nz + z
      z = o % nz;
      const long long r = o / nz;
      x = r % nx;
      y = r / nx;
    }
    dst[o] = src[(z * ny + y) * nx + x];
  }
}

cudaError_t launch_rotate_geom(const uint8_t* src, uint8_t* dst, int axis, int nx, int ny, int nz,
                               cudaStream_t st) {
  k_rotate_geom<<<1184, 256, 0, st>>>(src, dst, axis, nx, ny, nz);
  count_launches(1);
  return cudaGetLastError();
}

// Interior fluid voxels as linear interior indices, in brick order: the
// domain is cut into bricks of BX x BY x BZ voxels (BX = nx, BY = BZ = 1 is
// plain lexicographic order), bricks are visited lexicographically and the
// voxels inside a brick in x-fastest order.  A thread block's run of the list
// then covers a compact brick, so the stencil neighbours of its voxels are
// mostly in L1.  The list is built from "segments": the x-run of one (y, z)
// row inside one brick, counted, scanned and filled in order (deterministic).
struct Bricks {
  int bx, by, bz;     // brick extents
  int nbx, nby, nbz;  // bricks per axis
};

__device__ __forceinline__ void segment(const Grid& g, const Bricks& b, int s, int& x0, int& len,
                                        int& y, int& z) {
  const int per_brick = b.by * b.bz;
  const int brick = s / per_brick, in = s - brick * per_brick;
  const int ix = brick % b.nbx, r = brick / b.nbx;
  const int iy = r % b.nby, iz = r / b.nby;
  const int ly = in % b.by, lz = in / b.by;
  x0 = ix * b.bx;
  len = min(b.bx, g.nx - x0);
  y = iy * b.by + ly;
  z = iz * b.bz + lz;
  if (y >= g.ny || z >= g.nz) len = 0;
}

// parity < 0: every fluid voxel; 0 / 1: only those with (x + y + z) of that
// parity (the red / black half of a red-black sweep).
__device__ __forceinline__ bool keep(const uint8_t* c, int x, int x0, int y, int z, int parity) {
  return c[x] != 0 && (parity < 0 || ((x0 + x + y + z) & 1) == parity);
}

__global__ void k_seg_counts(const uint8_t* codes, Grid g, Bricks b, int parity,
                             int* seg_count) {
  int x0, len, y, z;
  segment(g, b, blockIdx.x, x0, len, y, z);
  int cnt = 0;
  if (len > 0) {
    const uint8_t* c = codes + ((long long)(z + 2) * g.NY + (y + 2)) * g.pxc + 2 + x0;
    for (int x = threadIdx.x; x < len; x += blockDim.x) cnt += keep(c, x, x0, y, z, parity);
  }
  __shared__ int s[32];
  for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s[w];
    seg_count[blockIdx.x] = t;
  }
}

__global__ void k_seg_fill(const uint8_t* codes, Grid g, Bricks b, int parity,
                           const int* seg_off, int* list) {
  int x0, len, y, z;
  segment(g, b, blockIdx.x, x0, len, y, z);
  if (len <= 0) return;
  const uint8_t* c = codes + ((long long)(z + 2) * g.NY + (y + 2)) * g.pxc + 2 + x0;
  int base = seg_off[blockIdx.x];
  const int lane = threadIdx.x;  // one warp walks the segment in x order
  for (int xs = 0; xs < len; xs += 32) {
    const int x = xs + lane;
    const bool f = x < len && keep(c, x, x0, y, z, parity);
    const unsigned m = __ballot_sync(0xffffffffu, f);
    if (f)
      list[base + __popc(m & ((1u << lane) - 1))] =
          (int)(((long long)z * g.ny + y) * g.nx + x0 + x);
    base += __popc(m);
  }
}

__global__ void k_scan_rows(const int* row_count, int nrows, int* row_off, int* total) {
  // single block, sequential chunks (set-up only)
  __shared__ int carry;
  __shared__ int s[1024];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int b = 0; b < nrows; b += blockDim.x) {
    int i = b + threadIdx.x;
    int v = i < nrows ? row_count[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
      int t = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0;
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < nrows) row_off[i] = carry + s[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += s[threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

cudaError_t launch_fluid_list(const uint8_t* codes, const Grid& g, int* list, int* count,
                              cudaStream_t st, int bx, int by, int bz, int parity) {
  Bricks b;
  b.bx = bx > 0 ? std::min(bx, g.nx) : g.nx;
  b.by = by > 0 ? std::min(by, g.ny) : 1;
  b.bz = bz > 0 ? std::min(bz, g.nz) : 1;
  b.nbx = (g.nx + b.bx - 1) / b.bx;
  b.nby = (g.ny + b.by - 1) / b.by;
  b.nbz = (g.nz + b.bz - 1) / b.bz;
  const long long nseg = (long long)b.nbx * b.nby * b.nbz * b.by * b.bz;
  if (nseg > (1LL << 30)) return cudaErrorInvalidValue;
  int* tmp = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&tmp, sizeof(int) * 2 * (size_t)nseg, st);
  if (e != cudaSuccess) return e;
  k_seg_counts<<<(unsigned)nseg, 128, 0, st>>>(codes, g, b, parity, tmp);
  k_scan_rows<<<1, 1024, 0, st>>>(tmp, (int)nseg, tmp + nseg, count);
  k_seg_fill<<<(unsigned)nseg, 32, 0, st>>>(codes, g, b, parity, tmp + nseg, list);
  count_launches(3);
  e = cudaGetLastError();
  cudaFreeAsync(tmp, st);
  return e;
}

// Fluid counts for the reductions (integers, deterministic).
__global__ void k_counts(const uint8_t* codes, Grid g, int d0, int d1, int d2, int d3, int d4,
                         int d5, unsigned long long* out) {
  unsigned long long c[4] = {0, 0, 0, 0};
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < g.nvox;
       q += (long long)gridDim.x * blockDim.x) {
    int x = (int)(q % g.nx);
    long long r = q / g.nx;
    int y = (int)(r % g.ny);
    int z = (int)(r / g.ny);
    if (codes[((long long)(z + 2) * g.NY + (y + 2)) * g.pxc + (x + 2)] == 0) continue;
    c[0]++;
    if (x < d0 || x > d1 || y < d2 || y > d3 || z < d4 || z > d5) continue;
    c[1]++;
    if (z == d4) c[2]++;
    if (z == d5) c[3]++;
  }
  for (int i = 0; i < 4; ++i) {
    unsigned long long v = c[i];
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(out + i, v);
  }
}

cudaError_t launch_counts(const uint8_t* codes, const Grid& g, const int di[6],
                          unsigned long long* out4, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(out4, 0, 4 * sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  k_counts<<<592, 256, 0, st>>>(codes, g, di[0], di[1], di[2], di[3], di[4], di[5], out4);
  count_launches(1);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ fields
__device__ __forceinline__ bool is_halo(const Grid& g, int x, int y, int z) {
  return x < 2 || y < 2 || z < 2 || x >= g.NX - 2 || y >= g.NY - 2 || z >= g.NZ - 2;
}

// allocate_initial_field (initialize.cc:69-121) + the pressure halo exchange
// + set_halos_initial + the iteration-0 reapply_pressure_gradient
// (calc_flow.cc:105-108), evaluated point-wise.
__global__ void k_init64(Fields<double> f, const uint8_t* codes, Grid g) {
  long long n = (long long)g.NX * g.NY * g.NZ;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    int x = (int)(q % g.NX);
    long long r = q / g.NX;
    int y = (int)(r % g.NY);
    int z = (int)(r / g.NY);
    long long c = ((long long)z * g.NY + y) * g.px64 + x;
    f.u[c] = 0.0;
    f.v[c] = 0.0;
    f.w[c] = 0.0;
    // source voxel of the pressure value after the X, Y, Z halo exchange
    int sx = x, sy = y, sz = z;
    bool minus1 = false;
    auto fold = [&](int& s, int n, int per) {
      if (s < 2 || s >= n + 2) {
        if (!per) minus1 = true;
        else s = s < 2 ? s + n : s - n;
      }
    };
    fold(sx, g.nx, g.per[0]);
    fold(sy, g.ny, g.per[1]);
    fold(sz, g.nz, g.per[2]);
    double p;
    if (minus1) {
      p = -1.0;
    } else {
      bool fl = codes[((long long)sz * g.NY + sy) * g.pxc + sx] != 0;
      p = fl ? (double)((g.nz - sz) + 2 + 2) : 0.0;
    }
    // reapply_pressure_gradient (boundary_conditions.cc:46-79) on planes 1,
    // NZ-2 and NZ-3 for interior (x, y), where the geometry is fluid
    bool ixy = x >= 2 && x < g.NX - 2 && y >= 2 && y < g.NY - 2;
    bool fluid_here = codes[((long long)z * g.NY + y) * g.pxc + x] != 0;
    if (ixy && fluid_here) {
      if (z == 1) p = (double)(g.nz + 2);
      if (z == g.NZ - 2) p = 2.0;
      if (z == g.NZ - 3) p = 3.0;
    }
    f.p[c] = p;
  }
}

cudaError_t launch_init64(Fields<double> f, const uint8_t* codes, const Grid& g,
                          cudaStream_t st) {
  k_init64<<<1184, 256, 0, st>>>(f, codes, g);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_copy_fields64(Fields<double> dst, Fields<double> src, const Grid& g,
                                 cudaStream_t st) {
  size_t bytes = sizeof(double) * (size_t)g.pl64 * g.NZ;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(dst.u, src.u, bytes, cudaMemcpyDeviceToDevice, st))) return e;
  if ((e = cudaMemcpyAsync(dst.v, src.v, bytes, cudaMemcpyDeviceToDevice, st))) return e;
  if ((e = cudaMemcpyAsync(dst.w, src.w, bytes, cudaMemcpyDeviceToDevice, st))) return e;
  return cudaMemcpyAsync(dst.p, src.p, bytes, cudaMemcpyDeviceToDevice, st);
}

// communicate_halos (parallelization.cc:193-318) on one rank: periodic axes
// copy the 2-deep faces from the opposite interior side; non-periodic halos
// are left untouched.  Only face halos at interior positions of the other
// two axes are ever read by the sweep, so those are the ones refreshed.
template <typename T>
__device__ __forceinline__ void halo_point(Fields<T> f, const Grid& g, long long px, long long pl,
                                           long long q) {
  // q enumerates 3 axes x 4 halo layers x (interior extent of the other two)
  long long nyz = (long long)g.ny * g.nz, nxz = (long long)g.nx * g.nz,
            nxy = (long long)g.nx * g.ny;
  int ax;
  long long r;
  if (q < 4 * nyz) { ax = 0; r = q; }
  else if (q < 4 * (nyz + nxz)) { ax = 1; r = q - 4 * nyz; }
  else { ax = 2; r = q - 4 * (nyz + nxz); }
  if (!g.per[ax]) return;
  int layer = (int)(r & 3);
  r >>= 2;
  int x, y, z, sx, sy, sz;
  // layer 0,1 -> halo 0,1 from interior n, n+1; layer 2,3 -> halo n+2, n+3 from 2, 3
  if (ax == 0) {
    y = (int)(r % g.ny) + 2; z = (int)(r / g.ny) + 2;
    x = layer < 2 ? layer : g.nx + layer;
    sx = layer < 2 ? g.nx + layer : layer;
    sy = y; sz = z;
  } else if (ax == 1) {
    x = (int)(r % g.nx) + 2; z = (int)(r / g.nx) + 2;
    y = layer < 2 ? layer : g.ny + layer;
    sy = layer < 2 ? g.ny + layer : layer;
    sx = x; sz = z;
  } else {
    x = (int)(r % g.nx) + 2; y = (int)(r / g.nx) + 2;
    z = layer < 2 ? layer : g.nz + layer;
    sz = layer < 2 ? g.nz + layer : layer;
    sx = x; sy = y;
  }
  long long d = (long long)z * pl + (long long)y * px + x;
  long long s = (long long)sz * pl + (long long)sy * px + sx;
  f.u[d] = f.u[s];
  f.v[d] = f.v[s];
  f.w[d] = f.w[s];
  f.p[d] = f.p[s];
  (void)nxy;
}

__global__ void k_halo64(Fields<double> f, Grid g) {
  long long n = 4LL * ((long long)g.ny * g.nz + (long long)g.nx * g.nz + (long long)g.nx * g.ny);
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    halo_point<double>(f, g, g.px64, g.pl64, q);
}

cudaError_t launch_halo64(Fields<double> f, const Grid& g, cudaStream_t st) {
  k_halo64<<<592, 256, 0, st>>>(f, g);
  count_launches(1);
  return cudaGetLastError();
}

__device__ __forceinline__ void reapply_point(double* p, const uint8_t* codes, const Grid& g,
                                              long long q) {
  int x = (int)(q % g.nx) + 2, y = (int)(q / g.nx) + 2;
  long long c1 = ((long long)1 * g.NY + y), c2 = ((long long)(g.NZ - 2) * g.NY + y),
            c3 = ((long long)(g.NZ - 3) * g.NY + y);
  if (codes[c1 * g.pxc + x]) p[c1 * g.px64 + x] = (double)(g.nz + 2);
  if (codes[c2 * g.pxc + x]) p[c2 * g.px64 + x] = 2.0;
  if (codes[c3 * g.pxc + x]) p[c3 * g.px64 + x] = 3.0;
}

__global__ void k_reapply64(double* p, const uint8_t* codes, Grid g) {
  long long n = (long long)g.nx * g.ny;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    reapply_point(p, codes, g, q);
}

cudaError_t launch_reapply64(double* p, const uint8_t* codes, const Grid& g, cudaStream_t st) {
  k_reapply64<<<148, 256, 0, st>>>(p, codes, g);
  count_launches(1);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ reference order
template <int SOLVER>
__global__ void __launch_bounds__(256) k_wavefront(Fields<double> f, const uint8_t* codes, Grid g,
                                                   int n_iter) {
  cg::grid_group grid = cg::this_grid();
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long nth = (long long)gridDim.x * blockDim.x;
  const long long px = g.px64, pl = g.pl64;
  const int T = g.nx + g.ny + g.nz - 2;
  const long long nhalo =
      4LL * ((long long)g.ny * g.nz + (long long)g.nx * g.nz + (long long)g.nx * g.ny);
  for (int it = 0; it < n_iter; ++it) {
    // central_diff5's lexicographic in-place order is reproduced exactly by
    // hyperplanes t = x'+y'+z': every read at offsets -1/-2 lies on t-1/t-2
    // (already updated), every read at +1/+2 on t+1/t+2 (not yet updated).
    for (int t = 0; t < T; ++t) {
      int zlo = max(0, t - (g.nx - 1) - (g.ny - 1)), zhi = min(g.nz - 1, t);
      long long npairs = (long long)(zhi - zlo + 1) * g.ny;
      for (long long q = tid; q < npairs; q += nth) {
        int zp = zlo + (int)(q / g.ny), yp = (int)(q % g.ny);
        int xp = t - zp - yp;
        if (xp < 0 || xp >= g.nx) continue;
        int x = xp + 2, y = yp + 2, z = zp + 2;
        int code = codes[((long long)z * g.NY + y) * g.pxc + x];
        if (!code) continue;
        long long c = (long long)z * pl + (long long)y * px + x;
        Stencil<double> s;
        gather<double, 0, false, 0>(s, f, f, c, x, y, z, g, px, pl);
        double un, vn, wn, pn;
        update_exact<SOLVER>(s, code, un, vn, wn, pn);
        f.u[c] = un;
        f.v[c] = vn;
        f.w[c] = wn;
        f.p[c] = pn;
      }
      grid.sync();
    }
    for (long long q = tid; q < nhalo; q += nth) halo_point<double>(f, g, px, pl, q);
    grid.sync();
    for (long long q = tid; q < (long long)g.nx * g.ny; q += nth) reapply_point(f.p, codes, g, q);
    grid.sync();
  }
}

// threads: block size (32..256).  The grid holds one thread per (y, z) pair
// of a hyperplane -- enough for any hyperplane -- as far as co-residency
// allows; smaller blocks spread the same threads over more SMs (more FP64
// throughput per hyperplane, a dearer grid barrier).
cudaError_t launch_wavefront(Fields<double> f, const uint8_t* codes, const Grid& g, int solver,
                             int n_iter, int threads, int* coop_blocks, cudaStream_t st) {
  void* fn = solver == 1 ? (void*)k_wavefront<1> : solver == 2 ? (void*)k_wavefront<2>
                                                               : (void*)k_wavefront<3>;
  if (threads < 32 || threads > 256) threads = 256;
  if (*coop_blocks <= 0) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, 0);
    if (e != cudaSuccess) return e;
    long long want = ((long long)g.ny * g.nz + threads - 1) / threads;
    long long maxb = (long long)sms * (per > 0 ? per : 1);
    *coop_blocks = (int)(want < maxb ? (want < 1 ? 1 : want) : maxb);
  }
  Fields<double> ff = f;
  const uint8_t* cc = codes;
  Grid gg = g;
  int n = n_iter;
  void* args[] = {&ff, &cc, &gg, &n};
  count_launches(1);
  return cudaLaunchCooperativeKernel(fn, dim3(*coop_blocks), dim3(threads), args, 0, st);
}

// ------------------------------------------------------------------ FP64 sweeps (exact)
template <int SOLVER, int PHASE>
__global__ void __launch_bounds__(256) k_sweep64_exact(Fields<double> A, Fields<double> B,
                                                       const uint8_t* codes, const int* list,
                                                       int nlist, Grid g) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nlist; q += gridDim.x * blockDim.x)
    sweep64_voxel<SOLVER, PHASE, true>(A, B, codes, g, list[q]);
}

template <int SOLVER>
static cudaError_t sweep_exact_s(Fields<double> A, Fields<double> B, const uint8_t* codes,
                                 const int* list, int nlist, const Grid& g, int phase,
                                 cudaStream_t st) {
  int blocks = (nlist + 255) / 256;
  if (blocks < 1) return cudaSuccess;
  if (phase == 0) k_sweep64_exact<SOLVER, 0><<<blocks, 256, 0, st>>>(A, B, codes, list, nlist, g);
  else if (phase == 1) k_sweep64_exact<SOLVER, 1><<<blocks, 256, 0, st>>>(A, B, codes, list, nlist, g);
  else k_sweep64_exact<SOLVER, 2><<<blocks, 256, 0, st>>>(A, B, codes, list, nlist, g);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t sweep64_exact(Fields<double> A, Fields<double> B, const uint8_t* codes,
                          const int* list, int nlist, const Grid& g, int solver, int phase,
                          cudaStream_t st) {
  if (solver == 1) return sweep_exact_s<1>(A, B, codes, list, nlist, g, phase, st);
  if (solver == 2) return sweep_exact_s<2>(A, B, codes, list, nlist, g, phase, st);
  return sweep_exact_s<3>(A, B, codes, list, nlist, g, phase, st);
}

// ------------------------------------------------------------------ reductions
// compute_convergence / compute_permeability sums (evaluation.cc:54-262) with
// a fixed grid and a fixed combination tree (bitwise reproducible).
template <int MODE>
__global__ void __launch_bounds__(kRedThreads) k_reduce(Fields<double> x, const float4* e,
                                                        const uint2* words, int full,
                                                        int implied3, const uint8_t* codes,
                                                        Grid g, int d0, int d1, int d2, int d3,
                                                        int d4, int d5, double* partials) {
  double acc[kRedVals];
  for (int i = 0; i < kRedVals; ++i) acc[i] = 0.0;
  const bool dofi = d0 | d1 | d2 | d3 | d4 | d5;
  const long long stride = (long long)kRedBlocks * kRedThreads;
  for (long long q = blockIdx.x * (long long)kRedThreads + threadIdx.x; q < g.nvox; q += stride) {
    int xp = (int)(q % g.nx);
    long long r = q / g.nx;
    int yp = (int)(r % g.ny), zp = (int)(r / g.ny);
    int X = xp + 2, Y = yp + 2, Z = zp + 2;
    if (!codes[((long long)Z * g.NY + Y) * g.pxc + X]) continue;
    long long c = (long long)Z * g.pl64 + (long long)Y * g.px64 + X;
    long long c4 = (long long)Z * g.pl4 + (long long)Y * g.px4 + X;
    float4 ev = make_float4(0.f, 0.f, 0.f, 0.f);
    if (MODE == 1) {
      if (words) {  // compact store: the voxel's position in the fluid list
        const int nw = (g.nx + 31) / 32;
        const uint2 wd = words[r * nw + (xp >> 5)];
        ev = e[(int)wd.y + __popc(wd.x & ((1u << (xp & 31)) - 1u))];
      } else {
        ev = e[c4];
      }
    }
    double w = x.w[c];
    if (MODE == 1) w += (double)ev.z;
    acc[2] += w;
    if (!full) continue;
    double u = x.u[c], v = x.v[c];
    if (MODE == 1) { u += (double)ev.x; v += (double)ev.y; }
    acc[0] += u;
    acc[1] += v;
    if (w > acc[3]) acc[3] = w;
    if (!dofi) continue;
    if (xp < d0 || xp > d1 || yp < d2 || yp > d3 || zp < d4 || zp > d5) continue;
    acc[4] += u;
    acc[5] += v;
    acc[6] += w;
    double p = x.p[c];
    if (MODE == 1) p += (double)ev.w;
    if (implied3 && zp == g.nz - 1) p = 3.0;
    if (zp == d4) acc[7] += p;
    if (zp == d5) acc[8] += p;
  }
  __shared__ double sh[kRedVals][kRedThreads];
  for (int i = 0; i < kRedVals; ++i) sh[i][threadIdx.x] = acc[i];
  __syncthreads();
  for (int o = kRedThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < (unsigned)o)
      for (int i = 0; i < kRedVals; ++i) {
        double a = sh[i][threadIdx.x], b = sh[i][threadIdx.x + o];
        sh[i][threadIdx.x] = (i == 3) ? (b > a ? b : a) : a + b;
      }
    __syncthreads();
  }
  if (threadIdx.x < kRedVals) partials[blockIdx.x * kRedVals + threadIdx.x] = sh[threadIdx.x][0];
}

// The convergence check's sum alone (sum of w over the fluid voxels, value 2
// of the partials; the others are 0) over the fluid list: fixed per-thread
// order, fixed shuffle tree per warp, fixed order over the block's warps.
template <int MODE>
__global__ void __launch_bounds__(kRedThreads) k_reduce_check(Fields<double> x, const float4* e,
                                                              int compact, const int* list,
                                                              int nlist, Grid g,
                                                              double* partials) {
  double acc = 0.0;
  for (int q = blockIdx.x * kRedThreads + threadIdx.x; q < nlist; q += kRedBlocks * kRedThreads) {
    int X, Y, Z;
    lin_to_xyz(__ldg(list + q), g, X, Y, Z);
    double w = x.w[(long long)Z * g.pl64 + (long long)Y * g.px64 + X];
    if (MODE == 1)
      w += (double)e[compact ? (long long)q : (long long)Z * g.pl4 + (long long)Y * g.px4 + X].z;
    acc += w;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double sw[kRedThreads / 32];
  if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < kRedVals) {
    double t = 0.0;
    if (threadIdx.x == 2)
      for (int w = 0; w < kRedThreads / 32; ++w) t += sw[w];
    partials[blockIdx.x * kRedVals + threadIdx.x] = t;
  }
}

// One warp per value: each lane folds the partials lane, lane + 32, ... in
// order, then a fixed shuffle tree combines the lanes (deterministic).
__global__ void __launch_bounds__(32 * kRedVals) k_reduce_final(const double* partials,
                                                                double* out) {
  const int i = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool is_max = i == 3;
  constexpr int kPer = (kRedBlocks + 31) / 32;
  double v[kPer];
#pragma unroll
  for (int k = 0; k < kPer; ++k) {  // every load in flight at once
    const int b = lane + 32 * k;
    v[k] = b < kRedBlocks ? partials[b * kRedVals + i] : 0.0;
  }
  // the partial maxima are >= 0 (each block's starts at 0), so 0 pads them
  double a = v[0];
#pragma unroll
  for (int k = 1; k < kPer; ++k) a = is_max ? (v[k] > a ? v[k] : a) : a + v[k];
  for (int o = 16; o > 0; o >>= 1) {
    const double y = __shfl_xor_sync(0xffffffffu, a, o);
    a = is_max ? (y > a ? y : a) : a + y;
  }
  if (lane == 0) out[i] = a;
}

cudaError_t launch_reduce_check(Fields<double> x, const float4* e, int mode, const int* list,
                                int nlist, const Grid& g, double* partials, double* out,
                                cudaStream_t st, int compact) {
  if (mode == 0)
    k_reduce_check<0><<<kRedBlocks, kRedThreads, 0, st>>>(x, e, compact, list, nlist, g,
                                                           partials);
  else
    k_reduce_check<1><<<kRedBlocks, kRedThreads, 0, st>>>(x, e, compact, list, nlist, g,
                                                           partials);
  k_reduce_final<<<1, 32 * kRedVals, 0, st>>>(partials, out);
  count_launches(2);
  return cudaGetLastError();
}

cudaError_t launch_reduce(Fields<double> x, const float4* e, int mode, int full, int implied3,
                          const uint8_t* codes, const Grid& g, const int di[6], double* partials,
                          double* out, cudaStream_t st, const uint2* words) {
  if (mode == 0)
    k_reduce<0><<<kRedBlocks, kRedThreads, 0, st>>>(x, e, words, full, implied3, codes, g, di[0],
                                                     di[1], di[2], di[3], di[4], di[5],
                                                     partials);
  else
    k_reduce<1><<<kRedBlocks, kRedThreads, 0, st>>>(x, e, words, full, implied3, codes, g, di[0],
                                                     di[1], di[2], di[3], di[4], di[5],
                                                     partials);
  k_reduce_final<<<1, 32 * kRedVals, 0, st>>>(partials, out);
  count_launches(2);
  return cudaGetLastError();
}


// Serial-order sums for the reference order: the reference accumulates voxel
// by voxel in lexicographic order (evaluation.cc:87-149, 231-241), so the
// bit-exact mode does the same.  One warp loads 32 consecutive x of a row,
// lane 0 adds them in x order (a dependent chain of adds, about 0.3 ms for a
// 48x48x64 domain, once per it_eval sweeps).
__global__ void k_reduce_serial(Fields<double> x, int full, const uint8_t* codes, Grid g, int d0,
                                int d1, int d2, int d3, int d4, int d5, double* out) {
  const int lane = threadIdx.x;
  const bool dofi = d0 | d1 | d2 | d3 | d4 | d5;
  double su = 0.0, sv = 0.0, sw = 0.0, mx = 0.0;
  double bu = 0.0, bv = 0.0, bw = 0.0, p0 = 0.0, pe = 0.0;
  for (int zp = 0; zp < g.nz; ++zp)
    for (int yp = 0; yp < g.ny; ++yp)
      for (int x0 = 0; x0 < g.nx; x0 += 32) {
        int xp = x0 + lane;
        bool fl = false;
        double u = 0.0, v = 0.0, w = 0.0, p = 0.0;
        if (xp < g.nx) {
          long long cc = (long long)(zp + 2) * g.plc + (long long)(yp + 2) * g.pxc + xp + 2;
          long long c = (long long)(zp + 2) * g.pl64 + (long long)(yp + 2) * g.px64 + xp + 2;
          fl = codes[cc] != 0;
          if (fl) {
            w = x.w[c];
            if (full) { u = x.u[c]; v = x.v[c]; p = x.p[c]; }
          }
        }
        unsigned m = __ballot_sync(0xffffffffu, fl);
        for (int k = 0; k < 32; ++k) {
          double wk = __shfl_sync(0xffffffffu, w, k);
          double uk = 0.0, vk = 0.0, pk = 0.0;
          if (full) {
            uk = __shfl_sync(0xffffffffu, u, k);
            vk = __shfl_sync(0xffffffffu, v, k);
            pk = __shfl_sync(0xffffffffu, p, k);
          }
          if (lane == 0 && ((m >> k) & 1u)) {
            sw += wk;
            if (full) {
              su += uk;
              sv += vk;
              if (wk > mx) mx = wk;
              int xk = x0 + k;
              if (dofi && !(xk < d0 || xk > d1 || yp < d2 || yp > d3 || zp < d4 || zp > d5)) {
                bu += uk;
                bv += vk;
                bw += wk;
                if (zp == d4) p0 += pk;
                if (zp == d5) pe += pk;
              }
            }
          }
        }
      }
  if (lane == 0) {
    out[0] = su; out[1] = sv; out[2] = sw; out[3] = mx;
    out[4] = bu; out[5] = bv; out[6] = bw; out[7] = p0; out[8] = pe;
  }
}

cudaError_t launch_reduce_serial(Fields<double> x, int full, const uint8_t* codes, const Grid& g,
                                 const int di[6], double* out, cudaStream_t st) {
  k_reduce_serial<<<1, 32, 0, st>>>(x, full, codes, g, di[0], di[1], di[2], di[3], di[4], di[5],
                                    out);
  count_launches(1);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ export
// Interior of a padded FP64 field into a dense x-fastest array (the layout of
// write_output_raw, output.cc:82-91), optionally plus an FP32 correction.
// With implied3, fluid voxels of the last interior plane export the
// reapplied pressure 3 (the out-of-place orderings store the swept value).
__global__ void k_pack64(const double* f, const uint8_t* codes, int implied3, Grid g,
                         double* out) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < g.nvox;
       q += (long long)gridDim.x * blockDim.x) {
    int x = (int)(q % g.nx);
    long long r = q / g.nx;
    int y = (int)(r % g.ny), z = (int)(r / g.ny);
    double v = f[(long long)(z + 2) * g.pl64 + (long long)(y + 2) * g.px64 + x + 2];
    if (implied3 && z == g.nz - 1 &&
        codes[(long long)(z + 2) * g.plc + (long long)(y + 2) * g.pxc + x + 2])
      v = 3.0;
    out[q] = v;
  }
}

cudaError_t launch_pack64(const double* f, const uint8_t* codes, int implied3, const Grid& g,
                          double* out, cudaStream_t st) {
  k_pack64<<<1184, 256, 0, st>>>(f, codes, implied3, g, out);
  count_launches(1);
  return cudaGetLastError();
}

// Inverse of k_pack64: interior values (x fastest) into the padded field.
__global__ void k_unpack64(const double* in, Grid g, double* f) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < g.nvox;
       q += (long long)gridDim.x * blockDim.x) {
    int x = (int)(q % g.nx);
    long long r = q / g.nx;
    int y = (int)(r % g.ny), z = (int)(r / g.ny);
    f[(long long)(z + 2) * g.pl64 + (long long)(y + 2) * g.px64 + x + 2] = in[q];
  }
}

cudaError_t launch_unpack64(const double* in, const Grid& g, double* f, cudaStream_t st) {
  k_unpack64<<<1184, 256, 0, st>>>(in, g, f);
  count_launches(1);
  return cudaGetLastError();
}

// Neighbourhood codes as the reference stores them: 100cx + 10cy + cz, -1 solid.
__global__ void k_pack_codes(const uint8_t* codes, Grid g, int* out) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < g.nvox;
       q += (long long)gridDim.x * blockDim.x) {
    int x = (int)(q % g.nx);
    long long r = q / g.nx;
    int y = (int)(r % g.ny), z = (int)(r / g.ny);
    int c = codes[(long long)(z + 2) * g.plc + (long long)(y + 2) * g.pxc + x + 2];
    int v = -1;
    if (c) {
      int cx, cy, cz;
      decode_cases(c, cx, cy, cz);
      v = 100 * cx + 10 * cy + cz;
    }
    out[q] = v;
  }
}

cudaError_t launch_pack_codes(const uint8_t* codes, const Grid& g, int* out, cudaStream_t st) {
  k_pack_codes<<<1184, 256, 0, st>>>(codes, g, out);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace pm
