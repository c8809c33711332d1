// Brick-tiled FP32 correction sweep of the mixed form, fed by TMA.
//
// A CTA owns one BX x BY x BZ brick of the interior.  One elected thread loads
// the brick's correction with the stencil's 2-voxel halo on every side (one
// 3-D TMA box of float4 u, v, w, p) and the brick's voxel codes (one box of
// bytes) into shared memory under a single mbarrier.  The CTA's threads then
// walk the brick's fluid voxels -- a contiguous range of the fluid list built
// in the same brick order -- read all 13 stencil points from shared memory,
// the residual from global memory, and write the new correction (and its
// periodic halo copies) to the other ping-pong buffer.  Only bricks that hold
// fluid are launched, so solid regions cost neither loads nor CTAs.
//
// The arithmetic per voxel is update_fast<float> of pm_stencil.cuh on the same
// operands as the global-memory kernels, so the fields are bitwise identical.
// The wait is bounded: on expiry the CTA records an error, waits (bounded) for
// its copy still in flight and returns.
#include <atomic>
#include <vector>

#include "pm_brick.h"
#include "pm_stencil.cuh"
#include "pm_tma.cuh"

namespace pm {

namespace {

template <int BX_, int BY_, int BZ_>
struct Shape {
  static constexpr int BX = BX_, BY = BY_, BZ = BZ_;
  static constexpr int HX = BX + 4, HY = BY + 4, HZ = BZ + 4;
  static constexpr unsigned EBYTES = HX * HY * HZ * 16;  // halo box of float4
  static constexpr unsigned CBYTES = BX * BY * BZ;       // interior codes
  static constexpr unsigned SMEM = EBYTES + CBYTES + 16;  // + mbarrier
  static_assert(EBYTES % 128 == 0, "the codes box must start 128-byte aligned");
  static_assert(CBYTES % 16 == 0, "the mbarrier must be 8-byte aligned");
  static_assert(4 * HX <= 256 && HY <= 256 && HZ <= 256, "TMA box extents");
};

using Shape0 = Shape<32, 8, 8>;
using Shape1 = Shape<32, 8, 4>;
using Shape2 = Shape<32, 4, 4>;

struct BrickMaps {
  CUtensorMap e;      // correction with halo (float4 viewed as 4 floats)
  CUtensorMap codes;  // voxel codes, interior box
};

constexpr int kThreads = 256;

template <class S, int SOLVER>
__global__ void __launch_bounds__(kThreads)
    k_brick_inner(const __grid_constant__ BrickMaps maps, const float4* __restrict__ R,
                  float4* E2, const int* __restrict__ list, const int4* __restrict__ work,
                  Grid g, long long budget, int* err) {
  extern __shared__ __align__(128) unsigned char smem[];
  const float4* se = reinterpret_cast<const float4*>(smem);
  const uint8_t* sc = smem + S::EBYTES;
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(smem + S::EBYTES + S::CBYTES);
  // work: interior origin of the brick (x0, y0, z0) and its first list entry;
  // the next entry's start ends the range
  const int4 w = work[blockIdx.x];
  const int end = work[blockIdx.x + 1].w;
  const bool leader = threadIdx.x == 0;
  if (leader) {
    tma::mbar_init(bar, 1);
    tma::fence_mbar_init();
  }
  __syncthreads();
  if (leader) {
    tma::mbar_expect(bar, S::EBYTES + S::CBYTES);
    // halo box from padded (x0, y0, z0) = interior (x0-2, y0-2, z0-2)
    tma::load3(const_cast<float4*>(se), &maps.e, 4 * (kXoff4 + w.x), w.y, w.z, bar);
    // interior box from padded (x0+2, y0+2, z0+2)
    tma::load3(const_cast<uint8_t*>(sc), &maps.codes, kXoffC + 2 + w.x, 2 + w.y, 2 + w.z, bar);
  }
  const bool ok = __syncthreads_and(tma::mbar_wait(bar, 0, budget));
  if (!ok) {
    if (leader) {
      atomicExch(err, 1);
      tma::mbar_wait(bar, 0, budget);  // the copy may still land in shared memory
    }
    return;
  }
  constexpr int PX = S::HX, PL = S::HX * S::HY;
  const long long px = g.px4, pl = g.pl4;
  for (int k = w.w + threadIdx.x; k < end; k += kThreads) {
    int x, y, z;  // padded coordinates
    lin_to_xyz(list[k], g, x, y, z);
    const int lx = x - w.x, ly = y - w.y, lz = z - w.z;  // in the halo box: 2 .. B+1
    const int c0 = lz * PL + ly * PX + lx;
    const int code = sc[((lz - 2) * S::BY + (ly - 2)) * S::BX + (lx - 2)];
    const float4 C = se[c0];
    const float4 XM = se[c0 - 1], XP = se[c0 + 1], XMM = se[c0 - 2], XPP = se[c0 + 2];
    const float4 YM = se[c0 - PX], YP = se[c0 + PX];
    const float4 YMM = se[c0 - 2 * PX], YPP = se[c0 + 2 * PX];
    const float4 ZM = se[c0 - PL], ZP = se[c0 + PL];
    const float4 ZMM = se[c0 - 2 * PL], ZPP = se[c0 + 2 * PL];
    Stencil<float> s;
    s.uc = C.x; s.uxm = XM.x; s.uxp = XP.x; s.uym = YM.x; s.uyp = YP.x;
    s.uymm = YMM.x; s.uypp = YPP.x; s.uzm = ZM.x; s.uzp = ZP.x; s.uzmm = ZMM.x; s.uzpp = ZPP.x;
    s.vc = C.y; s.vxm = XM.y; s.vxp = XP.y; s.vxmm = XMM.y; s.vxpp = XPP.y; s.vym = YM.y;
    s.vyp = YP.y; s.vzm = ZM.y; s.vzp = ZP.y; s.vzmm = ZMM.y; s.vzpp = ZPP.y;
    s.wc = C.z; s.wxm = XM.z; s.wxp = XP.z; s.wxmm = XMM.z; s.wxpp = XPP.z; s.wym = YM.z;
    s.wyp = YP.z; s.wymm = YMM.z; s.wypp = YPP.z; s.wzm = ZM.z; s.wzp = ZP.z;
    // the last interior plane's own pressure is the reapplied value: correction 0
    s.pc = (z == g.NZ - 3) ? 0.f : C.w;
    s.pxm = XM.w; s.pym = YM.w; s.pzm = ZM.w;
    float un, vn, wn, pn;
    update_fast<float, SOLVER>(s, code, un, vn, wn, pn);
    const long long c = (long long)z * pl + (long long)y * px + x;
    const float4 r = __ldg(R + c);
    write_voxel4(E2, c, x, y, z, g, un + r.x, vn + r.y, wn + r.z, pn + r.w);
  }
}

// start[b] = first list entry of brick b (entries of a brick are contiguous).
__global__ void k_brick_starts(const int* list, int n, Grid g, int bx, int by, int bz, int nbx,
                               int nby, int* start) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    auto brick = [&](int lin) {
      const int x = lin % g.nx, r = lin / g.nx;
      const int y = r % g.ny, z = r / g.ny;
      return ((z / bz) * nby + y / by) * nbx + x / bx;
    };
    const int b = brick(list[q]);
    if (q == 0 || brick(list[q - 1]) != b) start[b] = q;
  }
}

template <class S>
void set_smem_attr() {
  static std::atomic<bool> done{false};
  if (done.load()) return;
  cudaFuncSetAttribute(k_brick_inner<S, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)S::SMEM);
  cudaFuncSetAttribute(k_brick_inner<S, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)S::SMEM);
  cudaFuncSetAttribute(k_brick_inner<S, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)S::SMEM);
  done = true;
}

}  // namespace

struct BrickPlan {
  BrickMaps maps[2];  // source buffer E0 / E1
  int4* work = nullptr;
  int nwork = 0;      // bricks that hold fluid
  int shape = 0;
  int* err = nullptr;
};

int brick_shape_of(int bx, int by, int bz) {
  for (int s = 0; s < 3; ++s) {
    int a, b, c;
    brick_dims(s, &a, &b, &c);
    if (a == bx && b == by && c == bz) return s;
  }
  return -1;
}

void brick_dims(int shape, int* bx, int* by, int* bz) {
  static const int d[3][3] = {{Shape0::BX, Shape0::BY, Shape0::BZ},
                              {Shape1::BX, Shape1::BY, Shape1::BZ},
                              {Shape2::BX, Shape2::BY, Shape2::BZ}};
  *bx = d[shape][0];
  *by = d[shape][1];
  *bz = d[shape][2];
}

cudaError_t brick_create(BrickPlan** out, const Grid& g, float4* E0, float4* E1,
                         const uint8_t* codes, const int* list, int nlist, int shape,
                         cudaStream_t st) {
  *out = nullptr;
  if (shape < 0 || shape > 2) return cudaErrorInvalidValue;
  int bx, by, bz;
  brick_dims(shape, &bx, &by, &bz);
  BrickPlan* pl = new BrickPlan();
  pl->shape = shape;
  float4* src[2] = {E0, E1};
  bool ok = true;
  for (int b = 0; b < 2; ++b) {
    ok &= tma::encode(&pl->maps[b].e, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, src[b] - kXoff4, g,
                      4LL * g.px4, 4 * (bx + 4), by + 4, bz + 4);
    ok &= tma::encode(&pl->maps[b].codes, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1,
                      (void*)(codes - kXoffC), g, g.pxc, bx, by, bz);
  }
  if (!ok) {
    delete pl;
    return cudaErrorInvalidValue;
  }
  const int nbx = (g.nx + bx - 1) / bx, nby = (g.ny + by - 1) / by, nbz = (g.nz + bz - 1) / bz;
  const long long nb = (long long)nbx * nby * nbz;
  std::vector<int> start((size_t)nb);
  int* d_start = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&d_start, sizeof(int) * (size_t)nb, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_start, 0xff, sizeof(int) * (size_t)nb, st);
  if (e == cudaSuccess && nlist > 0) {
    k_brick_starts<<<(nlist + 255) / 256, 256, 0, st>>>(list, nlist, g, bx, by, bz, nbx, nby,
                                                        d_start);
    count_launches(1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(start.data(), d_start, sizeof(int) * (size_t)nb, cudaMemcpyDeviceToHost,
                        st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (d_start) cudaFree(d_start);
  if (e != cudaSuccess) {
    delete pl;
    return e;
  }
  std::vector<int4> work;
  for (long long b = 0; b < nb; ++b) {
    if (start[(size_t)b] < 0) continue;
    const int ix = (int)(b % nbx), r = (int)(b / nbx);
    const int iy = r % nby, iz = r / nby;
    work.push_back(make_int4(ix * bx, iy * by, iz * bz, start[(size_t)b]));
  }
  pl->nwork = (int)work.size();
  work.push_back(make_int4(0, 0, 0, nlist));  // end of the last brick's range
  e = cudaMalloc((void**)&pl->work, sizeof(int4) * work.size());
  if (e == cudaSuccess)
    e = cudaMemcpy(pl->work, work.data(), sizeof(int4) * work.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc((void**)&pl->err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(pl->err, 0, sizeof(int));
  if (e != cudaSuccess) {
    brick_destroy(pl);
    return e;
  }
  if (shape == 0) set_smem_attr<Shape0>();
  else if (shape == 1) set_smem_attr<Shape1>();
  else set_smem_attr<Shape2>();
  *out = pl;
  return cudaSuccess;
}

void brick_destroy(BrickPlan* pl) {
  if (!pl) return;
  cudaFree(pl->work);
  cudaFree(pl->err);
  delete pl;
}

template <class S>
static void launch_s(const BrickPlan* pl, int src, float4* E2, const float4* R, const int* list,
                     const Grid& g, int solver, cudaStream_t st) {
  const long long budget = 4000000000LL;  // ~2 s at 2 GHz
  const BrickMaps& m = pl->maps[src];
  if (solver == 3)
    k_brick_inner<S, 3><<<pl->nwork, kThreads, S::SMEM, st>>>(m, R, E2, list, pl->work, g,
                                                              budget, pl->err);
  else if (solver == 2)
    k_brick_inner<S, 2><<<pl->nwork, kThreads, S::SMEM, st>>>(m, R, E2, list, pl->work, g,
                                                              budget, pl->err);
  else
    k_brick_inner<S, 1><<<pl->nwork, kThreads, S::SMEM, st>>>(m, R, E2, list, pl->work, g,
                                                              budget, pl->err);
}

cudaError_t brick_inner(const BrickPlan* pl, int src, float4* E2, const float4* R,
                        const int* list, const Grid& g, int solver, cudaStream_t st) {
  if (pl->nwork == 0) return cudaSuccess;
  if (pl->shape == 0) launch_s<Shape0>(pl, src, E2, R, list, g, solver, st);
  else if (pl->shape == 1) launch_s<Shape1>(pl, src, E2, R, list, g, solver, st);
  else launch_s<Shape2>(pl, src, E2, R, list, g, solver, st);
  count_launches(1);
  return cudaGetLastError();
}

int* brick_error_flag(const BrickPlan* pl) { return pl->err; }

}  // namespace pm
