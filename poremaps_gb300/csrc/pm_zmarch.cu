// z-marching FP32 correction sweep of the mixed form, fed by TMA.
//
// A CTA owns a TX x TY tile of (x, y) columns and marches z over a chunk of
// planes.  Planes of the four correction fields (with the 2-voxel stencil halo
// in x and y), of the residual and of the voxel codes stream into shared
// memory rings through cp.async.bulk.tensor (one elected thread issues, one
// mbarrier per pipeline stage counts the bytes), prefetched D planes ahead;
// every thread then reads its stencil from shared memory and writes the new
// correction straight to global memory (the other ping-pong buffer, so reads
// and writes never alias).  The correction is interleaved (float4 u, v, w, p
// per voxel): one box per plane, planes z-2..z+2 resident plus D prefetched;
// the residual and the codes are needed for plane z only.  Each plane's fluid
// voxels are compacted into a shared list so computing lanes are full.
//
// Every mbarrier wait is bounded (clock64 budget); on expiry the CTA records
// an error code, drains its own copies still in flight (again bounded) and
// returns, so a broken pipeline never hangs the device.
#include <atomic>

#include "pm_stencil.cuh"
#include "pm_tma.cuh"

#include "pm_zmarch.h"

namespace pm {

namespace {

constexpr int D = 2;  // prefetch depth (planes)
constexpr int NE = 5 + D, NR = 1 + D;

// Tile geometry: TX x TY interior columns, the stencil's 2-voxel halo on each
// side in x and y; one float4 (u, v, w, p) per voxel, so any x start is
// 16-byte aligned and one TMA box carries all four fields of a plane.
template <int TX_, int TY_>
struct Tile {
  static constexpr int TX = TX_, TY = TY_;
  static constexpr int HX = TX + 4, HY = TY + 4;
  static constexpr int PLANE = HX * HY;  // float4 per halo plane
  static constexpr int TILE = TX * TY;   // voxels per interior tile
  static constexpr int THREADS = TILE / 2;  // two columns per thread
  static constexpr unsigned BYTES_PLANE = PLANE * 16, BYTES_TILE = TILE * 16;
  static constexpr unsigned BYTES_GROUP = BYTES_PLANE + BYTES_TILE + TILE;
  static constexpr unsigned BYTES_PRO = 4 * BYTES_PLANE;  // planes z0-2 .. z0+1
};

template <class T>
struct Smem {
  float4 e[NE][T::PLANE];
  float4 r[NR][T::TILE];
  uint8_t codes[NR][T::TILE];
  unsigned long long bar[NR];
  unsigned long long bar_pro;
  unsigned short list[T::TILE];  // fluid voxels of the current plane (tile offsets)
  int warp_count[T::THREADS / 32];
  static_assert(T::PLANE * 16 % 128 == 0, "TMA slots must stay 128-byte aligned");
  static_assert(T::TILE % 128 == 0, "code slots must stay 128-byte aligned");
};

using TileA = Tile<32, 16>;
using TileB = Tile<32, 8>;

using tma::mbar_expect;
using tma::mbar_init;
using tma::mbar_wait;

__device__ __forceinline__ void tma_load3(void* dst, const CUtensorMap* map, int x, int y, int z,
                                          unsigned long long* bar) {
  tma::load3(dst, map, x, y, z, bar);
}

struct Maps {
  CUtensorMap e;      // source correction (halo boxes), float4 viewed as 4 floats
  CUtensorMap r;      // residual (interior boxes)
  CUtensorMap codes;  // voxel codes (interior boxes)
};

template <class T, int SOLVER>
__global__ void __launch_bounds__(T::THREADS)
    k_zmarch_inner(const __grid_constant__ Maps maps, float4* E2, Grid g, int zchunk,
                   long long budget, int* err, int fail_first) {
  constexpr int TX = T::TX, TY = T::TY, HX = T::HX, THREADS = T::THREADS;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  Smem<T>& S = *reinterpret_cast<Smem<T>*>(smem_raw);
  const int bx = blockIdx.x, by = blockIdx.y;
  const int z0 = 2 + blockIdx.z * zchunk;
  const int z1 = min(z0 + zchunk, g.NZ - 2);
  if (z0 >= z1) return;
  const int L = z1 - z0;
  // TMA coordinates in floats (x) / rows (y) / planes (z); one float4 = 4 floats
  const int xe = 4 * (kXoff4 + bx * TX);      // halo box: padded x from bx*TX
  const int ye = by * TY;                     // halo box: padded y from by*TY
  const int xr = 4 * (kXoff4 + 2 + bx * TX);  // interior box
  const int yr = 2 + by * TY;
  const int xc = kXoffC + 2 + bx * TX;
  const bool leader = threadIdx.x == 0;

  auto issue_group = [&](int j) {  // loads needed first by compute step j
    const int z = z0 + j;
    unsigned long long* b = &S.bar[j % NR];
    mbar_expect(b, T::BYTES_GROUP);
    tma_load3(S.e[(j + 4) % NE], &maps.e, xe, ye, z + 2, b);
    tma_load3(S.r[j % NR], &maps.r, xr, yr, z, b);
    tma_load3(S.codes[j % NR], &maps.codes, xc, yr, z, b);
  };

  if (leader) {
    for (int i = 0; i < NR; ++i) mbar_init(&S.bar[i], 1);
    mbar_init(&S.bar_pro, 1);
    tma::fence_mbar_init();
  }
  __syncthreads();
  if (leader) {
    // prologue: planes z0-2 .. z0+1 into slots 0..3 (plane z0-2 is slot 0)
    mbar_expect(&S.bar_pro, T::BYTES_PRO);
    for (int k = 0; k < 4; ++k) tma_load3(S.e[k], &maps.e, xe, ye, z0 - 2 + k, &S.bar_pro);
    for (int j = 0; j < D + 1 && j < L; ++j) issue_group(j);
  }
  int issued = min(D + 1, L);
  int waited = 0;  // groups whose barrier phase every thread has observed
  // fail_first (test hook): the first wait reports a timeout without waiting,
  // which exercises the failure path below with real copies in flight
  bool ok = __syncthreads_and(fail_first ? false : mbar_wait(&S.bar_pro, 0, budget));

  const int tx = threadIdx.x % (TX / 2), ty = threadIdx.x / (TX / 2);
  const int yp = by * TY + ty;  // interior y
  const long long px = g.px4, pl = g.pl4;

  for (int j = 0; j < L && ok; ++j) {
    ok = __syncthreads_and(mbar_wait(&S.bar[j % NR], (j / NR) & 1, budget));
    if (!ok) break;
    waited = j + 1;
    const int z = z0 + j;
    const int sr = j % NR;
    // compact the fluid voxels of this plane so that every computing lane has one
    unsigned fl[2];
    int nmine = 0;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int xp = bx * TX + tx * 2 + q;
      fl[q] = (xp < g.nx && yp < g.ny && S.codes[sr][ty * TX + tx * 2 + q]) ? 1u : 0u;
      nmine += fl[q];
    }
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int pre = nmine;  // inclusive scan of nmine over the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, pre, o);
      if ((int)lane >= o) pre += t;
    }
    if (lane == 31) S.warp_count[warp] = pre;
    __syncthreads();
    int base = 0, nfl = 0;
#pragma unroll
    for (int w = 0; w < THREADS / 32; ++w) {
      const int c = S.warp_count[w];
      base += (w < (int)warp) ? c : 0;
      nfl += c;
    }
    int pos = base + pre - nmine;
#pragma unroll
    for (int q = 0; q < 2; ++q)
      if (fl[q]) S.list[pos++] = (unsigned short)(ty * TX + tx * 2 + q);
    __syncthreads();
    const float4* P[5];  // planes z-2 .. z+2
#pragma unroll
    for (int d = 0; d < 5; ++d) P[d] = S.e[(j + d) % NE];
    for (int k = threadIdx.x; k < nfl; k += THREADS) {
      const int t = S.list[k];
      const int ly = t / TX, lx = t - ly * TX;
      const int code = S.codes[sr][t];
      const int c0 = (ly + 2) * HX + lx + 2;  // centre in the halo planes
      const float4 C = P[2][c0];
      const float4 XM = P[2][c0 - 1], XP = P[2][c0 + 1], XMM = P[2][c0 - 2], XPP = P[2][c0 + 2];
      const float4 YM = P[2][c0 - HX], YP = P[2][c0 + HX];
      const float4 YMM = P[2][c0 - 2 * HX], YPP = P[2][c0 + 2 * HX];
      const float4 ZM = P[1][c0], ZP = P[3][c0], ZMM = P[0][c0], ZPP = P[4][c0];
      Stencil<float> s;
      s.uc = C.x; s.uxm = XM.x; s.uxp = XP.x; s.uym = YM.x; s.uyp = YP.x;
      s.uymm = YMM.x; s.uypp = YPP.x; s.uzm = ZM.x; s.uzp = ZP.x; s.uzmm = ZMM.x; s.uzpp = ZPP.x;
      s.vc = C.y; s.vxm = XM.y; s.vxp = XP.y; s.vxmm = XMM.y; s.vxpp = XPP.y; s.vym = YM.y;
      s.vyp = YP.y; s.vzm = ZM.y; s.vzp = ZP.y; s.vzmm = ZMM.y; s.vzpp = ZPP.y;
      s.wc = C.z; s.wxm = XM.z; s.wxp = XP.z; s.wxmm = XMM.z; s.wxpp = XPP.z; s.wym = YM.z;
      s.wyp = YP.z; s.wymm = YMM.z; s.wypp = YPP.z; s.wzm = ZM.z; s.wzp = ZP.z;
      s.pc = (z == g.NZ - 3) ? 0.f : C.w;
      s.pxm = XM.w; s.pym = YM.w; s.pzm = ZM.w;
      float un, vn, wn, pn;
      update_fast<float, SOLVER>(s, code, un, vn, wn, pn);
      const float4 r = S.r[sr][t];
      const int x = bx * TX + lx + 2, y = by * TY + ly + 2;
      write_voxel4(E2, (long long)z * pl + (long long)y * px + x, x, y, z, g, un + r.x,
                   vn + r.y, wn + r.z, pn + r.w);
    }
    __syncthreads();  // every thread is done with the slots group j+D+1 reuses
    if (leader && issued < L) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue_group(issued);
      ++issued;
    }
  }
  if (!ok) {
    // record the failure, then drain this CTA's copies still in flight (each
    // pending group has its own barrier: at most NR groups are outstanding)
    if (leader) {
      atomicExch(err, 1);
      mbar_wait(&S.bar_pro, 0, budget);
      for (int j = waited; j < issued; ++j) mbar_wait(&S.bar[j % NR], (j / NR) & 1, budget);
    }
    __syncthreads();
  }
}

}  // namespace

namespace tma {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  // looked up once; the initialisation of a function-local static is
  // thread-safe (problems are created from several host threads at once)
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return (PFN_cuTensorMapEncodeTiled_v12000)p;
    return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
  }();
  return fn;
}

// 3-D map over a padded array: dims {pitch elements, NY, NZ}, box {bx, by, bz}.
bool encode(CUtensorMap* m, CUtensorMapDataType t, int esize, void* base, const Grid& g,
            long long pitch, unsigned bx, unsigned by, unsigned bz) {
  auto fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[3] = {(cuuint64_t)pitch, (cuuint64_t)g.NY, (cuuint64_t)g.NZ};
  cuuint64_t strides[2] = {(cuuint64_t)pitch * esize, (cuuint64_t)pitch * g.NY * esize};
  cuuint32_t box[3] = {bx, by, bz};
  cuuint32_t es[3] = {1, 1, 1};
  return fn(m, t, 3, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace tma

struct ZmarchPlan {
  Maps maps[2];  // source buffer E0 / E1
  int* err = nullptr;
  int zchunk = 0;
  int tile = 0;  // 0: 32 x 16, 1: 32 x 8
  dim3 grid;
};

int zmarch_available() { return tma::encode_fn() != nullptr; }

template <class T>
static void set_smem_attr() {
  static std::atomic<bool> done{false};
  if (done.load()) return;
  cudaFuncSetAttribute(k_zmarch_inner<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(Smem<T>));
  cudaFuncSetAttribute(k_zmarch_inner<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(Smem<T>));
  cudaFuncSetAttribute(k_zmarch_inner<T, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(Smem<T>));
  done = true;
}

cudaError_t zmarch_create(ZmarchPlan** out, const Grid& g, float4* E0, float4* E1, float4* R,
                          const uint8_t* codes, int zchunk, int tile) {
  *out = nullptr;
  ZmarchPlan* pl = new ZmarchPlan();
  pl->tile = tile;
  const int TX = tile ? TileB::TX : TileA::TX, TY = tile ? TileB::TY : TileA::TY;
  const size_t smem = tile ? sizeof(Smem<TileB>) : sizeof(Smem<TileA>);
  const int per_sm = tile ? 3 : 2;  // resident CTAs per SM at this shared-memory size
  float4* src[2] = {E0, E1};
  bool ok = true;
  for (int b = 0; b < 2; ++b) {
    ok &= tma::encode(&pl->maps[b].e, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, src[b] - kXoff4, g,
                      4LL * g.px4, 4 * (TX + 4), TY + 4, 1);
    ok &= tma::encode(&pl->maps[b].r, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, R - kXoff4, g,
                      4LL * g.px4, 4 * TX, TY, 1);
    ok &= tma::encode(&pl->maps[b].codes, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1,
                      (void*)(codes - kXoffC), g, g.pxc, TX, TY, 1);
  }
  if (!ok) {
    delete pl;
    return cudaErrorInvalidValue;
  }
  cudaError_t e = cudaMalloc((void**)&pl->err, sizeof(int));
  if (e != cudaSuccess) {
    delete pl;
    return e;
  }
  cudaMemset(pl->err, 0, sizeof(int));
  int gx = (g.nx + TX - 1) / TX, gy = (g.ny + TY - 1) / TY;
  if (zchunk <= 0) {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // one wave of resident CTAs, never a partial second wave
    long long slots = (long long)per_sm * sms;
    int nch = (int)std::max(1LL, slots / ((long long)gx * gy));
    zchunk = (g.nz + nch - 1) / nch;
    if (zchunk < 8) zchunk = std::min(8, g.nz);
  }
  (void)smem;
  pl->zchunk = zchunk;
  pl->grid = dim3(gx, gy, (g.nz + zchunk - 1) / zchunk);
  if (tile) set_smem_attr<TileB>();
  else set_smem_attr<TileA>();
  *out = pl;
  return cudaSuccess;
}

void zmarch_destroy(ZmarchPlan* pl) {
  if (!pl) return;
  cudaFree(pl->err);
  delete pl;
}

// pm_debug_tma_fail: the next z-march launches report a timed-out first wait.
static std::atomic<int> g_tma_fail{0};

template <class T>
static void launch_t(const ZmarchPlan* pl, int src, float4* E2, const Grid& g, int solver,
                     cudaStream_t st) {
  const long long budget = 4000000000LL;  // ~2 s at 2 GHz per wait
  const size_t sm = sizeof(Smem<T>);
  const int ff = g_tma_fail.load();
  if (solver == 3)
    k_zmarch_inner<T, 3><<<pl->grid, T::THREADS, sm, st>>>(pl->maps[src], E2, g, pl->zchunk,
                                                          budget, pl->err, ff);
  else if (solver == 2)
    k_zmarch_inner<T, 2><<<pl->grid, T::THREADS, sm, st>>>(pl->maps[src], E2, g, pl->zchunk,
                                                          budget, pl->err, ff);
  else
    k_zmarch_inner<T, 1><<<pl->grid, T::THREADS, sm, st>>>(pl->maps[src], E2, g, pl->zchunk,
                                                          budget, pl->err, ff);
}

void zmarch_debug_fail(int on) { g_tma_fail.store(on ? 1 : 0); }

cudaError_t zmarch_inner(const ZmarchPlan* pl, int src, float4* E2, const Grid& g, int solver,
                         cudaStream_t st) {
  if (pl->tile) launch_t<TileB>(pl, src, E2, g, solver, st);
  else launch_t<TileA>(pl, src, E2, g, solver, st);
  count_launches(1);
  return cudaGetLastError();
}

int* zmarch_error_flag(const ZmarchPlan* pl) { return pl->err; }

}  // namespace pm
