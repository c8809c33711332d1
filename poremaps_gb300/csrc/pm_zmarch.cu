// z-marching FP32 correction sweep of the mixed form, fed by TMA.
//
// A CTA owns a TX x TY tile of (x, y) columns and marches z over a chunk of
// planes.  Planes of the four correction fields (with the 2-voxel stencil halo
// in x and y), of the residual and of the voxel codes stream into shared
// memory rings through cp.async.bulk.tensor (one elected thread issues, one
// mbarrier per pipeline stage counts the bytes), prefetched D planes ahead;
// every thread then reads its stencil from shared memory and writes the new
// correction straight to global memory (the other ping-pong buffer, so reads
// and writes never alias).  Ring depths follow the stencil reach: u, v need
// planes z-2..z+2, w z-1..z+1, p z-1..z, r and the codes plane z.
//
// Every mbarrier wait is bounded (clock64 budget); on expiry the CTA records
// an error code, drains its own copies still in flight (again bounded) and
// returns, so a broken pipeline never hangs the device.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "pm_stencil.cuh"
#include "pm_zmarch.h"

namespace pm {

namespace {

constexpr int VX = 2;
constexpr int D = 2;  // prefetch depth (planes)
constexpr int NU = 5 + D, NW = 3 + D, NP = 2 + D, NR = 1 + D;

// Tile geometry: TX x TY interior columns; the x halo starts on a 16-byte
// boundary (HX = TX + 8), the y halo is the stencil's 2 rows on each side.
template <int TX_, int TY_>
struct Tile {
  static constexpr int TX = TX_, TY = TY_;
  static constexpr int HX = TX + 8, HY = TY + 4;
  static constexpr int PLANE_F = HX * HY;  // floats per halo plane of one field
  static constexpr int TILE_F = TX * TY;   // floats per interior tile of one field
  static constexpr int THREADS = (TX / VX) * TY;
  static constexpr unsigned BYTES_PLANE = PLANE_F * 4, BYTES_TILE = TILE_F * 4;
  static constexpr unsigned BYTES_CODES = TILE_F;
  static constexpr unsigned BYTES_GROUP = 4 * BYTES_PLANE + 4 * BYTES_TILE + BYTES_CODES;
  static constexpr unsigned BYTES_PRO = (4 + 4 + 2 + 1) * BYTES_PLANE;  // u,v 4, w 2, p 1
};

template <class T>
struct Smem {
  static constexpr int PLANE_F = T::PLANE_F, TILE_F = T::TILE_F, THREADS = T::THREADS;
  float u[NU][PLANE_F];
  float v[NU][PLANE_F];
  float w[NW][PLANE_F];
  float p[NP][PLANE_F];
  float r[NR][4][TILE_F];
  uint8_t codes[NR][TILE_F];
  unsigned long long bar[NR];
  unsigned long long bar_pro;
  unsigned short list[TILE_F];  // fluid voxels of the current plane (tile offsets)
  int warp_count[THREADS / 32];
  static_assert(sizeof(float) * PLANE_F % 128 == 0, "TMA slots must stay 128-byte aligned");
  static_assert(sizeof(float) * TILE_F % 128 == 0, "TMA slots must stay 128-byte aligned");
  static_assert(TILE_F % 128 == 0, "code slots must stay 128-byte aligned");
};

using TileA = Tile<32, 16>;
using TileB = Tile<64, 8>;

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count));
}

__device__ __forceinline__ void mbar_expect(unsigned long long* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(b)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try(unsigned long long* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: false once about `budget` clock cycles have passed.
__device__ __forceinline__ bool mbar_wait(unsigned long long* b, unsigned parity,
                                          long long budget) {
  long long t0 = clock64();
  for (unsigned i = 0;; ++i) {
    if (mbar_try(b, parity)) return true;
    if ((i & 255) == 255 && clock64() - t0 > budget) return false;
  }
}

__device__ __forceinline__ void tma_load3(void* dst, const CUtensorMap* map, int x, int y, int z,
                                          unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
      "l"((unsigned long long)map), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

struct Maps {
  CUtensorMap e[4];  // source correction u, v, w, p (halo boxes)
  CUtensorMap r[4];  // residual (interior boxes)
  CUtensorMap codes; // voxel codes (interior boxes)
};

template <class T, int SOLVER>
__global__ void __launch_bounds__(T::THREADS, 2)
    k_zmarch_inner(const __grid_constant__ Maps maps, Fields<float> E2, Grid g, int zchunk,
                   long long budget, int* err) {
  constexpr int TX = T::TX, TY = T::TY, HX = T::HX, THREADS = T::THREADS;
  constexpr unsigned BYTES_GROUP = T::BYTES_GROUP, BYTES_PRO = T::BYTES_PRO;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  Smem<T>& S = *reinterpret_cast<Smem<T>*>(smem_raw);
  const int bx = blockIdx.x, by = blockIdx.y;
  const int z0 = 2 + blockIdx.z * zchunk;
  const int z1 = min(z0 + zchunk, g.NZ - 2);
  if (z0 >= z1) return;
  const int L = z1 - z0;
  const int xe = kXoff32 - 2 + bx * TX;  // halo box start: padded x = bx*TX - 2
  const int ye = by * TY;                          // halo box start: padded y = by*TY
  const int xr = kXoff32 + 2 + bx * TX, yr = 2 + by * TY;
  const int xc = kXoffC + 2 + bx * TX;
  const bool leader = threadIdx.x == 0;

  auto issue_group = [&](int j) {  // loads needed first by compute step j
    const int z = z0 + j;
    unsigned long long* b = &S.bar[j % NR];
    mbar_expect(b, BYTES_GROUP);
    tma_load3(S.u[(j + 4) % NU], &maps.e[0], xe, ye, z + 2, b);
    tma_load3(S.v[(j + 4) % NU], &maps.e[1], xe, ye, z + 2, b);
    tma_load3(S.w[(j + 2) % NW], &maps.e[2], xe, ye, z + 1, b);
    tma_load3(S.p[(j + 1) % NP], &maps.e[3], xe, ye, z, b);
    for (int f = 0; f < 4; ++f) tma_load3(S.r[j % NR][f], &maps.r[f], xr, yr, z, b);
    tma_load3(S.codes[j % NR], &maps.codes, xc, yr, z, b);
  };

  if (leader) {
    for (int i = 0; i < NR; ++i) mbar_init(&S.bar[i], 1);
    mbar_init(&S.bar_pro, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (leader) {
    // prologue: u, v planes z0-2..z0+1 (slots 0..3), w z0-1, z0 (slots 0, 1), p z0-1 (slot 0)
    mbar_expect(&S.bar_pro, BYTES_PRO);
    for (int k = 0; k < 4; ++k) {
      tma_load3(S.u[k], &maps.e[0], xe, ye, z0 - 2 + k, &S.bar_pro);
      tma_load3(S.v[k], &maps.e[1], xe, ye, z0 - 2 + k, &S.bar_pro);
    }
    tma_load3(S.w[0], &maps.e[2], xe, ye, z0 - 1, &S.bar_pro);
    tma_load3(S.w[1], &maps.e[2], xe, ye, z0, &S.bar_pro);
    tma_load3(S.p[0], &maps.e[3], xe, ye, z0 - 1, &S.bar_pro);
    for (int j = 0; j < D + 1 && j < L; ++j) issue_group(j);
  }
  int issued = min(D + 1, L);
  int waited = 0;  // groups whose barrier phase every thread has observed
  bool ok = __syncthreads_and(mbar_wait(&S.bar_pro, 0, budget));

  const int tx = threadIdx.x % (TX / VX), ty = threadIdx.x / (TX / VX);
  const int yp = by * TY + ty;  // interior y
  const long long px = g.px32, pl = g.pl32;

  for (int j = 0; j < L && ok; ++j) {
    ok = __syncthreads_and(mbar_wait(&S.bar[j % NR], (j / NR) & 1, budget));
    if (!ok) break;
    waited = j + 1;
    const int z = z0 + j;
    const int sr = j % NR;
    // compact the fluid voxels of this plane so that every computing lane has one
    unsigned fl[VX];
    int nmine = 0;
#pragma unroll
    for (int q = 0; q < VX; ++q) {
      const int xp = bx * TX + tx * VX + q;
      fl[q] = (xp < g.nx && yp < g.ny && S.codes[sr][ty * TX + tx * VX + q]) ? 1u : 0u;
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
    for (int q = 0; q < VX; ++q)
      if (fl[q]) S.list[pos++] = (unsigned short)(ty * TX + tx * VX + q);
    __syncthreads();
    // plane pointers of the rings for this step
    const float* up[5];
    const float* vp[5];
#pragma unroll
    for (int d = 0; d < 5; ++d) {
      up[d] = S.u[(j + d) % NU];  // plane z-2+d (plane z0-2 is slot 0)
      vp[d] = S.v[(j + d) % NU];
    }
    const float* wp[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) wp[d] = S.w[(j + d) % NW];  // plane z-1+d
    const float* pzm = S.p[j % NP];                         // plane z-1
    const float* pc = S.p[(j + 1) % NP];                    // plane z
    const float* rr[4] = {S.r[sr][0], S.r[sr][1], S.r[sr][2], S.r[sr][3]};
    for (int k = threadIdx.x; k < nfl; k += THREADS) {
      const int t = S.list[k];
      const int ly = t / TX, lx = t - ly * TX;
      const int code = S.codes[sr][t];
      const int c0 = (ly + 2) * HX + lx + 4;  // centre in the halo planes
      Stencil<float> s;
      s.uc = up[2][c0]; s.uxm = up[2][c0 - 1]; s.uxp = up[2][c0 + 1];
      s.uym = up[2][c0 - HX]; s.uyp = up[2][c0 + HX];
      s.uymm = up[2][c0 - 2 * HX]; s.uypp = up[2][c0 + 2 * HX];
      s.uzm = up[1][c0]; s.uzp = up[3][c0]; s.uzmm = up[0][c0]; s.uzpp = up[4][c0];
      s.vc = vp[2][c0]; s.vxm = vp[2][c0 - 1]; s.vxp = vp[2][c0 + 1];
      s.vxmm = vp[2][c0 - 2]; s.vxpp = vp[2][c0 + 2];
      s.vym = vp[2][c0 - HX]; s.vyp = vp[2][c0 + HX];
      s.vzm = vp[1][c0]; s.vzp = vp[3][c0]; s.vzmm = vp[0][c0]; s.vzpp = vp[4][c0];
      s.wc = wp[1][c0]; s.wxm = wp[1][c0 - 1]; s.wxp = wp[1][c0 + 1];
      s.wxmm = wp[1][c0 - 2]; s.wxpp = wp[1][c0 + 2];
      s.wym = wp[1][c0 - HX]; s.wyp = wp[1][c0 + HX];
      s.wymm = wp[1][c0 - 2 * HX]; s.wypp = wp[1][c0 + 2 * HX];
      s.wzm = wp[0][c0]; s.wzp = wp[2][c0];
      s.pc = (z == g.NZ - 3) ? 0.f : pc[c0];
      s.pxm = pc[c0 - 1]; s.pym = pc[c0 - HX]; s.pzm = pzm[c0];
      float un, vn, wn, pn;
      update_fast<float, SOLVER>(s, code, un, vn, wn, pn);
      un += rr[0][t];
      vn += rr[1][t];
      wn += rr[2][t];
      pn += rr[3][t];
      const int x = bx * TX + lx + 2, y = by * TY + ly + 2;
      write_voxel<float, true>(E2, (long long)z * pl + (long long)y * px + x, x, y, z, g, px, pl,
                               un, vn, wn, pn);
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

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

bool encode(CUtensorMap* m, CUtensorMapDataType t, int esize, void* base, const Grid& g,
            long long pitch, unsigned bx, unsigned by) {
  auto fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[3] = {(cuuint64_t)pitch, (cuuint64_t)g.NY, (cuuint64_t)g.NZ};
  cuuint64_t strides[2] = {(cuuint64_t)pitch * esize, (cuuint64_t)pitch * g.NY * esize};
  cuuint32_t box[3] = {bx, by, 1};
  cuuint32_t es[3] = {1, 1, 1};
  return fn(m, t, 3, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

struct ZmarchPlan {
  Maps maps[2];  // source buffer E0 / E1
  int* err = nullptr;
  int zchunk = 0;
  int tile = 0;  // 0: 32 x 16, 1: 64 x 8
  dim3 grid;
};

int zmarch_available() { return encode_fn() != nullptr; }

template <class T>
static void set_smem_attr() {
  static bool done = false;
  if (done) return;
  cudaFuncSetAttribute(k_zmarch_inner<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(Smem<T>));
  cudaFuncSetAttribute(k_zmarch_inner<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(Smem<T>));
  cudaFuncSetAttribute(k_zmarch_inner<T, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sizeof(Smem<T>));
  done = true;
}

cudaError_t zmarch_create(ZmarchPlan** out, const Grid& g, Fields<float> E0, Fields<float> E1,
                          Fields<float> R, const uint8_t* codes, int zchunk, int tile) {
  *out = nullptr;
  ZmarchPlan* pl = new ZmarchPlan();
  pl->tile = tile;
  const int TX = tile ? TileB::TX : TileA::TX, TY = tile ? TileB::TY : TileA::TY;
  const unsigned HX = TX + 8, HY = TY + 4;
  Fields<float> src[2] = {E0, E1};
  bool ok = true;
  for (int b = 0; b < 2; ++b) {
    float* f[4] = {src[b].u, src[b].v, src[b].w, src[b].p};
    float* rf[4] = {R.u, R.v, R.w, R.p};
    for (int k = 0; k < 4; ++k) {
      ok &= encode(&pl->maps[b].e[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, f[k] - kXoff32, g,
                   g.px32, HX, HY);
      ok &= encode(&pl->maps[b].r[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, rf[k] - kXoff32, g,
                   g.px32, TX, TY);
    }
    ok &= encode(&pl->maps[b].codes, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1,
                 (void*)(codes - kXoffC), g, g.pxc, TX, TY);
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
    // one wave: at most two resident CTAs per SM, so no partial second wave
    long long slots = 2LL * sms;
    int nch = (int)std::max(1LL, slots / ((long long)gx * gy));
    zchunk = (g.nz + nch - 1) / nch;
    if (zchunk < 8) zchunk = std::min(8, g.nz);
  }
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

template <class T>
static void launch_t(const ZmarchPlan* pl, int src, Fields<float> E2, const Grid& g, int solver,
                     cudaStream_t st) {
  const long long budget = 4000000000LL;  // ~2 s at 2 GHz per wait
  const size_t sm = sizeof(Smem<T>);
  if (solver == 3)
    k_zmarch_inner<T, 3><<<pl->grid, T::THREADS, sm, st>>>(pl->maps[src], E2, g, pl->zchunk,
                                                          budget, pl->err);
  else if (solver == 2)
    k_zmarch_inner<T, 2><<<pl->grid, T::THREADS, sm, st>>>(pl->maps[src], E2, g, pl->zchunk,
                                                          budget, pl->err);
  else
    k_zmarch_inner<T, 1><<<pl->grid, T::THREADS, sm, st>>>(pl->maps[src], E2, g, pl->zchunk,
                                                          budget, pl->err);
}

cudaError_t zmarch_inner(const ZmarchPlan* pl, int src, Fields<float> E2, const Grid& g,
                         int solver, cudaStream_t st) {
  if (pl->tile) launch_t<TileB>(pl, src, E2, g, solver, st);
  else launch_t<TileA>(pl, src, E2, g, solver, st);
  count_launches(1);
  return cudaGetLastError();
}

int* zmarch_error_flag(const ZmarchPlan* pl) { return pl->err; }

}  // namespace pm
