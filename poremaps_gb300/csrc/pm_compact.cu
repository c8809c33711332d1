// Compact correction store of the mixed-precision form (correction-sweep
// kernels 8 and 9, and the server's batched sweeps).
//
// The FP32 correction e and residual r hold one float4 (u, v, w, p) per
// fluid voxel, at the voxel's position in the lexicographic fluid list,
// instead of one per voxel of the padded box, plus one zero slot.  A sweep
// then reads and writes only fluid data: 32 consecutive list entries are 512
// contiguous bytes, so the centre, the residual and the store are fully
// coalesced 128-bit accesses, the +-x neighbours are the adjacent entries and
// a warp's +-y / +-z neighbours lie in a few contiguous runs of the
// neighbouring rows.  Each voxel reads six neighbour positions, set up once
// from the neighbourhood cases (eval_geometry, src/geometry.cc:273-296 of the
// reference): solid neighbours point at the zero slot (a solid voxel's
// correction is 0), and the twelve stencil points fit in six because a wall
// stencil that needs a second neighbour has a solid first neighbour on the
// other side.  Periodic halos are not stored; a read across a periodic face
// takes the image voxel, a read across a wall face the zero slot
// (homogeneous boundary values of the correction).
//
// Positions of the voxels of other rows come from a bit-packed fluid mask:
// per row and 32 consecutive x one word {fluid bits, number of fluid voxels
// before the word}, i.e. 1/4 byte per voxel; position = base + popc(bits
// below x).  The mask also serves the reductions that read the correction.
//
// Every kernel here gives the same values as its padded counterpart in
// pm_fast.cu bit for bit: the stencil sees the same numbers (zeros where the
// padded store holds zeros, images where it holds halo copies) and runs the
// same update_fast<float>.
#include <atomic>

#include "pm_compact.h"
#include "pm_compact.cuh"
#include "pm_tma.cuh"

namespace pm {

namespace {

// Persistent: one wave of MINB CTAs per SM walks the list positions with a
// grid stride.  PF: each thread loads the metadata and slots of its next
// position before it sweeps the current one, so only the correction loads
// wait (3 or 4 CTAs per SM).  Without PF the kernel fits in 48 registers and
// runs 5 CTAs per SM: the slot loads wait too, but 40 resident warps instead
// of 32 hide more of the latency when several problems share the device (the
// three rotations of the tensor: 2.75 against 2.86 ms per 100-sweep step of
// the 128^3 sphere pack; alone both take 10.4 us).
template <int SOLVER, int MINB, bool PF>
__global__ void __launch_bounds__(256, MINB) k_dc_inner_c(const float4* __restrict__ E,
                                                         float4* __restrict__ E2,
                                                         const float4* __restrict__ R,
                                                         const unsigned* __restrict__ meta,
                                                         const int4* __restrict__ sa,
                                                         const int2* __restrict__ sb,
                                                         int nlist) {
  const int stride = gridDim.x * blockDim.x;
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (!PF) {
    for (; q < nlist; q += stride) inner_c_voxel<SOLVER>(E, E2, R, meta, sa, sb, q);
    return;
  }
  if (q >= nlist) return;
  unsigned m = __ldg(meta + q);
  CompactSlots sl;
  sl.a = __ldg(sa + q);
  sl.b = __ldg(sb + q);
  for (; q < nlist; q += stride) {
    const int qn = q + stride;
    unsigned mn = 0;
    CompactSlots sn;
    sn.a = make_int4(0, 0, 0, 0);
    sn.b = make_int2(0, 0);
    if (qn < nlist) {
      mn = __ldg(meta + qn);
      sn.a = __ldg(sa + qn);
      sn.b = __ldg(sb + qn);
    }
    inner_c_compute<SOLVER>(E, E2, R, q, m, sl);
    m = mn;
    sl = sn;
  }
}

// Bulk-staged form (kernel 11): the metadata and neighbour slots of a chunk of
// kChunk consecutive list positions (one per thread) reach shared memory by
// three untiled bulk copies (cp.async.bulk, one mbarrier per stage counting
// the bytes), kStages chunks ahead, so each voxel issues its eight correction
// loads at once instead of after its slot loads; no slot registers are held
// across voxels.  Thread 0 issues the copies; each warp arrives on the
// stage's `empty` barrier once its threads have read their entries, and
// thread 0 waits for all eight before it reuses the stage.  Every wait is
// bounded (clock64 budget): on expiry the CTA records the failure in *err,
// thread 0 waits (bounded) for the copies it issued and the CTA returns.
// The arrays are read past the last position up to the next 16 bytes: meta
// needs nlist + 4 entries and sb nlist + 2 (compact store allocation).
// Bitwise equal to kernels 8-10 but slower on the 128^3 sphere pack: 13.4 /
// 12.4 us per sweep alone at 5 / 4 CTAs per SM against 10.4 us for kernel
// 10, 3.35 / 3.28 against 2.76 ms per step of the three rotated problems.
// Each chunk ties the CTA's eight warps to one pipeline (a slow warp holds
// the refill of its stage), and the 21.5 KB of stages per CTA come out of
// the L1 that serves the neighbour gathers.  Selectable, not autotuned.
constexpr int kChunk = 256;
constexpr int kStages = 3;

template <int SOLVER, int MINB>
__global__ void __launch_bounds__(kChunk, MINB)
    k_dc_inner_cb(const float4* __restrict__ E, float4* __restrict__ E2,
                  const float4* __restrict__ R, const unsigned* __restrict__ meta,
                  const int4* __restrict__ sa, const int2* __restrict__ sb, int nlist, int* err,
                  long long budget, int fail_first) {
  __shared__ __align__(16) int4 s_sa[kStages][kChunk];
  __shared__ __align__(16) int2 s_sb[kStages][kChunk];
  __shared__ __align__(16) unsigned s_m[kStages][kChunk];
  __shared__ __align__(8) unsigned long long full[kStages], empty[kStages];
  const int nchunks = (nlist + kChunk - 1) / kChunk;
  const int my = (int)blockIdx.x < nchunks ? (nchunks - 1 - (int)blockIdx.x) / (int)gridDim.x + 1
                                           : 0;
  const bool leader = threadIdx.x == 0;
  if (leader) {
    for (int s = 0; s < kStages; ++s) {
      tma::mbar_init(&full[s], 1);
      tma::mbar_init(&empty[s], kChunk / 32);
    }
    tma::fence_mbar_init();
  }
  __syncthreads();
  auto first_pos = [&](int j) {
    return ((long long)blockIdx.x + (long long)j * gridDim.x) * kChunk;
  };
  auto issue = [&](int j) {
    const int s = j % kStages;
    const long long q0 = first_pos(j);
    const int n = (int)min((long long)kChunk, (long long)nlist - q0);
    const unsigned bm = (unsigned)(n * 4 + 15) & ~15u, bb = (unsigned)(n * 8 + 15) & ~15u,
                   ba = (unsigned)n * 16u;
    tma::mbar_expect(&full[s], bm + bb + ba);
    tma::bulk_g2s(s_m[s], meta + q0, bm, &full[s]);
    tma::bulk_g2s(s_sb[s], sb + q0, bb, &full[s]);
    tma::bulk_g2s(s_sa[s], sa + q0, ba, &full[s]);
  };
  int issued = 0;
  if (leader)
    for (; issued < kStages && issued < my; ++issued) issue(issued);
  bool ok = true;
  int j = 0;
  for (; j < my; ++j) {
    const int s = j % kStages;
    const unsigned par = (unsigned)(j / kStages) & 1u;
    // fail_first (test hook): the first wait reports a timeout without waiting
    if ((fail_first && j == 0) || !tma::mbar_wait(&full[s], par, budget)) {
      ok = false;
      break;
    }
    const long long q = first_pos(j) + threadIdx.x;
    const bool act = q < nlist;
    unsigned m = 0;
    CompactSlots sl;
    if (act) {
      m = s_m[s][threadIdx.x];
      sl.a = s_sa[s][threadIdx.x];
      sl.b = s_sb[s][threadIdx.x];
    }
    __syncwarp();
    if ((threadIdx.x & 31) == 0) tma::mbar_arrive(&empty[s]);
    if (leader && issued < my) {
      // every warp has read stage s: refill it with chunk j + kStages
      if (!tma::mbar_wait(&empty[s], par, budget)) {
        ok = false;
        break;
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(issued);
      ++issued;
    }
    if (act) inner_c_compute<SOLVER>(E, E2, R, (int)q, m, sl);
  }
  if (!ok) {
    atomicExch(err, 1);
    // drain: thread 0 waits for the copies it issued that nobody waited for
    if (leader)
      for (int k = j; k < issued; ++k)
        tma::mbar_wait(&full[k % kStages], (unsigned)(k / kStages) & 1u, budget);
  }
}

// r = F(x) - x in FP64 from the padded state (as dc_residual_voxel), stored
// at the list position, and e1 = r.
template <int SOLVER>
__global__ void __launch_bounds__(256, 2) k_dc_residual_c(Fields<double> X, float4* R,
                                                        float4* E, const uint8_t* codes,
                                                        const int* list, int nlist, Grid g) {
  __shared__ double ctab[16];
  fill_centre_table<SOLVER>(ctab);
  __syncthreads();
  const int stride = gridDim.x * blockDim.x;
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  int lin = q < nlist ? __ldg(list + q) : 0;
  for (; q < nlist; q += stride) {
    const int qn = q + stride;
    const int next = qn < nlist ? __ldg(list + qn) : 0;
    residual_c_voxel<SOLVER>(X, R, E, codes, g, q, lin, ctab);
    lin = next;
  }
}

// x += e at each fluid voxel and at the periodic halo copies the padded form
// keeps of it (the z copies that land on the planes holding reapplied
// pressure take no pressure correction), as dc_correct_voxel.
__global__ void k_dc_correct_c(Fields<double> X, const float4* __restrict__ E,
                               const int* __restrict__ list, int nlist, Grid g) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nlist; q += gridDim.x * blockDim.x)
    correct_c_voxel(X, __ldg(E + q), g, __ldg(list + q));
}

// Fluid mask words from the codes; base = number of list entries before the
// word's first voxel (binary search in the ascending lexicographic list).
// The word after the last row is a sentinel {0, nlist}.
__global__ void k_mask_words(const uint8_t* codes, Grid g, int nw, const int* list, int nlist,
                             uint2* words, long long nwords) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t <= nwords;
       t += (long long)gridDim.x * blockDim.x) {
    if (t == nwords) {
      words[t] = make_uint2(0u, (unsigned)nlist);
      continue;
    }
    const int w = (int)(t % nw);
    const long long row = t / nw;
    const int y = (int)(row % g.ny), z = (int)(row / g.ny);
    const int x0 = 32 * w;
    unsigned bits = 0;
    const uint8_t* rowc = codes + ((long long)(z + 2) * g.NY + (y + 2)) * g.pxc + 2;
    for (int b = 0; b < 32 && x0 + b < g.nx; ++b)
      if (rowc[x0 + b]) bits |= 1u << b;
    const long long lin0 = row * g.nx + x0;
    int lo = 0, hi = nlist;  // first entry >= lin0
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if ((long long)list[mid] < lin0) lo = mid + 1;
      else hi = mid;
    }
    words[t] = make_uint2(bits, (unsigned)lo);
  }
}

// Position of interior voxel (x, y, z) in the fluid list (a fluid voxel).
__device__ __forceinline__ int list_pos(const uint2* words, int nw, const Grid& g, int x, int y,
                                        int z) {
  return word_rank(words[((long long)z * g.ny + y) * nw + (x >> 5)], x);
}

// Slots and metadata of every list position (see CompactSlots).
__global__ void k_compact_slots(const uint8_t* codes, Grid g, int nw, const int* list, int nlist,
                                const uint2* words, int4* sa, int2* sb, unsigned* meta) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nlist; q += gridDim.x * blockDim.x) {
    int x, y, z;
    interior_xyz(list[q], g, x, y, z);
    const int code = codes[((long long)(z + 2) * g.NY + (y + 2)) * g.pxc + (x + 2)];
    int cs[3];
    decode_cases(code, cs[0], cs[1], cs[2]);
    const int c[3] = {x, y, z}, n[3] = {g.nx, g.ny, g.nz};
    int slot[6];
    for (int ax = 0; ax < 3; ++ax) {
      // the neighbour at offset d along ax, or the zero slot where the padded
      // store holds 0 there
      auto pos = [&](int d) {
        bool ok = true;
        int cc[3] = {x, y, z};
        cc[ax] = wrap(c[ax] + d, n[ax], g.per[ax], ok);
        return ok ? list_pos(words, nw, g, cc[0], cc[1], cc[2]) : nlist;
      };
      const int k = cs[ax];
      slot[2 * ax] = left_fluid(k) ? pos(-1) : (k == 4 ? pos(2) : nlist);
      slot[2 * ax + 1] = right_fluid(k) ? pos(1) : (k == 5 ? pos(-2) : nlist);
    }
    sa[q] = make_int4(slot[0], slot[1], slot[2], slot[3]);
    sb[q] = make_int2(slot[4], slot[5]);
    meta[q] = make_meta(cs[0], cs[1], cs[2], z == 0, z == g.nz - 1);
  }
}

// Packed records (kernel 13) from the slots and metadata.
__global__ void k_pack_records(const unsigned* __restrict__ meta, const int4* __restrict__ sa,
                               const int2* __restrict__ sb, int nlist, uint4* __restrict__ rec) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nlist; q += gridDim.x * blockDim.x) {
    const int4 a = sa[q];
    const int2 b = sb[q];
    unsigned d[6];
    bool ok = pack16(a.x, q, nlist, d[0]) & pack16(a.y, q, nlist, d[1]) &
              pack16(a.z, q, nlist, d[2]) & pack16(a.w, q, nlist, d[3]) &
              pack16(b.x, q, nlist, d[4]) & pack16(b.y, q, nlist, d[5]);
    rec[q] = ok ? make_uint4(meta[q], d[0] | d[1] << 16, d[2] | d[3] << 16, d[4] | d[5] << 16)
                : make_uint4(meta[q] | kMetaEscape, 0u, 0u, 0u);
  }
}

// The correction sweep over packed records (kernel 13): one 128-bit load of
// index data per position; an escaped position (a periodic face more than
// 32767 positions away) reads its full slots.  Persistent, no prefetch.
template <int SOLVER, int MINB>
__global__ void __launch_bounds__(256, MINB) k_dc_inner_cr(const float4* __restrict__ E,
                                                          float4* __restrict__ E2,
                                                          const float4* __restrict__ R,
                                                          const uint4* __restrict__ rec,
                                                          const int4* __restrict__ sa,
                                                          const int2* __restrict__ sb,
                                                          int nlist) {
  const int stride = gridDim.x * blockDim.x;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nlist; q += stride) {
    const uint4 r = __ldg(rec + q);
    CompactSlots sl;
    if (r.x & kMetaEscape) {
      sl.a = __ldg(sa + q);
      sl.b = __ldg(sb + q);
    } else {
      decode_record(r, q, nlist, sl);
    }
    inner_c_compute<SOLVER>(E, E2, R, q, r.x & ~kMetaEscape, sl);
  }
}

int grid_for(long long n, int threads, int cap) {
  long long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (int)b;
}

}  // namespace

long long compact_words(const Grid& g) {
  return (long long)g.nz * g.ny * ((g.nx + 31) / 32) + 1;
}

cudaError_t compact_setup(const uint8_t* codes, const Grid& g, const int* list, int nlist,
                          uint2* words, int4* sa, int2* sb, unsigned* meta, cudaStream_t st,
                          uint4* rec) {
  const int nw = (g.nx + 31) / 32;
  const long long nwords = compact_words(g) - 1;
  const int sms = sm_count();
  k_mask_words<<<grid_for(nwords + 1, 256, 16 * sms), 256, 0, st>>>(codes, g, nw, list, nlist,
                                                                    words, nwords);
  k_compact_slots<<<grid_for(nlist, 256, 16 * sms), 256, 0, st>>>(codes, g, nw, list, nlist,
                                                                   words, sa, sb, meta);
  count_launches(2);
  if (rec && nlist > 0) {
    k_pack_records<<<grid_for(nlist, 256, 16 * sms), 256, 0, st>>>(meta, sa, sb, nlist, rec);
    count_launches(1);
  }
  return cudaGetLastError();
}

cudaError_t launch_dc_inner_cr(const float4* e, float4* e2, const float4* r, const uint4* rec,
                               const int4* sa, const int2* sb, int nlist, int solver,
                               cudaStream_t st) {
  if (nlist < 1) return cudaSuccess;
  const int blocks = grid_for(nlist, 256, 5 * sm_count());
  if (solver == 1) k_dc_inner_cr<1, 5><<<blocks, 256, 0, st>>>(e, e2, r, rec, sa, sb, nlist);
  else if (solver == 2) k_dc_inner_cr<2, 5><<<blocks, 256, 0, st>>>(e, e2, r, rec, sa, sb, nlist);
  else k_dc_inner_cr<3, 5><<<blocks, 256, 0, st>>>(e, e2, r, rec, sa, sb, nlist);
  count_launches(1);
  return cudaGetLastError();
}

template <int MINB, bool PF>
static cudaError_t inner_c_launch(const float4* e, float4* e2, const float4* r,
                                  const unsigned* meta, const int4* sa, const int2* sb,
                                  int nlist, int solver, cudaStream_t st) {
  if (nlist < 1) return cudaSuccess;
  const int blocks = grid_for(nlist, 256, MINB * sm_count());
  if (solver == 1)
    k_dc_inner_c<1, MINB, PF><<<blocks, 256, 0, st>>>(e, e2, r, meta, sa, sb, nlist);
  else if (solver == 2)
    k_dc_inner_c<2, MINB, PF><<<blocks, 256, 0, st>>>(e, e2, r, meta, sa, sb, nlist);
  else
    k_dc_inner_c<3, MINB, PF><<<blocks, 256, 0, st>>>(e, e2, r, meta, sa, sb, nlist);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_dc_inner_c(const float4* e, float4* e2, const float4* r, const unsigned* meta,
                              const int4* sa, const int2* sb, int nlist, int solver, int minb,
                              cudaStream_t st) {
  if (minb <= 2) return inner_c_launch<2, true>(e, e2, r, meta, sa, sb, nlist, solver, st);
  if (minb == 3) return inner_c_launch<3, true>(e, e2, r, meta, sa, sb, nlist, solver, st);
  if (minb == 4) return inner_c_launch<4, true>(e, e2, r, meta, sa, sb, nlist, solver, st);
  return inner_c_launch<5, false>(e, e2, r, meta, sa, sb, nlist, solver, st);
}

// pm_debug_tma_fail: the next bulk-staged sweeps report a timed-out first wait.
static std::atomic<int> g_cb_fail{0};

void compact_debug_fail(int on) { g_cb_fail.store(on ? 1 : 0); }

template <int MINB>
static cudaError_t inner_cb_launch(const float4* e, float4* e2, const float4* r,
                                   const unsigned* meta, const int4* sa, const int2* sb,
                                   int nlist, int solver, int* err, cudaStream_t st) {
  const long long budget = 4000000000LL;  // ~2 s at 2 GHz per wait
  const int ff = g_cb_fail.load();
  const int blocks = grid_for(nlist, kChunk, MINB * sm_count());
  if (solver == 1)
    k_dc_inner_cb<1, MINB><<<blocks, kChunk, 0, st>>>(e, e2, r, meta, sa, sb, nlist, err,
                                                      budget, ff);
  else if (solver == 2)
    k_dc_inner_cb<2, MINB><<<blocks, kChunk, 0, st>>>(e, e2, r, meta, sa, sb, nlist, err,
                                                      budget, ff);
  else
    k_dc_inner_cb<3, MINB><<<blocks, kChunk, 0, st>>>(e, e2, r, meta, sa, sb, nlist, err,
                                                      budget, ff);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_dc_inner_cb(const float4* e, float4* e2, const float4* r,
                               const unsigned* meta, const int4* sa, const int2* sb, int nlist,
                               int solver, int minb, int* err, cudaStream_t st) {
  if (nlist < 1) return cudaSuccess;
  if (minb >= 5) return inner_cb_launch<5>(e, e2, r, meta, sa, sb, nlist, solver, err, st);
  return inner_cb_launch<4>(e, e2, r, meta, sa, sb, nlist, solver, err, st);
}

cudaError_t launch_dc_residual_c(Fields<double> x, float4* r, float4* e, const uint8_t* codes,
                                 const int* list, int nlist, const Grid& g, int solver,
                                 cudaStream_t st) {
  if (nlist < 1) return cudaSuccess;
  const int blocks = grid_for(nlist, 256, 2 * sm_count());
  if (solver == 1) k_dc_residual_c<1><<<blocks, 256, 0, st>>>(x, r, e, codes, list, nlist, g);
  else if (solver == 2) k_dc_residual_c<2><<<blocks, 256, 0, st>>>(x, r, e, codes, list, nlist, g);
  else k_dc_residual_c<3><<<blocks, 256, 0, st>>>(x, r, e, codes, list, nlist, g);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_dc_correct_c(Fields<double> x, const float4* e, const int* list, int nlist,
                                const Grid& g, cudaStream_t st) {
  if (nlist < 1) return cudaSuccess;
  k_dc_correct_c<<<(nlist + 255) / 256, 256, 0, st>>>(x, e, list, nlist, g);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace pm
