// Device functions of the compact correction store (pm_compact.cu): shared
// by the single-problem kernels and the batched kernels of the server, so a
// sample computes the same values alone and in a batch.
#pragma once

#include "pm_stencil.cuh"

namespace pm {

// Wrap a neighbour coordinate q = c + d (d in -2..2) on an axis of length n.
// The padded store's halo cell at q holds a copy of the interior voxel one
// period away when that voxel exists (periodic axis, q -+ n inside [0, n)),
// and 0 otherwise (wall axes, and the outer halo cell of an axis of length 1);
// ok becomes false where the padded store holds 0.
__device__ __forceinline__ int wrap(int q, int n, int per, bool& ok) {
  if (q < 0) {
    ok = ok && per && q + n >= 0;
    return q + n;
  }
  if (q >= n) {
    ok = ok && per && q - n < n;
    return q - n;
  }
  return q;
}

// Fluid flags from a neighbourhood case (1 = solid in the reference's
// geometry): left fluid for cases 3, 5, 6; right fluid for 2, 4, 6; the
// second left is used (and fluid) in case 5, the second right in case 4.
__device__ __forceinline__ bool left_fluid(int c) { return c == 3 || c == 5 || c == 6; }
__device__ __forceinline__ bool right_fluid(int c) { return c == 2 || c == 4 || c == 6; }

// The sweep of list position i reads its correction and six neighbour
// positions, two per axis, chosen by the axis' neighbourhood case when the
// compact store is set up:
//   case 1 (both sides solid)         L = zero slot, R = zero slot
//   case 2 (l solid, r fluid, rr solid)  L = zero slot, R = r
//   case 3 (ll solid, l fluid, r solid)  L = l,         R = zero slot
//   case 4 (l solid, r and rr fluid)  L = rr,        R = r
//   case 5 (ll and l fluid, r solid)  L = l,         R = ll
//   case 6 (both sides fluid)         L = l,         R = r
// (a neighbour that is fluid in the geometry but has no stored value -- a
// wall-face halo, the outer halo of an axis of length 1 -- is the zero slot
// too).  The zero slot is position nlist of every correction buffer, which
// holds 0 forever.  In a case-4 or case-5 axis one side is solid, so its slot
// carries the second neighbour the wall stencil needs: six slots cover all
// twelve stencil points.
struct CompactSlots {
  int4 a;  // x L, x R, y L, y R
  int2 b;  // z L, z R
};

// Per-voxel metadata (32 bits): the three neighbourhood cases (3 bits each,
// x in bits 0-2), two plane flags and which +-1 neighbours are fluid.
constexpr unsigned kMetaZFirst = 1u << 9;   // first interior plane: -z pressure reads 0
constexpr unsigned kMetaZLast = 1u << 10;   // last interior plane: own pressure reads 0
constexpr int kMetaFluidShift = 11;         // bits 11 + 2 axis (+1): -side (+side) fluid

__device__ __forceinline__ unsigned make_meta(int cx, int cy, int cz, bool zfirst, bool zlast);

__device__ __forceinline__ unsigned make_meta(int cx, int cy, int cz, bool zfirst, bool zlast) {
  unsigned m = (unsigned)cx | ((unsigned)cy << 3) | ((unsigned)cz << 6);
  if (zfirst) m |= kMetaZFirst;
  if (zlast) m |= kMetaZLast;
  const int c[3] = {cx, cy, cz};
  for (int a = 0; a < 3; ++a) {
    if (left_fluid(c[a])) m |= 1u << (kMetaFluidShift + 2 * a);
    if (right_fluid(c[a])) m |= 1u << (kMetaFluidShift + 2 * a + 1);
  }
  return m;
}

// Packed record of a list position (kernel 13): the metadata word and the six
// slots as signed 16-bit offsets from the position itself,
//   {meta, xL | xR << 16, yL | yR << 16, zL | zR << 16},
// with kZeroSlot16 for the zero slot.  A position whose slots do not all fit
// (an offset beyond +-32767: a periodic face more than one plane of fluid
// away, or planes of more than 32767 fluid voxels) has kMetaEscape set and
// reads its full slots instead.  16 bytes per position instead of 28.
constexpr unsigned kMetaEscape = 1u << 31;
constexpr int kZeroSlot16 = -32768;

__device__ __forceinline__ bool pack16(int slot, int q, int nlist, unsigned& out) {
  const int d = slot == nlist ? kZeroSlot16 : slot - q;
  if (slot != nlist && (d < -32767 || d > 32767)) return false;
  out = (unsigned)d & 0xFFFFu;
  return true;
}

__device__ __forceinline__ int unpack16(unsigned w, int hi, int q, int nlist) {
  const int d = hi ? ((int)w >> 16) : ((int)(w << 16) >> 16);
  return d == kZeroSlot16 ? nlist : q + d;
}

__device__ __forceinline__ void decode_record(uint4 rec, int q, int nlist, CompactSlots& sl) {
  sl.a = make_int4(unpack16(rec.y, 0, q, nlist), unpack16(rec.y, 1, q, nlist),
                   unpack16(rec.z, 0, q, nlist), unpack16(rec.z, 1, q, nlist));
  sl.b = make_int2(unpack16(rec.w, 0, q, nlist), unpack16(rec.w, 1, q, nlist));
}

__device__ __forceinline__ int word_rank(uint2 w, int x) {
  return (int)w.y + __popc(w.x & ((1u << (x & 31)) - 1u));
}

__device__ __forceinline__ void interior_xyz(int lin, const Grid& g, int& x, int& y, int& z) {
  lin_to_xyz(lin, g, x, y, z);
  x -= 2;
  y -= 2;
  z -= 2;
}

// Loads of the correction and residual.  COHERENT: they were written earlier
// in the same launch by another CTA (the persistent round kernel of the
// server), so they bypass L1 (ld.global.cg); otherwise the read-only path.
template <bool COHERENT>
__device__ __forceinline__ float4 ld_corr(const float4* p) {
  return COHERENT ? __ldcg(p) : __ldg(p);
}

// e2 = L(e) + r for list position i.
template <int SOLVER, bool COHERENT = false>
__device__ __forceinline__ void inner_c_compute(const float4* __restrict__ E,
                                                float4* __restrict__ E2,
                                                const float4* __restrict__ R, int i,
                                                unsigned meta, const CompactSlots& sl) {
  const int cx = (int)(meta & 7u), cy = (int)((meta >> 3) & 7u), cz = (int)((meta >> 6) & 7u);
  auto fl = [&](int axis, int side) { return (meta >> (kMetaFluidShift + 2 * axis + side)) & 1u; };
  const float4 C = ld_corr<COHERENT>(E + i);
  const float4 XL = ld_corr<COHERENT>(E + sl.a.x), XR = ld_corr<COHERENT>(E + sl.a.y);
  const float4 YL = ld_corr<COHERENT>(E + sl.a.z), YR = ld_corr<COHERENT>(E + sl.a.w);
  const float4 ZL = ld_corr<COHERENT>(E + sl.b.x), ZR = ld_corr<COHERENT>(E + sl.b.y);
  const float4 r = ld_corr<COHERENT>(R + i);
  Stencil<float> s;
  // along-axis terms and the divergence read the true +-1 neighbours (0 where
  // solid; in cases 4 / 5 the solid side's slot holds the second neighbour);
  // the wall stencils across an axis take (ll, l, r, rr) = (R, L, R, L),
  // which case_pick resolves to exactly the points each case uses
  s.uc = C.x;
  s.uxm = fl(0, 0) ? XL.x : 0.f;
  s.uxp = fl(0, 1) ? XR.x : 0.f;
  s.uymm = YR.x; s.uym = YL.x; s.uyp = YR.x; s.uypp = YL.x;
  s.uzmm = ZR.x; s.uzm = ZL.x; s.uzp = ZR.x; s.uzpp = ZL.x;
  s.vc = C.y;
  s.vym = fl(1, 0) ? YL.y : 0.f;
  s.vyp = fl(1, 1) ? YR.y : 0.f;
  s.vxmm = XR.y; s.vxm = XL.y; s.vxp = XR.y; s.vxpp = XL.y;
  s.vzmm = ZR.y; s.vzm = ZL.y; s.vzp = ZR.y; s.vzpp = ZL.y;
  s.wc = C.z;
  s.wzm = fl(2, 0) ? ZL.z : 0.f;
  s.wzp = fl(2, 1) ? ZR.z : 0.f;
  s.wxmm = XR.z; s.wxm = XL.z; s.wxp = XR.z; s.wxpp = XL.z;
  s.wymm = YR.z; s.wym = YL.z; s.wyp = YR.z; s.wypp = YL.z;
  // a pressure difference is taken only where the -side neighbour is fluid,
  // and then its slot holds it; the plane flags carry the reapplied pressure
  // (correction 0) of the last interior plane and of the z halo below the first
  s.pc = (meta & kMetaZLast) ? 0.f : C.w;
  s.pxm = XL.w;
  s.pym = YL.w;
  s.pzm = (meta & kMetaZFirst) ? 0.f : ZL.w;
  float un, vn, wn, pn;
  update_fast_cases<float, SOLVER>(s, cx, cy, cz, un, vn, wn, pn);
  E2[i] = make_float4(un + r.x, vn + r.y, wn + r.z, pn + r.w);
}

// One voxel of the batched kernels.
template <int SOLVER, bool COHERENT = false>
__device__ __forceinline__ void inner_c_voxel(const float4* __restrict__ E,
                                              float4* __restrict__ E2,
                                              const float4* __restrict__ R,
                                              const unsigned* __restrict__ meta,
                                              const int4* __restrict__ sa,
                                              const int2* __restrict__ sb, int i) {
  CompactSlots sl;
  sl.a = __ldg(sa + i);
  sl.b = __ldg(sb + i);
  inner_c_compute<SOLVER, COHERENT>(E, E2, R, i, __ldg(meta + i), sl);
}

// r = F(x) - x in FP64 from the padded state (as dc_residual_voxel), stored
// at list position q, and e1 = r.
template <int SOLVER>
__device__ __forceinline__ void residual_c_voxel(const Fields<double>& X, float4* R, float4* E,
                                                 const uint8_t* codes, const Grid& g, int q,
                                                 int lin, const double* ctab = nullptr) {
  int x, y, z;
  lin_to_xyz(lin, g, x, y, z);
  const int code = codes[((long long)z * g.NY + y) * g.pxc + x];
  const long long c = (long long)z * g.pl64 + (long long)y * g.px64 + x;
  Stencil<double> s;
  gather<double, 0>(s, X, X, c, x, y, z, g, g.px64, g.pl64);
  double un, vn, wn, pn;
  update_fast<double, SOLVER>(s, code, un, vn, wn, pn, ctab);
  const double pstored = (z == g.NZ - 3) ? __ldg(X.p + c) : s.pc;
  const float4 rv = make_float4((float)(un - s.uc), (float)(vn - s.vc), (float)(wn - s.wc),
                                (float)(pn - pstored));
  R[q] = rv;
  E[q] = rv;
}

// x += e at a fluid voxel and at the periodic halo copies the padded form
// keeps of it (the z copies that land on the planes holding reapplied
// pressure take no pressure correction), as dc_correct_voxel.
__device__ __forceinline__ void correct_c_voxel(const Fields<double>& X, float4 e, const Grid& g,
                                                int lin) {
  int x, y, z;
  lin_to_xyz(lin, g, x, y, z);
  auto add = [&](int xx, int yy, int zz, bool pz) {
    const long long c = (long long)zz * g.pl64 + (long long)yy * g.px64 + xx;
    X.u[c] += (double)e.x;
    X.v[c] += (double)e.y;
    X.w[c] += (double)e.z;
    X.p[c] += pz ? 0.0 : (double)e.w;
  };
  add(x, y, z, false);
  if (g.per[0]) {
    if (x < 4) add(x + g.nx, y, z, false);
    if (x >= g.nx) add(x - g.nx, y, z, false);
  }
  if (g.per[1]) {
    if (y < 4) add(x, y + g.ny, z, false);
    if (y >= g.ny) add(x, y - g.ny, z, false);
  }
  if (g.per[2]) {
    if (z < 4) add(x, y, z + g.nz, z == 2);
    if (z >= g.nz) add(x, y, z - g.nz, z == g.nz + 1);
  }
}

}  // namespace pm
