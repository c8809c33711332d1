// Per-voxel update of the pseudo-time Stokes sweep (the body of
// central_diff5, src/solver.cc:136-220 of the reference) in two arithmetic
// forms:
//   * update_exact: the reference's operation order term by term (translation
//     units that use it are compiled with -fmad=false), bit-identical to the
//     reference CPU program;
//   * update_fast: the same linear map regrouped into a coefficient form with
//     FMAs (31 FP64 instructions per fluid voxel in FP64, where the relaxation
//     is folded into the coefficients and the centre coefficient comes from a
//     16-entry table; about 39 in FP32; instead of ~70 plus three divisions),
//     used by the FP64 fast sweeps, the FP64 residual and the FP32 correction
//     sweeps of the mixed-precision form.
#pragma once

#include "pm_internal.h"

namespace pm {

// Values of the 4 fields a fluid voxel reads (axis-aligned offsets only).
template <typename T>
struct Stencil {
  T uc, uxm, uxp, uym, uyp, uymm, uypp, uzm, uzp, uzmm, uzpp;
  T vc, vxm, vxp, vxmm, vxpp, vym, vyp, vzm, vzp, vzmm, vzpp;
  T wc, wxm, wxp, wxmm, wxpp, wym, wyp, wymm, wypp, wzm, wzp;
  T pc, pxm, pym, pzm;
};

// code byte 1..216 -> neighbourhood cases (cx, cy, cz) in 1..6 (the
// split_number of src/solver.cc:94-109 applied to 100cx + 10cy + cz).
__device__ __forceinline__ void decode_cases(int code, int& cx, int& cy, int& cz) {
  int c = code - 1;
  int a = c / 36;
  int rem = c - a * 36;
  int b = rem / 6;
  cx = a + 1;
  cy = b + 1;
  cz = rem - b * 6 + 1;
}

// The left neighbour along an axis is solid exactly for cases 1, 2 and 4 of
// eval_geometry (src/geometry.cc:273-296).
__device__ __forceinline__ bool left_solid(int cs) { return cs == 1 || cs == 2 || cs == 4; }

// get_2nd_derivation, src/solver.cc:57-91, operand order preserved.
__device__ __forceinline__ double d2_exact(int cs, double ll, double l, double m, double r,
                                           double rr) {
  double d = 0.0;
  if (cs == 1) d = -8.0 * m;
  else if (cs == 2) d = 8.0 / 3.0 * r - 16.0 / 3.0 * m;
  else if (cs == 3) d = 8.0 / 3.0 * l - 16.0 / 3.0 * m;
  else if (cs == 4) d = 2.0 * r - 5.0 * m - 1.0 / 5.0 * rr;
  else if (cs == 5) d = 2.0 * l - 1.0 / 5.0 * ll - 5.0 * m;
  else if (cs == 6) d = l - 2.0 * m + r;
  return d;
}

// central_diff5 body (src/solver.cc:142-219) for one fluid voxel.
template <int SOLVER>
__device__ __forceinline__ void update_exact(const Stencil<double>& s, int code, double& un,
                                             double& vn, double& wn, double& pn) {
  int cx, cy, cz;
  decode_cases(code, cx, cy, cz);
  const bool lx = left_solid(cx), ly = left_solid(cy), lz = left_solid(cz);
  double dp_dz = lz ? 0. : -s.pzm + s.pc;
  double dp_dy = ly ? 0. : -s.pym + s.pc;
  double dp_dx = lx ? 0. : -s.pxm + s.pc;
  double uxx = (s.uxm - 2 * s.uc + s.uxp);
  double vyy = (s.vym - 2 * s.vc + s.vyp);
  double wzz = (s.wzm - 2 * s.wc + s.wzp);
  double vxx = d2_exact(cx, s.vxmm, s.vxm, s.vc, s.vxp, s.vxpp);
  double wxx = d2_exact(cx, s.wxmm, s.wxm, s.wc, s.wxp, s.wxpp);
  double uyy = d2_exact(cy, s.uymm, s.uym, s.uc, s.uyp, s.uypp);
  double wyy = d2_exact(cy, s.wymm, s.wym, s.wc, s.wyp, s.wypp);
  double uzz = d2_exact(cz, s.uzmm, s.uzm, s.uc, s.uzp, s.uzpp);
  double vzz = d2_exact(cz, s.vzmm, s.vzm, s.vc, s.vzp, s.vzpp);
  double fu = uxx + uyy + uzz;
  double fv = vyy + vzz + vxx;
  double fw = wzz + wxx + wyy;
  double v_sum = 0.0;
  if (SOLVER == 1) v_sum = (s.wzp - s.wc + s.vyp - s.vc + s.uxp - s.uc);
  if (SOLVER == 1 || SOLVER == 2) {
    un = lx ? 0.0 : s.uc + (-dp_dx + fu / kRe) * kDt;
    vn = ly ? 0.0 : s.vc + (-dp_dy + fv / kRe) * kDt;
    wn = lz ? 0.0 : s.wc + (-dp_dz + fw / kRe) * kDt;
  } else {
    un = (1.0 - kOmega) * s.uc + kOmega * (-dp_dx + fu / kRe) * kDt;
    vn = (1.0 - kOmega) * s.vc + kOmega * (-dp_dy + fv / kRe) * kDt;
    wn = (1.0 - kOmega) * s.wc + kOmega * (-dp_dz + fw / kRe) * kDt;
  }
  if (SOLVER == 2 || SOLVER == 3) v_sum = (s.wzp - wn + s.vyp - vn + s.uxp - un);
  pn = s.pc - kC2 * v_sum * kDt;
}

// Coefficient form.  Each wall-aware stencil of case cs is
//   a(cs) * centre + cA(cs) * A + cB(cs) * B
// with A, B the (at most two) off-centre points it uses.
template <typename T>
struct CaseCoef {
  T a, cA, cB;
};

// Coefficients per case: 1 (-8, 0, 0); 2, 3 (-16/3, 8/3, 0); 4, 5 (-5, 2, -0.2);
// 6 (-2, 1, 1).  In FP32 as selects on three comparisons (no branches; the
// FP32 correction sweep measured 20.5 us against 22.6 us with a switch on the
// 128^3 sphere pack); in FP64 as a switch (the FP64 Jacobi sweep measured
// 68 us against 76 us with selects, which cost register pairs).
template <typename T>
__device__ __forceinline__ CaseCoef<T> case_coef(int cs) {
  CaseCoef<T> k;
  if (sizeof(T) == 8) {
    switch (cs) {
      case 1: k.a = T(-8.0); k.cA = T(0.0); k.cB = T(0.0); break;
      case 2: case 3: k.a = T(-16.0 / 3.0); k.cA = T(8.0 / 3.0); k.cB = T(0.0); break;
      case 4: case 5: k.a = T(-5.0); k.cA = T(2.0); k.cB = T(-0.2); break;
      default: k.a = T(-2.0); k.cA = T(1.0); k.cB = T(1.0); break;
    }
    return k;
  }
  const bool c1 = cs == 1, le3 = cs <= 3, le5 = cs <= 5;
  k.a = c1 ? T(-8.0) : (le3 ? T(-16.0 / 3.0) : (le5 ? T(-5.0) : T(-2.0)));
  k.cA = c1 ? T(0.0) : (le3 ? T(8.0 / 3.0) : (le5 ? T(2.0) : T(1.0)));
  k.cB = le3 ? T(0.0) : (le5 ? T(-0.2) : T(1.0));
  return k;
}

// A = left for cases 3, 5, 6, else right; B = second right (4), second left
// (5), right (6); unused (coefficient 0) otherwise.
template <typename T>
__device__ __forceinline__ void case_pick(int cs, T ll, T l, T r, T rr, T& A, T& B) {
  A = (cs == 3 || cs == 5 || cs == 6) ? l : r;
  B = cs == 4 ? rr : (cs == 5 ? ll : r);
}

// One velocity component: the along-axis 3-point term plus two cross-axis
// wall stencils, the pressure difference, and the solver's relaxation.
// Group of a case by its centre coefficient a: 1 -> 0, 2/3 -> 1, 4/5 -> 2, 6 -> 3.
__device__ __forceinline__ int case_group(int cs) {
  return cs == 1 ? 0 : (cs <= 3 ? 1 : (cs <= 5 ? 2 : 3));
}

// Centre coefficient a of a case group (the FP64 form's centre table is built
// from it: see centre64).
__device__ __forceinline__ double group_a(int g) {
  return g == 0 ? -8.0 : (g == 1 ? -16.0 / 3.0 : (g == 2 ? -5.0 : -2.0));
}

// FP64 form: the relaxation of the solver is folded into the coefficients,
// so a new velocity is one FMA chain over its nine stencil values
//   v' = Cc c + K' (am + ap + cA1 A1 + cB1 B1 + cA2 A2 + cB2 B2) - dt' (pc - pm)
// with K' = dt/Re, dt' = dt (solvers 1, 2) or K' = omega dt/Re, dt' = omega dt
// (solver 3, whose update is (1 - omega) c + omega dt (-dp + f/Re)), and the
// centre coefficient Cc = 1 + K' ctr (solvers 1, 2) or (1 - omega) + K' ctr
// (solver 3), ctr = -2 + a1 + a2.  -dt' pc is shared by the three velocities.
// 31 FP64 instructions per fluid voxel instead of 36 (SOR) / 33: GB300's
// FP64 pipe (1/64 of the FP32 rate) bounds the FP64 sweeps.
template <int SOLVER>
struct Relax64 {
  static constexpr double K = SOLVER == 3 ? kDt / kRe * kOmega : kDt / kRe;
  static constexpr double Dt = SOLVER == 3 ? kDt * kOmega : kDt;
  static constexpr double Base = SOLVER == 3 ? 1.0 - kOmega : 1.0;
};

template <int SOLVER>
__device__ __forceinline__ double centre64(int g1, int g2) {
  const double ctr = (-2.0 + group_a(g1)) + group_a(g2);
  return __fma_rn(Relax64<SOLVER>::K, ctr, Relax64<SOLVER>::Base);
}

template <int SOLVER>
__device__ __forceinline__ void fill_centre_table(double* tab) {
  for (int i = threadIdx.x; i < 16; i += blockDim.x) tab[i] = centre64<SOLVER>(i >> 2, i & 3);
}

// Off-centre coefficients of a wall stencil of case cs times K' (see case_coef).
template <int SOLVER>
__device__ __forceinline__ void case_coef64(int cs, double& cA, double& cB) {
  constexpr double K = Relax64<SOLVER>::K;
  switch (cs) {
    case 1: cA = 0.0; cB = 0.0; break;
    case 2: case 3: cA = K * (8.0 / 3.0); cB = 0.0; break;
    case 4: case 5: cA = K * 2.0; cB = K * -0.2; break;
    default: cA = K; cB = K; break;
  }
}

template <int SOLVER>
__device__ __forceinline__ double vel64(double c, double am, double ap, int cs1, double ll1,
                                        double l1, double r1, double rr1, int cs2, double ll2,
                                        double l2, double r2, double rr2, double pm, double P,
                                        bool lsolid, const double* ctab) {
  double cA1, cB1, cA2, cB2, A1, B1, A2, B2;
  case_coef64<SOLVER>(cs1, cA1, cB1);
  case_coef64<SOLVER>(cs2, cA2, cB2);
  case_pick<double>(cs1, ll1, l1, r1, rr1, A1, B1);
  case_pick<double>(cs2, ll2, l2, r2, rr2, A2, B2);
  constexpr double K = Relax64<SOLVER>::K;
  const double Cc = ctab ? ctab[case_group(cs1) * 4 + case_group(cs2)]
                         : centre64<SOLVER>(case_group(cs1), case_group(cs2));
  // no pressure difference where the left neighbour is solid
  double t = lsolid ? 0.0 : fma(Relax64<SOLVER>::Dt, pm, P);
  t = fma(Cc, c, t);
  t = fma(K, am, t);
  t = fma(K, ap, t);
  t = fma(cA1, A1, t);
  t = fma(cB1, B1, t);
  t = fma(cA2, A2, t);
  t = fma(cB2, B2, t);
  return (SOLVER != 3 && lsolid) ? 0.0 : t;
}

template <typename T, int SOLVER>
__device__ __forceinline__ T vel_fast(T c, T am, T ap, int cs1, T ll1, T l1, T r1, T rr1, int cs2,
                                      T ll2, T l2, T r2, T rr2, T dp, bool zero,
                                      const T* ctab = nullptr) {
  const CaseCoef<T> k1 = case_coef<T>(cs1), k2 = case_coef<T>(cs2);
  T A1, B1, A2, B2;
  case_pick<T>(cs1, ll1, l1, r1, rr1, A1, B1);
  case_pick<T>(cs2, ll2, l2, r2, rr2, A2, B2);
  T f = am + ap;
  f = fma(k1.cA, A1, f);
  f = fma(k1.cB, B1, f);
  f = fma(k2.cA, A2, f);
  f = fma(k2.cB, B2, f);
  const T centre = ctab ? ctab[case_group(cs1) * 4 + case_group(cs2)]
                        : T(-2.0) + k1.a + k2.a;  // centre coefficient (exact small sums)
  f = fma(centre, c, f);
  const T K = T(kDt / kRe);
  if (SOLVER == 3) {
    // (1 - w) c + w (-dp + f / Re) dt
    T t = fma(T(kDt / kRe * kOmega), f, T(1.0 - kOmega) * c);
    return fma(T(-kDt * kOmega), dp, t);
  }
  T t = fma(K, f, c);
  t = fma(T(-kDt), dp, t);
  return zero ? T(0.0) : t;
}

template <typename T, int SOLVER>
__device__ __forceinline__ void update_fast_cases(const Stencil<T>& s, int cx, int cy, int cz,
                                                  T& un, T& vn, T& wn, T& pn,
                                                  const T* ctab = nullptr) {
  const bool lx = left_solid(cx), ly = left_solid(cy), lz = left_solid(cz);
  if constexpr (sizeof(T) == 8) {
    const double P = -Relax64<SOLVER>::Dt * s.pc;
    double d0 = 0.0;
    if (SOLVER == 1) d0 = ((s.wzp - s.wc) + (s.vyp - s.vc)) + (s.uxp - s.uc);
    un = vel64<SOLVER>(s.uc, s.uxm, s.uxp, cy, s.uymm, s.uym, s.uyp, s.uypp, cz, s.uzmm, s.uzm,
                       s.uzp, s.uzpp, s.pxm, P, lx, ctab);
    vn = vel64<SOLVER>(s.vc, s.vym, s.vyp, cx, s.vxmm, s.vxm, s.vxp, s.vxpp, cz, s.vzmm, s.vzm,
                       s.vzp, s.vzpp, s.pym, P, ly, ctab);
    wn = vel64<SOLVER>(s.wc, s.wzm, s.wzp, cx, s.wxmm, s.wxm, s.wxp, s.wxpp, cy, s.wymm, s.wym,
                       s.wyp, s.wypp, s.pzm, P, lz, ctab);
    const double dv = (SOLVER == 1) ? d0 : ((s.wzp - wn) + (s.vyp - vn)) + (s.uxp - un);
    pn = fma(-kC2 * kDt, dv, s.pc);
    return;
  }
  const T dpx = lx ? T(0) : s.pc - s.pxm;
  const T dpy = ly ? T(0) : s.pc - s.pym;
  const T dpz = lz ? T(0) : s.pc - s.pzm;
  T div0 = T(0);
  if (SOLVER == 1) div0 = ((s.wzp - s.wc) + (s.vyp - s.vc)) + (s.uxp - s.uc);
  // u: along x, cross y (cy) and z (cz)
  un = vel_fast<T, SOLVER>(s.uc, s.uxm, s.uxp, cy, s.uymm, s.uym, s.uyp, s.uypp, cz, s.uzmm,
                           s.uzm, s.uzp, s.uzpp, dpx, lx, ctab);
  // v: along y, cross x (cx) and z (cz)
  vn = vel_fast<T, SOLVER>(s.vc, s.vym, s.vyp, cx, s.vxmm, s.vxm, s.vxp, s.vxpp, cz, s.vzmm,
                           s.vzm, s.vzp, s.vzpp, dpy, ly, ctab);
  // w: along z, cross x (cx) and y (cy)
  wn = vel_fast<T, SOLVER>(s.wc, s.wzm, s.wzp, cx, s.wxmm, s.wxm, s.wxp, s.wxpp, cy, s.wymm,
                           s.wym, s.wyp, s.wypp, dpz, lz, ctab);
  T div = (SOLVER == 1) ? div0 : ((s.wzp - wn) + (s.vyp - vn)) + (s.uxp - un);
  pn = fma(T(-kC2 * kDt), div, s.pc);
}

template <typename T, int SOLVER>
__device__ __forceinline__ void update_fast(const Stencil<T>& s, int code, T& un, T& vn, T& wn,
                                            T& pn, const T* ctab = nullptr) {
  int cx, cy, cz;
  decode_cases(code, cx, cy, cz);
  update_fast_cases<T, SOLVER>(s, cx, cy, cz, un, vn, wn, pn, ctab);
}

// Gather of the stencil values of one interior voxel.
template <typename T>
__device__ __forceinline__ T ldA(const T* p, bool nc) {
  return nc ? __ldg(p) : __ldcg(p);
}

// P3 selects how the centre pressure of a voxel on the last interior plane
// (z = NZ-3) is read.  The out-of-place orderings store the swept,
// pre-reapply pressure there (their -x/-y neighbours on that plane must see it,
// as in the reference's in-place order, boundary_conditions.cc:46-79 runs only
// after the sweep) and imply the reapplied value 3 for the voxel itself:
//   0: stored value (in-place reference order, explicit reapply)
//   1: 3 (FP64 state)         2: 0 (homogeneous correction of the mixed form)
template <typename T, int PHASE, bool NC = true, int P3 = 1>
__device__ __forceinline__ void gather(Stencil<T>& s, const Fields<T>& A, const Fields<T>& B,
                                       long long c, int x, int y, int z, const Grid& g,
                                       long long px, long long pl) {
  const long long sx = 1, sy = px, sz = pl;
  // PHASE 2 (black): interior +-1 neighbours are red and already updated (in
  // B); every other read (centre, +-2, halos) is the previous iterate (A).
  // (one load from a selected base: the red values this pass reads from B are
  // not written by it)
  auto P = [&](const T* a, const T* b, long long o, bool interior) -> T {
    if (PHASE == 2) return ldA((interior ? b : a) + c + o, NC);
    return ldA(a + c + o, NC);
  };
  const bool ixm = x - 1 >= 2, ixp = x + 1 <= g.NX - 3;
  const bool iym = y - 1 >= 2, iyp = y + 1 <= g.NY - 3;
  const bool izm = z - 1 >= 2, izp = z + 1 <= g.NZ - 3;
  s.uc = ldA(A.u + c, NC);
  s.vc = ldA(A.v + c, NC);
  s.wc = ldA(A.w + c, NC);
  s.pc = (P3 != 0 && z == g.NZ - 3) ? T(P3 == 1 ? 3.0 : 0.0) : ldA(A.p + c, NC);
  s.uxm = P(A.u, B.u, -sx, ixm); s.uxp = P(A.u, B.u, sx, ixp);
  s.uym = P(A.u, B.u, -sy, iym); s.uyp = P(A.u, B.u, sy, iyp);
  s.uzm = P(A.u, B.u, -sz, izm); s.uzp = P(A.u, B.u, sz, izp);
  s.uymm = ldA(A.u + c - 2 * sy, NC); s.uypp = ldA(A.u + c + 2 * sy, NC);
  s.uzmm = ldA(A.u + c - 2 * sz, NC); s.uzpp = ldA(A.u + c + 2 * sz, NC);
  s.vxm = P(A.v, B.v, -sx, ixm); s.vxp = P(A.v, B.v, sx, ixp);
  s.vym = P(A.v, B.v, -sy, iym); s.vyp = P(A.v, B.v, sy, iyp);
  s.vzm = P(A.v, B.v, -sz, izm); s.vzp = P(A.v, B.v, sz, izp);
  s.vxmm = ldA(A.v + c - 2 * sx, NC); s.vxpp = ldA(A.v + c + 2 * sx, NC);
  s.vzmm = ldA(A.v + c - 2 * sz, NC); s.vzpp = ldA(A.v + c + 2 * sz, NC);
  s.wxm = P(A.w, B.w, -sx, ixm); s.wxp = P(A.w, B.w, sx, ixp);
  s.wym = P(A.w, B.w, -sy, iym); s.wyp = P(A.w, B.w, sy, iyp);
  s.wzm = P(A.w, B.w, -sz, izm); s.wzp = P(A.w, B.w, sz, izp);
  s.wxmm = ldA(A.w + c - 2 * sx, NC); s.wxpp = ldA(A.w + c + 2 * sx, NC);
  s.wymm = ldA(A.w + c - 2 * sy, NC); s.wypp = ldA(A.w + c + 2 * sy, NC);
  s.pxm = P(A.p, B.p, -sx, ixm);
  s.pym = P(A.p, B.p, -sy, iym);
  s.pzm = P(A.p, B.p, -sz, izm);
}

// Write the new values of interior voxel (x, y, z) and, on periodic axes,
// its halo copies (the halo exchange fused into the sweep).  The pressure
// reapply is fused too: the z-halo copies on planes 1 and NZ-2 hold nz+2 and 2
// (their geometry is this fluid voxel); x/y halo copies and the last interior
// plane keep the swept, pre-reapply value, as the reference's
// exchange-then-reapply order leaves the halos (the 3 of the last plane is
// implied, see gather).  HOMOG (correction sweeps of the mixed form) writes 0
// where the reapply writes a constant.
template <typename T, bool HOMOG>
__device__ __forceinline__ void write_voxel(const Fields<T>& B, long long c, int x, int y, int z,
                                            const Grid& g, long long px, long long pl, T un,
                                            T vn, T wn, T pn) {
  const T pin = HOMOG ? T(0) : T(g.nz + 2), pout = HOMOG ? T(0) : T(2.0);
  B.u[c] = un;
  B.v[c] = vn;
  B.w[c] = wn;
  B.p[c] = pn;  // last interior plane: swept value stored, reapplied 3 implied
  auto put = [&](long long o, T pv) {
    B.u[c + o] = un; B.v[c + o] = vn; B.w[c + o] = wn; B.p[c + o] = pv;
  };
  if (g.per[0]) {
    if (x < 4) put((long long)g.nx, pn);
    if (x >= g.nx) put(-(long long)g.nx, pn);
  }
  if (g.per[1]) {
    if (y < 4) put((long long)g.ny * px, pn);
    if (y >= g.ny) put(-(long long)g.ny * px, pn);
  }
  if (g.per[2]) {
    if (z < 4) put((long long)g.nz * pl, z == 2 ? pout : pn);
    if (z >= g.nz) put(-(long long)g.nz * pl, z == g.nz + 1 ? pin : pn);
  }
}


// ------------------------------------------------------------------ per-voxel bodies
// Shared by the single-problem kernels and the batched (many-sample) kernels,
// so a sample computes exactly the same values alone and in a batch.

// Interior linear index (x fastest) -> padded coordinates.
__device__ __forceinline__ unsigned div_magic(unsigned n, unsigned long long m, int s) {
  return (unsigned)(((unsigned long long)n * m) >> (32 + s));
}

__device__ __forceinline__ void lin_to_xyz(int lin, const Grid& g, int& x, int& y, int& z) {
  const unsigned r = div_magic((unsigned)lin, g.mnx, g.snx);  // lin / nx
  const unsigned zz = div_magic(r, g.mny, g.sny);             // r / ny
  x = lin - (int)r * g.nx + 2;
  y = (int)r - (int)zz * g.ny + 2;
  z = (int)zz + 2;
}

// One voxel of an FP64 sweep (Jacobi phase 0, red 1, black 2) from A into B.
template <int SOLVER, int PHASE, bool EXACT>
__device__ __forceinline__ void sweep64_voxel(const Fields<double>& A, const Fields<double>& B,
                                              const uint8_t* codes, const Grid& g, int lin,
                                              const double* ctab = nullptr) {
  int x, y, z;
  lin_to_xyz(lin, g, x, y, z);
  if (PHASE && (((x + y + z) & 1) != PHASE - 1)) return;  // (x+y+z) - 6 has the same parity
  const long long px = g.px64, pl = g.pl64;
  int code = codes[((long long)z * g.NY + y) * g.pxc + x];
  long long c = (long long)z * pl + (long long)y * px + x;
  Stencil<double> s;
  gather<double, PHASE>(s, A, B, c, x, y, z, g, px, pl);
  double un, vn, wn, pn;
  if (EXACT) update_exact<SOLVER>(s, code, un, vn, wn, pn);
  else update_fast<double, SOLVER>(s, code, un, vn, wn, pn, ctab);
  write_voxel<double, false>(B, c, x, y, z, g, px, pl, un, vn, wn, pn);
}

// ---- interleaved FP32 correction fields (float4 u, v, w, p per voxel)

// The stencil of one voxel from the correction: the union of its offsets is
// 13 points, each one 128-bit load.  The voxel's own pressure on the last
// interior plane is the reapplied (fixed) value, whose correction is 0.
__device__ __forceinline__ void gather4(Stencil<float>& s, const float4* E, long long c, int z,
                                        const Grid& g) {
  const long long px = g.px4, pl = g.pl4;
  const float4 C = __ldg(E + c);
  const float4 XM = __ldg(E + c - 1), XP = __ldg(E + c + 1);
  const float4 XMM = __ldg(E + c - 2), XPP = __ldg(E + c + 2);
  const float4 YM = __ldg(E + c - px), YP = __ldg(E + c + px);
  const float4 YMM = __ldg(E + c - 2 * px), YPP = __ldg(E + c + 2 * px);
  const float4 ZM = __ldg(E + c - pl), ZP = __ldg(E + c + pl);
  const float4 ZMM = __ldg(E + c - 2 * pl), ZPP = __ldg(E + c + 2 * pl);
  s.uc = C.x; s.uxm = XM.x; s.uxp = XP.x; s.uym = YM.x; s.uyp = YP.x;
  s.uymm = YMM.x; s.uypp = YPP.x; s.uzm = ZM.x; s.uzp = ZP.x; s.uzmm = ZMM.x; s.uzpp = ZPP.x;
  s.vc = C.y; s.vxm = XM.y; s.vxp = XP.y; s.vxmm = XMM.y; s.vxpp = XPP.y; s.vym = YM.y;
  s.vyp = YP.y; s.vzm = ZM.y; s.vzp = ZP.y; s.vzmm = ZMM.y; s.vzpp = ZPP.y;
  s.wc = C.z; s.wxm = XM.z; s.wxp = XP.z; s.wxmm = XMM.z; s.wxpp = XPP.z; s.wym = YM.z;
  s.wyp = YP.z; s.wymm = YMM.z; s.wypp = YPP.z; s.wzm = ZM.z; s.wzp = ZP.z;
  s.pc = (z == g.NZ - 3) ? 0.f : C.w;
  s.pxm = XM.w; s.pym = YM.w; s.pzm = ZM.w;
}

// write_voxel for the interleaved correction (homogeneous boundary values).
__device__ __forceinline__ void write_voxel4(float4* B, long long c, int x, int y, int z,
                                             const Grid& g, float un, float vn, float wn,
                                             float pn) {
  const long long px = g.px4, pl = g.pl4;
  const float4 val = make_float4(un, vn, wn, pn);
  B[c] = val;
  if (g.per[0]) {
    if (x < 4) B[c + g.nx] = val;
    if (x >= g.nx) B[c - g.nx] = val;
  }
  if (g.per[1]) {
    if (y < 4) B[c + (long long)g.ny * px] = val;
    if (y >= g.ny) B[c - (long long)g.ny * px] = val;
  }
  if (g.per[2]) {
    // the z copies landing on planes NZ-2 and 1 hold reapplied pressure: 0
    if (z < 4) B[c + (long long)g.nz * pl] = make_float4(un, vn, wn, z == 2 ? 0.f : pn);
    if (z >= g.nz)
      B[c - (long long)g.nz * pl] = make_float4(un, vn, wn, z == g.nz + 1 ? 0.f : pn);
  }
}

// r = F(x) - x (FP64, stored FP32) and the first correction e1 = r.  On the
// last interior plane the state stores the swept pressure (the reapplied 3 is
// implied), so its residual is taken against that stored value.
template <int SOLVER>
__device__ __forceinline__ void dc_residual_voxel(const Fields<double>& X, float4* R, float4* E,
                                                  const uint8_t* codes, const Grid& g, int lin,
                                                  const double* ctab = nullptr) {
  int x, y, z;
  lin_to_xyz(lin, g, x, y, z);
  int code = codes[((long long)z * g.NY + y) * g.pxc + x];
  long long c = (long long)z * g.pl64 + (long long)y * g.px64 + x;
  Stencil<double> s;
  gather<double, 0>(s, X, X, c, x, y, z, g, g.px64, g.pl64);
  double un, vn, wn, pn;
  update_fast<double, SOLVER>(s, code, un, vn, wn, pn, ctab);
  const double pstored = (z == g.NZ - 3) ? __ldg(X.p + c) : s.pc;
  float ru = (float)(un - s.uc), rv = (float)(vn - s.vc), rw = (float)(wn - s.wc),
        rp = (float)(pn - pstored);
  long long c4 = (long long)z * g.pl4 + (long long)y * g.px4 + x;
  R[c4] = make_float4(ru, rv, rw, rp);
  write_voxel4(E, c4, x, y, z, g, ru, rv, rw, rp);
}

// e2 = L(e) + r (FP32 correction sweep).
template <int SOLVER>
__device__ __forceinline__ void dc_inner_voxel(const float4* E, float4* E2, const float4* R,
                                               const uint8_t* codes, const Grid& g, int lin) {
  int x, y, z;
  lin_to_xyz(lin, g, x, y, z);
  int code = codes[((long long)z * g.NY + y) * g.pxc + x];
  long long c = (long long)z * g.pl4 + (long long)y * g.px4 + x;
  Stencil<float> s;
  gather4(s, E, c, z, g);
  float un, vn, wn, pn;
  update_fast<float, SOLVER>(s, code, un, vn, wn, pn);
  const float4 r = __ldg(R + c);
  write_voxel4(E2, c, x, y, z, g, un + r.x, vn + r.y, wn + r.z, pn + r.w);
}

// x += e at a fluid voxel and at every halo copy a sweep writes for it (the
// only places where e can be non-zero).
__device__ __forceinline__ void dc_correct_voxel(const Fields<double>& X, const float4* E,
                                                 const Grid& g, int lin) {
  int x, y, z;
  lin_to_xyz(lin, g, x, y, z);
  auto add = [&](int xx, int yy, int zz) {
    long long c64 = (long long)zz * g.pl64 + (long long)yy * g.px64 + xx;
    const float4 e = E[(long long)zz * g.pl4 + (long long)yy * g.px4 + xx];
    X.u[c64] += (double)e.x;
    X.v[c64] += (double)e.y;
    X.w[c64] += (double)e.z;
    X.p[c64] += (double)e.w;
  };
  add(x, y, z);
  if (g.per[0]) {
    if (x < 4) add(x + g.nx, y, z);
    if (x >= g.nx) add(x - g.nx, y, z);
  }
  if (g.per[1]) {
    if (y < 4) add(x, y + g.ny, z);
    if (y >= g.ny) add(x, y - g.ny, z);
  }
  if (g.per[2]) {
    if (z < 4) add(x, y, z + g.nz);
    if (z >= g.nz) add(x, y, z - g.nz);
  }
}

}  // namespace pm
