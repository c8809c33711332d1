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
  const long long px = g.px64, pl = g.pl64;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nlist; q += gridDim.x * blockDim.x) {
    int lin = list[q];
    int xp = lin % g.nx;
    int r = lin / g.nx;
    int yp = r % g.ny, zp = r / g.ny;
    if (PHASE && (((xp + yp + zp) & 1) != PHASE - 1)) continue;
    int x = xp + 2, y = yp + 2, z = zp + 2;
    int code = codes[((long long)z * g.NY + y) * g.pxc + x];
    long long c = (long long)z * pl + (long long)y * px + x;
    Stencil<double> s;
    gather<double, PHASE>(s, A, B, c, x, y, z, g, px, pl);
    double un, vn, wn, pn;
    update_fast<double, SOLVER>(s, code, un, vn, wn, pn);
    write_voxel<double, false>(B, c, x, y, z, g, px, pl, un, vn, wn, pn);
  }
}

cudaError_t sweep64_exact(Fields<double> A, Fields<double> B, const uint8_t* codes,
                          const int* list, int nlist, const Grid& g, int solver, int phase,
                          cudaStream_t st);

template <int SOLVER>
static cudaError_t sweep_fast_s(Fields<double> A, Fields<double> B, const uint8_t* codes,
                                const int* list, int nlist, const Grid& g, int phase,
                                cudaStream_t st) {
  int blocks = (nlist + 255) / 256;
  if (blocks < 1) return cudaSuccess;
  if (phase == 0) k_sweep64_fast<SOLVER, 0><<<blocks, 256, 0, st>>>(A, B, codes, list, nlist, g);
  else if (phase == 1) k_sweep64_fast<SOLVER, 1><<<blocks, 256, 0, st>>>(A, B, codes, list, nlist, g);
  else k_sweep64_fast<SOLVER, 2><<<blocks, 256, 0, st>>>(A, B, codes, list, nlist, g);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_sweep64(Fields<double> A, Fields<double> B, const uint8_t* codes,
                           const int* list, int nlist, const Grid& g, int solver, int exact,
                           int phase, cudaStream_t st) {
  if (exact) return sweep64_exact(A, B, codes, list, nlist, g, solver, phase, st);
  if (solver == 1) return sweep_fast_s<1>(A, B, codes, list, nlist, g, phase, st);
  if (solver == 2) return sweep_fast_s<2>(A, B, codes, list, nlist, g, phase, st);
  return sweep_fast_s<3>(A, B, codes, list, nlist, g, phase, st);
}

// ------------------------------------------------------------------ mixed precision
// x += e over the whole padded state (e is zero wherever no sweep writes).
__global__ void k_dc_correct(Fields<double> x, Fields<float> e, Grid g) {
  long long n = (long long)g.NX * g.NY * g.NZ;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    int X = (int)(q % g.NX);
    long long r = q / g.NX;
    long long c64 = r * g.px64 + X, c32 = r * g.px32 + X;
    x.u[c64] += (double)e.u[c32];
    x.v[c64] += (double)e.v[c32];
    x.w[c64] += (double)e.w[c32];
    x.p[c64] += (double)e.p[c32];
  }
}

cudaError_t launch_dc_correct(Fields<double> x, Fields<float> e, const Grid& g,
                              cudaStream_t st) {
  k_dc_correct<<<1184, 256, 0, st>>>(x, e, g);
  count_launches(1);
  return cudaGetLastError();
}

// r = F(x) - x in FP64 (stored FP32) and the first correction e1 = r.  On the
// last interior plane the state stores the swept pressure (the reapplied 3 is
// implied), so its residual is taken against that stored value.
template <int SOLVER>
__global__ void __launch_bounds__(256) k_dc_residual(Fields<double> X, Fields<float> R,
                                                     Fields<float> E, const uint8_t* codes,
                                                     const int* list, int nlist, Grid g) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nlist; q += gridDim.x * blockDim.x) {
    int lin = list[q];
    int xp = lin % g.nx;
    int rr = lin / g.nx;
    int yp = rr % g.ny, zp = rr / g.ny;
    int x = xp + 2, y = yp + 2, z = zp + 2;
    int code = codes[((long long)z * g.NY + y) * g.pxc + x];
    long long c = (long long)z * g.pl64 + (long long)y * g.px64 + x;
    Stencil<double> s;
    gather<double, 0>(s, X, X, c, x, y, z, g, g.px64, g.pl64);
    double un, vn, wn, pn;
    update_fast<double, SOLVER>(s, code, un, vn, wn, pn);
    // the stored pressure (swept, pre-reapply on the last interior plane)
    const double pstored = (z == g.NZ - 3) ? __ldg(X.p + c) : s.pc;
    float ru = (float)(un - s.uc), rv = (float)(vn - s.vc), rw = (float)(wn - s.wc),
          rp = (float)(pn - pstored);
    long long c32 = (long long)z * g.pl32 + (long long)y * g.px32 + x;
    R.u[c32] = ru;
    R.v[c32] = rv;
    R.w[c32] = rw;
    R.p[c32] = rp;
    write_voxel<float, true>(E, c32, x, y, z, g, g.px32, g.pl32, ru, rv, rw, rp);
  }
}

cudaError_t launch_dc_residual(Fields<double> x, Fields<float> r, Fields<float> e,
                               const uint8_t* codes, const int* list, int nlist, const Grid& g,
                               int solver, cudaStream_t st) {
  int blocks = (nlist + 255) / 256;
  if (blocks < 1) return cudaSuccess;
  if (solver == 1) k_dc_residual<1><<<blocks, 256, 0, st>>>(x, r, e, codes, list, nlist, g);
  else if (solver == 2) k_dc_residual<2><<<blocks, 256, 0, st>>>(x, r, e, codes, list, nlist, g);
  else k_dc_residual<3><<<blocks, 256, 0, st>>>(x, r, e, codes, list, nlist, g);
  count_launches(1);
  return cudaGetLastError();
}

// e2 = L(e) + r over the fluid list (FP32).
template <int SOLVER>
__global__ void __launch_bounds__(256) k_dc_inner(Fields<float> E, Fields<float> E2,
                                                  Fields<float> R, const uint8_t* codes,
                                                  const int* list, int nlist, Grid g) {
  const long long px = g.px32, pl = g.pl32;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nlist; q += gridDim.x * blockDim.x) {
    int lin = list[q];
    int xp = lin % g.nx;
    int rr = lin / g.nx;
    int yp = rr % g.ny, zp = rr / g.ny;
    int x = xp + 2, y = yp + 2, z = zp + 2;
    int code = codes[((long long)z * g.NY + y) * g.pxc + x];
    long long c = (long long)z * pl + (long long)y * px + x;
    Stencil<float> s;
    gather<float, 0, true, 2>(s, E, E, c, x, y, z, g, px, pl);
    float un, vn, wn, pn;
    update_fast<float, SOLVER>(s, code, un, vn, wn, pn);
    un += __ldg(R.u + c);
    vn += __ldg(R.v + c);
    wn += __ldg(R.w + c);
    pn += __ldg(R.p + c);
    write_voxel<float, true>(E2, c, x, y, z, g, px, pl, un, vn, wn, pn);
  }
}

cudaError_t launch_dc_inner(Fields<float> e, Fields<float> e2, Fields<float> r,
                            const uint8_t* codes, const int* list, int nlist, const Grid& g,
                            int solver, cudaStream_t st) {
  int blocks = (nlist + 255) / 256;
  if (blocks < 1) return cudaSuccess;
  if (solver == 1) k_dc_inner<1><<<blocks, 256, 0, st>>>(e, e2, r, codes, list, nlist, g);
  else if (solver == 2) k_dc_inner<2><<<blocks, 256, 0, st>>>(e, e2, r, codes, list, nlist, g);
  else k_dc_inner<3><<<blocks, 256, 0, st>>>(e, e2, r, codes, list, nlist, g);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_zero32(Fields<float> e, const Grid& g, cudaStream_t st) {
  size_t bytes = sizeof(float) * (size_t)g.pl32 * g.NZ;
  cudaError_t err;
  if ((err = cudaMemsetAsync(e.u, 0, bytes, st))) return err;
  if ((err = cudaMemsetAsync(e.v, 0, bytes, st))) return err;
  if ((err = cudaMemsetAsync(e.w, 0, bytes, st))) return err;
  return cudaMemsetAsync(e.p, 0, bytes, st);
}

int zmarch_available() { return 0; }

}  // namespace pm
