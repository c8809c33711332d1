// Host-side helpers shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include <vector>

#include "../../include/poremaps.h"
#include "pm_internal.h"
#include "pm_brick.h"
#include "pm_zmarch.h"

namespace pm {

// Stop rule of calc_flow: conv < eps, evaluated every it_eval iterations
// after iteration 1000 (calc_flow.cc:92-168); a NaN conv also stops it.
// pm_params.eps_fixed_point > 0 replaces eps by that threshold and adds a
// stagnation stop for thresholds below the rounding floor of conv: the
// evaluations are grouped in windows of kStallChecks, and the run ends as
// converged when a window's largest conv is below kConvFloor and no smaller
// than the previous window's.  Above the floor conv need not fall
// monotonically: on tortuous media the pseudo-time scheme's weakly damped
// pressure-wave modes make it wander for tens of thousands of iterations
// around 1e-7 (a 512^3 Gaussian medium), so a rise there says nothing about
// convergence and only the threshold or max_iter ends the run.
constexpr int kStallChecks = 10;
constexpr double kConvFloor = 1e-13;  // ~450 rounding units of k

struct StopState {
  double win_max = 0.0;          // largest conv of the current window
  int win_n = 0;                 // evaluations in the current window
  double prev_max = HUGE_VAL;    // largest conv of the previous window
  bool stalled = false;
};

inline double stop_threshold(const pm_params& p) {
  return p.eps_fixed_point > 0 ? p.eps_fixed_point : p.eps;
}

// Records one convergence evaluation.
inline void stop_record(const pm_params& p, double conv, StopState& s) {
  if (p.eps_fixed_point <= 0 || s.stalled) return;
  s.win_max = conv > s.win_max ? conv : s.win_max;
  if (++s.win_n < kStallChecks) return;
  s.stalled = s.win_max < kConvFloor && s.win_max >= s.prev_max;
  s.prev_max = s.win_max;
  s.win_max = 0.0;
  s.win_n = 0;
}

// Whether the loop ends after an evaluation that gave conv.
inline bool stop_met(const pm_params& p, double conv, const StopState& s) {
  return !(conv >= stop_threshold(p)) || s.stalled;
}

// The result's converged flag.
inline bool stop_converged(const pm_params& p, double conv, const StopState& s) {
  return isfinite(conv) && (conv < stop_threshold(p) || s.stalled);
}

}  // namespace pm

// One device-resident domain (the state behind a pm_problem handle).
struct pm_problem {
  pm_params prm;
  pm::Grid g;
  cudaStream_t st = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int order = PM_ORDER_JACOBI;
  int precision = PM_PREC_FP64;
  int solver = 2;
  int exact = 1;
  // device memory: `arena` holds codes, list, both FP64 states, partials,
  // dout and scratch; `carena` the compact store; f32_base the padded store
  void* arena = nullptr;
  void* carena = nullptr;
  uint8_t* codes_base = nullptr;
  uint8_t* codes = nullptr;
  int* list = nullptr;
  int nlist = 0;
  int nred = 0;             // red-black order: the list holds the red voxels first, then black
  int pf64[3] = {1, 1, 1};  // per FP64 phase (Jacobi, red, black): persistent sweep
  double* f64_base[2] = {nullptr, nullptr};
  pm::Fields<double> F[2];
  float4* f32_base = nullptr;  // e0, e1, r (interleaved u, v, w, p)
  float4* E[2] = {nullptr, nullptr};
  float4* R = nullptr;
  // compact store of the mixed form (kernels 8-13): e0, e1, r at the
  // positions of the lexicographic fluid list (nlist + 1 entries each, the
  // last the zero slot), the neighbour slots and metadata of every position
  // and the fluid-mask words (pm_compact.h)
  float4* c_base = nullptr;
  float4* Ec[2] = {nullptr, nullptr};
  float4* Rc = nullptr;
  int4* cslot4 = nullptr;
  int2* cslot2 = nullptr;
  unsigned* cmeta = nullptr;
  uint2* cwords = nullptr;
  int* cerr = nullptr;  // bulk-staged compact sweep (kernels 11, 12): a wait ran out
  uint4* crec = nullptr;  // packed records of kernel 13 (own allocation, kernel 13 pinned only)
  double* partials = nullptr;
  double* dout = nullptr;
  double* hout = nullptr;  // pinned (a 256-byte slot of the process-wide pool)
  void* scratch = nullptr;  // export buffer
  size_t scratch_bytes = 0;
  int coop_blocks = 0;
  int coop_threads = 256;  // block size of the reference-order wavefront
  pm::ZmarchPlan* zp = nullptr;  // TMA z-march plan of the mixed form
  pm::BrickPlan* bp = nullptr;   // TMA brick plan of the mixed form
  int kern = 1;                  // correction-sweep kernel in use (see choose_correction_kernel)
  bool compact() const { return kern >= 8 && kern <= 13; }
  int brick[3] = {0, 0, 0};      // fluid-list order: bricks (0 = lexicographic rows)
  bool compact_ready = false;    // the compact store's slots match the current list
  // state
  int cur = 0;        // FP64 state buffer holding the current iterate
  int ecur = 0;       // FP32 correction buffer holding e
  int dc_pos = 0;     // sweeps since the last FP64 correction (mixed form)
  int mixed_inner = 100;
  int iteration = 0;  // next iteration index of calc_flow
  double perm_prev = 0.0;
  double conv = 0.0;
  bool conv_valid = false;
  pm::StopState stop;
  bool first_log = true;
  pm::Counts counts{};
  double phi = 0.0;
  double device_ms = 0.0;
  long long sweeps_done = 0;
  // CUDA graphs of sweep blocks, keyed by the block length and the state
  // parities at its start (the kernel sequence and its pointers depend on
  // nothing else); each records the parities it ends with.
  struct BlockGraph {
    int n, cur, ecur, dc_pos, phase;  // phase: iteration % mixed_inner at the start
    int cur1, ecur1, dc_pos1;
    unsigned long long launches;
    cudaGraphExec_t exec;
  };
  std::vector<BlockGraph> graphs;
};

namespace pm {

pm_status set_error(pm_status st, const char* fmt, ...);
pm_status cuda_error(cudaError_t e, const char* where);
pm_status write_log_row(const char* path, bool first, int iteration, double conv, double tps,
                        const pm_result& r);
size_t problem_device_bytes(const pm_params* p);
// pm_problem_create; rot_axis 0 / 1 rotates the uploaded geometry on the
// device for the tensor's x / y solve (launch_rotate_geom), -1 none.
pm_status problem_create(const pm_params* p, const uint8_t* geom, int rot_axis, pm_problem** out);
const pm_params* problem_params(const pm_problem* pr);
long long problem_nvox(const pm_problem* pr);
cudaStream_t problem_stream(const pm_problem* pr);
// calc_flow pieces shared with the server
pm_status iterate_n(pm_problem* pr, int n);
// mixed form: fold the FP32 correction into the FP64 state (no-op otherwise)
pm_status problem_flush(pm_problem* pr);
pm_status reduce(pm_problem* pr, int full);
void convergence_from(pm_problem* pr, double velz_sum, double* perm, double* conv);

}  // namespace pm
