// Batched / continuously batching solver (pm_server_* of include/poremaps.h).
//
// Requests queue on the host.  A scheduling round (pm_server_step):
//   1. admits queued requests in arrival order while their device footprint
//      fits the HBM budget and a slot is free; when the head of the queue does
//      not fit, later requests that do are admitted past it (backfill), at most
//      max_bypass times before the head goes in, so no request starves.  Each
//      admission sets the problem up on the device and runs one sweep, so every
//      resident sample sits at the start of an it_eval block (the reference
//      evaluates convergence after the sweeps it_eval, 2 it_eval, ...);
//   2. runs one it_eval block for all resident samples over a work table of
//      (sample, fluid-voxel run) items: the FP64 residual, the it_eval - 1
//      FP32 correction sweeps as one persistent kernel walking a device tile
//      queue (or one launch per sweep), the FP64 correction and a per-item sum
//      of w, captured once per change of the resident set in a CUDA graph;
//   3. evaluates compute_convergence per sample (the reference's stop rule)
//      and retires the finished ones (permeability, completion record,
//      device memory freed) without touching the others.
// A sample's values do not depend on what else is resident: every voxel runs
// the same device code as the single-problem path, and its sums follow its own
// items in a fixed order.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <deque>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "../../include/poremaps.h"
#include "pm_api_internal.h"
#include "pm_batch.h"

using namespace pm;

namespace {

struct Req {
  uint64_t ticket;
  pm_params prm;
  std::vector<uint8_t> geom;
  double submit_ms;
  int bypassed = 0;  // admissions of later requests past this one at the head
};

struct Res {
  uint64_t ticket;
  pm_problem* pr;
  double submit_ms, admit_ms;
  size_t bytes;
  double perm = 0.0, conv = 0.0;
  bool conv_valid = false;
  StopState stop;
  int last_check = 0;
  int it = 0;  // next iteration index
  int item0 = 0, nitems = 0;
};

}  // namespace

struct pm_server {
  pm_server_config cfg;
  std::mutex mu;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  std::deque<Req> queue;
  std::vector<Res> res;
  std::deque<pm_completion> done;
  size_t budget = 0, used = 0;
  uint64_t next_ticket = 1;
  std::chrono::steady_clock::time_point t0;
  int block = 0;  // sweeps per scheduling round = it_eval of the requests
  std::vector<SampleDesc> h_desc;
  std::vector<WorkItem> h_items;
  SampleDesc* d_desc = nullptr;
  size_t cap_desc = 0;
  WorkItem* d_items = nullptr;
  size_t cap_items = 0;
  double* d_part = nullptr;
  double* h_part = nullptr;
  size_t cap_part = 0;
  unsigned* d_sync = nullptr;  // persistent round: ticket, error flag, per-sample counters
  size_t cap_sync = 0;
  unsigned* h_flag = nullptr;  // pinned copy of the error flag
  bool dirty = true;
  cudaGraphExec_t gexec = nullptr;
  int graph_kernels = 0;
  int threads = 256, chunk = 8192;
  int round_ctas = 4;      // CTAs per SM of the persistent round kernel
  int round_threads = 256;  // and their block size
  bool shape_pinned = false;  // pm_server_set_launch_shape: no autotuning
  int solver = 0;  // the solver every resident sample uses, 0 when they differ
  long long tuned_for = -1;
  double busy_ms = 0.0;
  unsigned long long lups = 0;
};

namespace {

// pm_debug_round_wait: added to every wait target of the persistent round,
// and its poll limit (0 = the kernel's own).
std::atomic<unsigned> g_round_extra{0};
std::atomic<int> g_round_polls{0};

double now_ms(pm_server* s) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - s->t0)
      .count();
}

#define SCK(expr)                                        \
  do {                                                   \
    cudaError_t _e = (expr);                             \
    if (_e != cudaSuccess) return cuda_error(_e, #expr); \
  } while (0)

template <typename T>
pm_status grow(T** d, size_t* cap, size_t n) {
  if (n <= *cap) return PM_OK;
  size_t c = std::max(n, *cap * 2 + 16);
  if (*d) cudaFree(*d);
  *d = nullptr;
  SCK(cudaMalloc((void**)d, c * sizeof(T)));
  *cap = c;
  return PM_OK;
}

void complete(pm_server* s, uint64_t ticket, pm_status st, const pm_result* r, double submit,
              double admit) {
  pm_completion c;
  memset(&c, 0, sizeof c);
  c.ticket = ticket;
  c.status = st;
  if (r) c.result = *r;
  c.submit_ms = submit;
  c.admit_ms = admit;
  c.finish_ms = now_ms(s);
  s->done.push_back(c);
}

void drop_graph(pm_server* s) {
  if (s->gexec) cudaGraphExecDestroy(s->gexec);
  s->gexec = nullptr;
}

// calc_flow runs iterations 0 .. max_iter-1.  A sample whose next block
// would pass that runs its last iterations alone on its own stream with the
// single-problem sweeps; they hold no convergence check (the last one was at
// the end of the previous block, and the next would be a full block away).
pm_status run_tail(Res& r) {
  pm_problem* pr = r.pr;
  const int n = pr->prm.max_iter - r.it;
  if (n <= 0) return PM_OK;
  pr->iteration = r.it;
  pm_status st = iterate_n(pr, n);
  if (st == PM_OK) st = problem_flush(pr);
  if (st == PM_OK && cudaStreamSynchronize(problem_stream(pr)) != cudaSuccess)
    st = cuda_error(cudaGetLastError(), "final iterations");
  r.it += n;
  pr->sweeps_done = r.it;
  return st;
}

// Completes a finished sample (result from its resident state) and frees it.
void retire(pm_server* s, Res& r, pm_status st) {
  pm_problem* pr = r.pr;
  const pm_params& p = pr->prm;
  pm_result out;
  memset(&out, 0, sizeof out);
  if (st == PM_OK) st = pm_compute_permeability(pr, &out);
  out.iterations = r.last_check;
  out.sweeps = r.it;
  out.conv = r.conv;
  out.converged = r.conv_valid && stop_converged(p, r.conv, r.stop);
  out.permeability = r.perm;
  if (st == PM_OK && (!isfinite(out.wk33) || !isfinite(r.perm))) st = PM_ERR_NONFINITE;
  complete(s, r.ticket, st, st == PM_OK || st == PM_ERR_NONFINITE ? &out : nullptr, r.submit_ms,
           r.admit_ms);
  pm_problem_destroy(pr);
  s->used -= r.bytes;
}

pm_params request_params(const pm_server* s, const Req& q) {
  pm_params p = q.prm;
  p.precision = s->cfg.precision;
  p.order = PM_ORDER_JACOBI;
  p.write_log = 0;
  p.mixed_inner = p.it_eval;  // corrections after iterations 0, it_eval, 2 it_eval, ...
  p.kernel = 8;               // the batched kernels use the compact correction store
  return p;
}

int bypass_limit(const pm_server* s) {
  return s->cfg.max_bypass == 0 ? 64 : s->cfg.max_bypass;
}

// How far behind the head the backfill scan looks for a request that fits.
constexpr size_t kBackfillScan = 256;

pm_status admit(pm_server* s) {
  size_t i = 0;  // queue position under consideration (0 = head)
  while (i < s->queue.size() && i < kBackfillScan &&
         (int)s->res.size() < s->cfg.max_resident) {
    Req& q = s->queue[i];
    pm_params p = request_params(s, q);
    size_t bytes = problem_device_bytes(&p);
    if (bytes > s->budget) {  // can never fit: fail it instead of blocking the queue
      pm_status e = set_error(PM_ERR_NOMEM, "request needs %zu bytes, budget %zu", bytes,
                              s->budget);
      complete(s, q.ticket, e, nullptr, q.submit_ms, now_ms(s));
      s->queue.erase(s->queue.begin() + i);
      continue;
    }
    // a request behind the head goes in only while the head may still be
    // passed (backfill on, fewer than max_bypass admissions past it so far)
    const int lim = bypass_limit(s);
    if (i > 0 && (lim < 0 || s->queue.front().bypassed >= lim)) break;
    if (s->used + bytes > s->budget) {
      if (lim < 0 || s->queue.front().bypassed >= lim) break;  // the head waits
      ++i;  // does not fit now: look behind it
      continue;
    }
    if (i > 0) s->queue.front().bypassed++;
    Req qq = std::move(q);
    s->queue.erase(s->queue.begin() + i);
    pm_problem* pr = nullptr;
    pm_status st = pm_problem_create(&p, qq.geom.data(), &pr);
    if (st != PM_OK) {
      complete(s, qq.ticket, st, nullptr, qq.submit_ms, now_ms(s));
      continue;
    }
    // iteration 0 on its own: afterwards every block ends on a check iteration
    if ((st = iterate_n(pr, 1)) == PM_OK) st = problem_flush(pr);
    if (st == PM_OK && cudaStreamSynchronize(problem_stream(pr)) != cudaSuccess)
      st = cuda_error(cudaGetLastError(), "admission sweep");
    if (st != PM_OK) {
      pm_problem_destroy(pr);
      complete(s, qq.ticket, st, nullptr, qq.submit_ms, now_ms(s));
      continue;
    }
    Res r;
    r.ticket = qq.ticket;
    r.pr = pr;
    r.submit_ms = qq.submit_ms;
    r.admit_ms = now_ms(s);
    r.bytes = bytes;
    r.it = 1;
    s->used += bytes;
    if (r.it + s->block > p.max_iter) {  // fewer iterations than one block: alone
      retire(s, r, run_tail(r));
      continue;
    }
    s->res.push_back(r);
    s->dirty = true;
  }
  return PM_OK;
}

// Work items of at most `chunk` fluid voxels, and small enough that a round
// has at least ~8 items per SM: when a few samples remain (the slow ones of a
// batch) the device still gets a full grid.
void build_items(pm_server* s, int chunk) {
  s->h_items.clear();
  const int sms = sm_count();
  long long total = 0;
  for (auto& r : s->res) total += r.pr->nlist;
  const long long fill = (total + 8LL * sms - 1) / (8LL * sms);
  chunk = (int)std::max(512LL, std::min<long long>(chunk, fill));
  for (size_t i = 0; i < s->res.size(); ++i) {
    Res& r = s->res[i];
    r.item0 = (int)s->h_items.size();
    int n = r.pr->nlist;
    for (int a = 0; a < n; a += chunk)
      s->h_items.push_back({(int)i, a, std::min(chunk, n - a), 0});
    r.nitems = (int)s->h_items.size() - r.item0;
    for (int k = r.item0; k < r.item0 + r.nitems; ++k) s->h_items[k].sample_items = r.nitems;
  }
}

pm_status upload(pm_server* s) {
  pm_status e;
  if ((e = grow(&s->d_desc, &s->cap_desc, s->h_desc.size())) != PM_OK) return e;
  if ((e = grow(&s->d_items, &s->cap_items, s->h_items.size())) != PM_OK) return e;
  if ((e = grow(&s->d_sync, &s->cap_sync, 2 + s->h_desc.size())) != PM_OK) return e;
  if (s->h_items.size() > s->cap_part) {
    if (s->d_part) cudaFree(s->d_part);
    if (s->h_part) cudaFreeHost(s->h_part);
    s->d_part = nullptr;
    s->h_part = nullptr;
    size_t c = s->h_items.size() * 2 + 16;
    SCK(cudaMalloc((void**)&s->d_part, c * sizeof(double)));
    SCK(cudaMallocHost((void**)&s->h_part, c * sizeof(double)));
    s->cap_part = c;
  }
  SCK(cudaMemcpyAsync(s->d_desc, s->h_desc.data(), s->h_desc.size() * sizeof(SampleDesc),
                      cudaMemcpyHostToDevice, s->st));
  SCK(cudaMemcpyAsync(s->d_items, s->h_items.data(), s->h_items.size() * sizeof(WorkItem),
                      cudaMemcpyHostToDevice, s->st));
  SCK(cudaStreamSynchronize(s->st));
  return PM_OK;
}

bool mixed(const pm_server* s) { return s->cfg.precision == PM_PREC_MIXED; }

// The launches of one block (recorded into a graph or issued directly).
pm_status issue_block(pm_server* s, int* nk) {
  const int n = (int)s->h_items.size(), T = s->threads;
  int k = 0;
  if (mixed(s)) {
    SCK(launch_batch(kBatchResidual, s->d_desc, s->d_items, n, 0, T, 0, nullptr, s->st,
                     s->solver));
    ++k;
    if (s->cfg.relaunch_sweeps) {
      for (int r = 1; r < s->block; ++r, ++k)
        SCK(launch_batch(kBatchInner, s->d_desc, s->d_items, n, r, T, 0, nullptr, s->st,
                         s->solver));
    } else if (s->block > 1) {
      SCK(launch_batch_round(s->d_desc, s->d_items, n, (int)s->h_desc.size(), s->block - 1,
                             s->d_sync, s->st, s->solver, g_round_extra.load(),
                             g_round_polls.load(), s->round_ctas, s->round_threads));
      ++k;
    }
    SCK(launch_batch(kBatchCorrect, s->d_desc, s->d_items, n, s->block, T, 0, nullptr, s->st));
    SCK(launch_batch(kBatchSumW, s->d_desc, s->d_items, n, 0, T, 0, s->d_part, s->st));
    k += 2;
  } else {
    for (int r = 0; r < s->block; ++r, ++k)
      SCK(launch_batch(kBatchSweep64, s->d_desc, s->d_items, n, r, T, 0, nullptr, s->st,
                       s->solver));
    SCK(launch_batch(kBatchSumW, s->d_desc, s->d_items, n, s->block, T, 0, s->d_part, s->st));
    ++k;
  }
  *nk = k;
  return PM_OK;
}

// Launch shape of the batched sweeps, timed on the current resident set:
// the work-item size (voxels per tile of the queue) and, for the persistent
// round, the block size and CTAs per SM of its grid (128 or 256 threads at
// the same range of resident warps; a 3-sweep round per candidate); for one
// launch per sweep, the threads per block.  Decisions are kept per size
// class (precision, launch form, solver, log2 of the resident fluid voxels,
// log2 of the resident samples), so a stream whose resident set keeps its
// size tunes once.  Safe at a block boundary: the timed launches only write
// correction buffers the next block's residual and first sweep rewrite.
struct TuneKey {
  int mixed, persistent, solver, fluid_class, samples_class;
  bool operator<(const TuneKey& o) const {
    return std::tie(mixed, persistent, solver, fluid_class, samples_class) <
           std::tie(o.mixed, o.persistent, o.solver, o.fluid_class, o.samples_class);
  }
};
struct TuneVal {
  int threads, chunk, ctas, round_threads;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneVal> g_tuned;

int log2_class(long long v) {
  int c = 0;
  while (v > 1) { v >>= 1; ++c; }
  return c;
}

pm_status autotune(pm_server* s) {
  static const int kThreads[] = {128, 256, 512};
  static const int kChunks[] = {2048, 8192, 32768};
  static const int kCtas[] = {2, 3, 4};
  static const int kRoundThreads[] = {256, 128};
  long long total = 0;
  for (auto& r : s->res) total += r.pr->nlist;
  if (s->tuned_for > 0 && total < 4 * s->tuned_for && 4 * total > s->tuned_for) return PM_OK;
  const bool persistent = mixed(s) && !s->cfg.relaunch_sweeps && s->block > 1;
  const TuneKey key{mixed(s) ? 1 : 0, persistent ? 1 : 0, s->solver, log2_class(total),
                    log2_class((long long)s->res.size())};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
      s->threads = it->second.threads;
      s->chunk = it->second.chunk;
      s->round_ctas = it->second.ctas;
      s->round_threads = it->second.round_threads;
      s->tuned_for = total;
      return PM_OK;
    }
  }
  float best = 1e30f;
  int bt = s->threads, bc = s->chunk, bm = s->round_ctas, brt = s->round_threads;
  const int kind = mixed(s) ? kBatchInner : kBatchSweep64;
  auto time_it = [&](auto&& issue, float* ms) -> pm_status {
    pm_status e = issue();  // warm-up
    if (e != PM_OK) return e;
    SCK(cudaEventRecord(s->e0, s->st));
    for (int i = 0; i < 3; ++i)
      if ((e = issue()) != PM_OK) return e;
    SCK(cudaEventRecord(s->e1, s->st));
    SCK(cudaEventSynchronize(s->e1));
    SCK(cudaEventElapsedTime(ms, s->e0, s->e1));
    return PM_OK;
  };
  // persistent round: the work-item size at the current block shape first,
  // then the block shape for that size (9 timed rounds, not 3 x 6)
  auto time_round = [&](int n, int m, int rt, float* ms) -> pm_status {
    return time_it([&]() -> pm_status {
      SCK(launch_batch_round(s->d_desc, s->d_items, n, (int)s->h_desc.size(), 3, s->d_sync,
                             s->st, s->solver, 0, 0, m, rt));
      return PM_OK;
    }, ms);
  };
  for (int c : kChunks) {
    build_items(s, c);
    pm_status e = upload(s);
    if (e != PM_OK) return e;
    const int n = (int)s->h_items.size();
    if (persistent) {
      float ms = 0.f;
      if ((e = time_round(n, bm, brt, &ms)) != PM_OK) return e;
      if (ms < best) { best = ms; bc = c; }
    } else {
      for (int t : kThreads) {
        float ms = 0.f;
        e = time_it([&]() -> pm_status {
          SCK(launch_batch(kind, s->d_desc, s->d_items, n, 1, t, 0, nullptr, s->st, s->solver));
          return PM_OK;
        }, &ms);
        if (e != PM_OK) return e;
        if (ms < best) { best = ms; bt = t; bc = c; }
      }
    }
  }
  if (persistent) {
    build_items(s, bc);
    pm_status e = upload(s);
    if (e != PM_OK) return e;
    const int n = (int)s->h_items.size();
    const int m_in = bm, rt_in = brt;
    // another block shape only for a clear win: a 3-sweep round is short,
    // and 128-thread rounds that won such trials by a few per cent were
    // slower over whole runs (c4: 117-118 k against 121-122 k solves/h)
    const float keep = 0.95f * best;
    float best2 = keep;
    for (int rt : kRoundThreads)
      for (int m0 : kCtas) {
        const int m = m0 * (256 / rt);  // the same resident warps at either block size
        if (m == m_in && rt == rt_in) continue;  // timed in the first stage
        float ms = 0.f;
        if ((e = time_round(n, m, rt, &ms)) != PM_OK) return e;
        if (ms < best2) { best2 = ms; bm = m; brt = rt; }
      }
  }
  s->threads = bt;
  s->chunk = bc;
  s->round_ctas = bm;
  s->round_threads = brt;
  s->tuned_for = total;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tuned[key] = {bt, bc, bm, brt};
  return PM_OK;
}

pm_status rebuild(pm_server* s) {
  s->h_desc.clear();
  s->solver = s->res.empty() ? 0 : s->res[0].pr->solver;
  for (auto& r : s->res)
    if (r.pr->solver != s->solver) s->solver = 0;
  for (auto& r : s->res) {
    pm_problem* pr = r.pr;
    SampleDesc d;
    memset(&d, 0, sizeof d);
    d.g = pr->g;
    d.codes = pr->codes;
    d.list = pr->list;
    d.solver = pr->solver;
    if (mixed(s)) {
      d.X0 = pr->F[pr->cur];
      d.X1 = pr->F[1 - pr->cur];
      d.E0 = pr->Ec[0];
      d.E1 = pr->Ec[1];
      d.R = pr->Rc;
      d.meta = pr->cmeta;
      d.sa = pr->cslot4;
      d.sb = pr->cslot2;
      d.ecur0 = 0;
      d.xcur0 = 0;
    } else {
      d.X0 = pr->F[0];
      d.X1 = pr->F[1];
      d.xcur0 = pr->cur;
    }
    s->h_desc.push_back(d);
  }
  pm_status e;
  if (s->cfg.autotune && !s->shape_pinned && (e = autotune(s)) != PM_OK) return e;
  build_items(s, s->chunk);
  if ((e = upload(s)) != PM_OK) return e;
  drop_graph(s);
  s->dirty = false;
  return PM_OK;
}

pm_status run_block(pm_server* s) {
  pm_status e;
  int nk = 0;
  if (s->cfg.use_graphs && !s->gexec) {
    cudaGraph_t g = nullptr;
    SCK(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
    e = issue_block(s, &nk);
    cudaError_t ce = cudaStreamEndCapture(s->st, &g);
    if (e != PM_OK) {
      if (g) cudaGraphDestroy(g);
      return e;
    }
    if (ce != cudaSuccess) return cuda_error(ce, "cudaStreamEndCapture");
    ce = cudaGraphInstantiate(&s->gexec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return cuda_error(ce, "cudaGraphInstantiate");
    s->graph_kernels = nk;
  }
  SCK(cudaEventRecord(s->e0, s->st));
  if (s->gexec) {
    SCK(cudaGraphLaunch(s->gexec, s->st));
    count_launches(s->graph_kernels);
  } else if ((e = issue_block(s, &nk)) != PM_OK) {
    return e;
  }
  SCK(cudaMemcpyAsync(s->h_part, s->d_part, s->h_items.size() * sizeof(double),
                      cudaMemcpyDeviceToHost, s->st));
  const bool round = mixed(s) && !s->cfg.relaunch_sweeps && s->block > 1;
  if (round)
    SCK(cudaMemcpyAsync(s->h_flag, s->d_sync + 1, sizeof(unsigned), cudaMemcpyDeviceToHost,
                        s->st));
  SCK(cudaEventRecord(s->e1, s->st));
  SCK(cudaStreamSynchronize(s->st));
  if (round && *s->h_flag)
    return set_error(PM_ERR_CUDA, "batched round: a wait of the persistent sweep kernel timed out");
  float ms = 0.f;
  SCK(cudaEventElapsedTime(&ms, s->e0, s->e1));
  s->busy_ms += ms;
  for (auto& r : s->res) s->lups += (unsigned long long)r.pr->g.nvox * s->block;
  return PM_OK;
}

pm_status after_block(pm_server* s) {
  std::vector<Res> keep;
  bool changed = false;
  for (auto& r : s->res) {
    pm_problem* pr = r.pr;
    r.it += s->block;
    pr->iteration = r.it;
    pr->sweeps_done = r.it;
    pr->dc_pos = 0;
    if (!mixed(s)) pr->cur = (pr->cur + s->block) & 1;
    const pm_params& p = pr->prm;
    const int last = r.it - 1;
    if (last % p.it_eval == 0 && last > 1000) {
      double sum = 0.0;
      for (int k = 0; k < r.nitems; ++k) sum += s->h_part[r.item0 + k];
      convergence_from(pr, sum, &r.perm, &r.conv);
      r.conv_valid = true;
      r.last_check = last;
      stop_record(p, r.conv, r.stop);
    }
    const bool finished = (r.conv_valid && stop_met(p, r.conv, r.stop)) || r.it >= p.max_iter;
    if (!finished && r.it + s->block <= p.max_iter) {
      keep.push_back(r);
      continue;
    }
    retire(s, r, finished ? PM_OK : run_tail(r));
    changed = true;
  }
  s->res.swap(keep);
  if (changed || (!mixed(s) && (s->block & 1))) s->dirty = true;
  return PM_OK;
}

}  // namespace

extern "C" {

pm_status pm_server_create(const pm_server_config* cfg, pm_server** out) {
  if (!out) return set_error(PM_ERR_INVALID, "out is NULL");
  *out = nullptr;
  pm_server* s = new pm_server();
  if (cfg) s->cfg = *cfg;
  else memset(&s->cfg, 0, sizeof s->cfg);
  if (s->cfg.precision != PM_PREC_FP64 && s->cfg.precision != PM_PREC_MIXED) {
    delete s;
    return set_error(PM_ERR_INVALID, "bad precision");
  }
  if (s->cfg.max_resident <= 0) s->cfg.max_resident = 1024;
  size_t fr = 0, tot = 0;
  cudaError_t e = cudaMemGetInfo(&fr, &tot);
  if (e != cudaSuccess) {
    delete s;
    return cuda_error(e, "cudaMemGetInfo");
  }
  s->budget = s->cfg.hbm_budget_bytes ? s->cfg.hbm_budget_bytes : (size_t)(0.8 * (double)fr);
  if ((e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreate(&s->e0)) != cudaSuccess ||
      (e = cudaEventCreate(&s->e1)) != cudaSuccess ||
      (e = cudaMallocHost((void**)&s->h_flag, sizeof(unsigned))) != cudaSuccess) {
    pm_server_destroy(s);
    return cuda_error(e, "server stream/events");
  }
  s->t0 = std::chrono::steady_clock::now();
  *out = s;
  return PM_OK;
}

pm_status pm_server_destroy(pm_server* s) {
  if (!s) return PM_OK;
  if (s->st) cudaStreamSynchronize(s->st);
  for (auto& r : s->res) pm_problem_destroy(r.pr);
  drop_graph(s);
  cudaFree(s->d_desc);
  cudaFree(s->d_items);
  cudaFree(s->d_part);
  cudaFree(s->d_sync);
  if (s->h_part) cudaFreeHost(s->h_part);
  if (s->h_flag) cudaFreeHost(s->h_flag);
  if (s->e0) cudaEventDestroy(s->e0);
  if (s->e1) cudaEventDestroy(s->e1);
  if (s->st) cudaStreamDestroy(s->st);
  delete s;
  return PM_OK;
}

pm_status pm_server_submit(pm_server* s, const pm_params* p, const uint8_t* geom,
                           uint64_t* ticket) {
  if (!s || !p || !geom || !ticket) return set_error(PM_ERR_INVALID, "bad arguments");
  std::lock_guard<std::mutex> lk(s->mu);
  if (p->size[0] < 1 || p->size[1] < 1 || p->size[2] < 1 || p->it_eval <= 0)
    return set_error(PM_ERR_INVALID, "bad request size or it_eval");
  if (s->block == 0) s->block = p->it_eval;
  if (p->it_eval != s->block)
    return set_error(PM_ERR_INVALID, "server runs it_eval blocks of %d sweeps, request has %d",
                     s->block, p->it_eval);
  if (s->cfg.precision == PM_PREC_MIXED && p->solving_algorithm == 1)
    return set_error(PM_ERR_INVALID, "mixed precision needs solver 2 or 3");
  Req q;
  q.ticket = s->next_ticket++;
  q.prm = *p;
  size_t n = (size_t)p->size[0] * p->size[1] * p->size[2];
  q.geom.assign(geom, geom + n);
  q.submit_ms = now_ms(s);
  s->queue.push_back(std::move(q));
  *ticket = s->queue.back().ticket;
  return PM_OK;
}

pm_status pm_server_step(pm_server* s, int* active) {
  if (!s) return set_error(PM_ERR_INVALID, "bad arguments");
  std::lock_guard<std::mutex> lk(s->mu);
  pm_status e;
  if ((e = admit(s)) != PM_OK) return e;
  if (!s->res.empty()) {
    if (s->dirty && (e = rebuild(s)) != PM_OK) return e;
    if ((e = run_block(s)) != PM_OK) return e;
    if ((e = after_block(s)) != PM_OK) return e;
    if ((e = admit(s)) != PM_OK) return e;
  }
  if (active) *active = (int)(s->res.size() + s->queue.size());
  return PM_OK;
}

pm_status pm_server_poll(pm_server* s, pm_completion* out, int max, int* n) {
  if (!s || !n || (max > 0 && !out)) return set_error(PM_ERR_INVALID, "bad arguments");
  std::lock_guard<std::mutex> lk(s->mu);
  int k = 0;
  while (k < max && !s->done.empty()) {
    out[k++] = s->done.front();
    s->done.pop_front();
  }
  *n = k;
  return PM_OK;
}

pm_status pm_server_stats(pm_server* s, double* busy_ms, double* wall_ms, uint64_t* lups) {
  if (!s) return set_error(PM_ERR_INVALID, "bad arguments");
  std::lock_guard<std::mutex> lk(s->mu);
  if (busy_ms) *busy_ms = s->busy_ms;
  if (wall_ms) *wall_ms = now_ms(s);
  if (lups) *lups = s->lups;
  return PM_OK;
}

double pm_server_clock_ms(pm_server* s) { return s ? now_ms(s) : 0.0; }

pm_status pm_debug_round_wait(unsigned extra, int polls) {
  if (polls < 0) return set_error(PM_ERR_INVALID, "polls must be >= 0");
  g_round_extra.store(extra);
  g_round_polls.store(polls);
  return PM_OK;
}

pm_status pm_server_request_bytes(pm_server* s, const pm_params* p, size_t* bytes) {
  if (!s || !p || !bytes) return set_error(PM_ERR_INVALID, "bad arguments");
  Req q;
  q.prm = *p;
  pm_params rp = request_params(s, q);
  return pm_problem_footprint(&rp, bytes);
}

pm_status pm_server_launch_shape(pm_server* s, int shape[4]) {
  if (!s || !shape) return set_error(PM_ERR_INVALID, "bad arguments");
  std::lock_guard<std::mutex> lk(s->mu);
  shape[0] = s->chunk;
  shape[1] = s->round_ctas;
  shape[2] = s->round_threads;
  shape[3] = s->threads;
  return PM_OK;
}

pm_status pm_server_set_launch_shape(pm_server* s, const int shape[4]) {
  if (!s || !shape) return set_error(PM_ERR_INVALID, "bad arguments");
  const int chunk = shape[0], ctas = shape[1], rt = shape[2], t = shape[3];
  if (chunk < 1 || (rt != 128 && rt != 256) || ctas < 1 || ctas > (rt == 128 ? 8 : 4) ||
      (t != 128 && t != 256 && t != 512))
    return set_error(PM_ERR_INVALID,
                     "launch shape: voxels per item >= 1, round threads 128 (1-8 CTAs per SM) "
                     "or 256 (1-4), threads 128, 256 or 512");
  std::lock_guard<std::mutex> lk(s->mu);
  s->chunk = chunk;
  s->round_ctas = ctas;
  s->round_threads = rt;
  s->threads = t;
  s->shape_pinned = true;
  s->dirty = true;  // items and graph are rebuilt at the next round
  return PM_OK;
}

pm_status pm_server_cancel(pm_server* s, uint64_t ticket) {
  if (!s) return set_error(PM_ERR_INVALID, "bad arguments");
  std::lock_guard<std::mutex> lk(s->mu);
  for (size_t i = 0; i < s->queue.size(); ++i) {
    if (s->queue[i].ticket != ticket) continue;
    complete(s, ticket, PM_ERR_CANCELLED, nullptr, s->queue[i].submit_ms, now_ms(s));
    s->queue.erase(s->queue.begin() + i);
    return PM_OK;
  }
  for (size_t i = 0; i < s->res.size(); ++i) {
    if (s->res[i].ticket != ticket) continue;
    // between rounds the server stream is idle: free the sample now and
    // rebuild the work table (and graph) for the rest before the next round
    Res r = s->res[i];
    s->res.erase(s->res.begin() + i);
    complete(s, ticket, PM_ERR_CANCELLED, nullptr, r.submit_ms, r.admit_ms);
    pm_problem_destroy(r.pr);
    s->used -= r.bytes;
    s->dirty = true;
    return PM_OK;
  }
  return set_error(PM_ERR_NOT_FOUND, "ticket %llu is not queued or resident",
                   (unsigned long long)ticket);
}

}  // extern "C"
