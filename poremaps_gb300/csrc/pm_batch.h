// Batched (many-sample) sweep kernels: descriptors and launcher.
#pragma once

#include "pm_internal.h"

namespace pm {

// One resident sample as the batched kernels see it.
struct SampleDesc {
  Grid g;
  Fields<double> X0, X1;  // FP64 state (mixed form: X0 is x; FP64 form: ping-pong)
  float4 *E0, *E1, *R;    // FP32 correction (ping-pong) and residual: the compact store,
                          // one float4 (u, v, w, p) per fluid-list position and a zero slot
  const uint8_t* codes;
  const unsigned* meta;   // compact store: cases, flags per list position
  const int4* sa;         // compact store: x L, x R, y L, y R neighbour positions
  const int2* sb;         // compact store: z L, z R neighbour positions
  const int* list;
  int solver;
  int ecur0;  // correction buffer the residual writes (mixed form)
  int xcur0;  // FP64 buffer holding the state at the start of a block (FP64 form)
};

// A contiguous run of one sample's fluid list.
struct WorkItem {
  int sample;
  int start;
  int count;
  int sample_items;  // items of the same sample in the table
};

enum { kBatchResidual = 0, kBatchInner = 1, kBatchCorrect = 2, kBatchSweep64 = 3, kBatchSumW = 4 };

// kind: kBatch*; round: sweep index inside the block (inner / sweep64), the
// number of rounds (correct), or the state parity (sumw).  blocks <= 0: one
// block per item.  solver: the solver all samples use (1..3; a kernel
// specialised for it), or 0 when they differ.
cudaError_t launch_batch(int kind, const SampleDesc* d, const WorkItem* items, int nitems,
                         int round, int threads, int blocks, double* out, cudaStream_t st,
                         int solver = 0);

// The FP32 correction sweeps 1 .. sweeps of a round (mixed form) in one
// persistent launch walking a device tile queue: CTAs take tickets (sweep k,
// item j) in sweep-major order from sync[0], and item j's sweep k starts once
// every item of its sample has finished sweep k - 1 (per-sample counters
// sync[2 + sample]).  Every wait is bounded; on expiry the CTA sets sync[1]
// and leaves.  sync holds 2 + samples words
// (launch_batch_round clears them itself).  extra / polls: the test hook of
// pm_debug_round_wait (a target that is never reached, a short poll limit);
// 0 / 0 in normal operation.
// ctas_per_sm / threads: resident CTAs per SM the persistent grid holds and
// their block size (128: 1..8 CTAs, 256: 1..4; the server's autotuner picks
// both).
cudaError_t launch_batch_round(const SampleDesc* d, const WorkItem* items, int nitems,
                               int nsamples, int sweeps, unsigned* sync, cudaStream_t st,
                               int solver = 0, unsigned extra = 0, int polls = 0,
                               int ctas_per_sm = 4, int threads = 256);

}  // namespace pm
