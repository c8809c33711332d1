// TMA-fed z-marching FP32 correction sweep (mixed form).
#pragma once

#include "pm_internal.h"

namespace pm {

struct ZmarchPlan;

// 1 when the driver provides cuTensorMapEncodeTiled.
int zmarch_available();
// Tensor maps for both correction buffers, the residual and the codes of one
// problem; zchunk <= 0 picks the z-chunk so that about two CTAs run per SM;
// tile 0: 32 x 16 columns per CTA, 1: 32 x 8.  E0, E1, R: interleaved float4.
cudaError_t zmarch_create(ZmarchPlan** out, const Grid& g, float4* E0, float4* E1, float4* R,
                          const uint8_t* codes, int zchunk, int tile);
void zmarch_destroy(ZmarchPlan* pl);
// e2 = L(e_src) + r, src = 0/1 selects the source correction buffer.
cudaError_t zmarch_inner(const ZmarchPlan* pl, int src, float4* E2, const Grid& g, int solver,
                         cudaStream_t st);
// Device int set to 1 when a pipeline wait timed out.
int* zmarch_error_flag(const ZmarchPlan* pl);
// Test hook: while on, every launch reports its first wait as timed out
// without waiting (the failure path then drains the CTA's copies in flight).
void zmarch_debug_fail(int on);

}  // namespace pm
