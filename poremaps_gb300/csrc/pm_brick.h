// TMA-fed brick-tiled FP32 correction sweep (mixed form).
#pragma once

#include "pm_internal.h"

namespace pm {

struct BrickPlan;

// Brick shapes (interior voxels per CTA): 0 -> 32x8x8, 1 -> 32x8x4, 2 -> 32x4x4;
// -1 when (bx, by, bz) is none of them.
int brick_shape_of(int bx, int by, int bz);
void brick_dims(int shape, int* bx, int* by, int* bz);
// Tensor maps for both correction buffers and the codes, and the table of
// bricks that hold fluid.  `list` must be the fluid list in the brick order of
// the same shape (launch_fluid_list with its extents).  Synchronises `st`.
cudaError_t brick_create(BrickPlan** out, const Grid& g, float4* E0, float4* E1,
                         const uint8_t* codes, const int* list, int nlist, int shape,
                         cudaStream_t st);
void brick_destroy(BrickPlan* pl);
// e2 = L(e_src) + r, src = 0/1 selects the source correction buffer.
cudaError_t brick_inner(const BrickPlan* pl, int src, float4* E2, const float4* R,
                        const int* list, const Grid& g, int solver, cudaStream_t st);
// Device int set to 1 when a TMA wait timed out.
int* brick_error_flag(const BrickPlan* pl);

}  // namespace pm
