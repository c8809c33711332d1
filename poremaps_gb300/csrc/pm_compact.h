// Compact correction store of the mixed form (pm_compact.cu): e and r hold
// one float4 per fluid voxel at its position in the lexicographic fluid
// list; a bit-packed fluid mask (one uint2 {fluid bits, fluid voxels before}
// per row and 32 consecutive x) locates the voxels of other rows.
#pragma once

#include "pm_internal.h"

namespace pm {

// Mask words of a grid: nz * ny * ceil(nx / 32) and one sentinel.
long long compact_words(const Grid& g);
// Mask words, the six neighbour slots (sa: x L, x R, y L, y R; sb: z L, z R)
// and the metadata (code, plane flags) of every list position, from the codes
// and the ascending lexicographic fluid list; with rec, also the packed
// records of kernel 13 (pm_compact.cuh).
cudaError_t compact_setup(const uint8_t* codes, const Grid& g, const int* list, int nlist,
                          uint2* words, int4* sa, int2* sb, unsigned* meta, cudaStream_t st,
                          uint4* rec = nullptr);
// The sweep over packed records (kernel 13, 5 CTAs per SM): 16 bytes of
// index data per position instead of 28; escaped positions read sa / sb.
cudaError_t launch_dc_inner_cr(const float4* e, float4* e2, const float4* r, const uint4* rec,
                               const int4* sa, const int2* sb, int nlist, int solver,
                               cudaStream_t st);
// e2 = L(e) + r (FP32), persistent with minb CTAs of 256 threads per SM (2-4:
// next slots prefetched; 5: without the prefetch, in 48 registers).  The
// correction buffers hold nlist + 1 entries, the last the zero slot.
cudaError_t launch_dc_inner_c(const float4* e, float4* e2, const float4* r, const unsigned* meta,
                              const int4* sa, const int2* sb, int nlist, int solver, int minb,
                              cudaStream_t st);
// The same sweep with each chunk's slots and metadata staged in shared memory
// by bulk copies (kernels 11 and 12: minb 5 or 4 CTAs per SM).  meta must
// hold nlist + 4 entries and sb nlist + 2 (the copies round up to 16 bytes).
// A wait that runs out sets *err (device int) and the launch ends early.
cudaError_t launch_dc_inner_cb(const float4* e, float4* e2, const float4* r,
                               const unsigned* meta, const int4* sa, const int2* sb, int nlist,
                               int solver, int minb, int* err, cudaStream_t st);
// Test hook: while on, every bulk-staged sweep reports a timed-out first wait.
void compact_debug_fail(int on);
// r = F(x) - x (FP64, stored FP32) and e = r.
cudaError_t launch_dc_residual_c(Fields<double> x, float4* r, float4* e, const uint8_t* codes,
                                 const int* list, int nlist, const Grid& g, int solver,
                                 cudaStream_t st);
// x += e at every fluid voxel and its periodic halo copies.
cudaError_t launch_dc_correct_c(Fields<double> x, const float4* e, const int* list, int nlist,
                                const Grid& g, cudaStream_t st);

}  // namespace pm
