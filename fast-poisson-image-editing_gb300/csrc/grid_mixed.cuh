// Refinement kernels of the mixed-precision grid form (grid_mixed.cu).
#pragma once

#include "common.cuh"

namespace fpie {

// x_out = x_in + e (masked pixels; e may be NULL for no fold), r = FP32
// residual of the folded state (r may be NULL), per-block FP64 max|r| and
// sum|r| per channel into parts[6*block] (parts may be NULL).  Launch geometry: the one-sweep
// kernel's (grid_launch(G).sweep_grid / sweep_block).
void launch_refine(int precision, dim3 grid, dim3 block, const GridGeom& G, const uint8_t* mask,
                   const float* g, const float* xin, const void* e, float* xout, float* r,
                   double* parts, cudaStream_t st);

// out[0..2] = max over blocks of max|r|, out[3..5] = sum of sum|r| (double).
void launch_norms_finalize(const double* parts, int nparts, double* out, cudaStream_t st);

}  // namespace fpie
