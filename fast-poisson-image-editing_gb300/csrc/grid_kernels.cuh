// Launch plans for the grid sweep / finish kernels (grid_kernels.cu).
#pragma once

#include "common.cuh"

namespace fpie {

struct GridLaunch {
  dim3 sweep_block, sweep_grid;    // one-sweep kernel
  dim3 finish_block, finish_grid;  // residual + image kernel
  int nparts;                      // residual partials (finish blocks)
};

GridLaunch grid_launch(const GridGeom& G);

// One Jacobi sweep xin -> xout over the crop (all three channels).
void launch_grid_sweep(const GridLaunch& L, const GridGeom& G,
                       const uint8_t* mask, const float* g, const float* xin,
                       float* xout, cudaStream_t st);

// Residual partials (|r| summed per block, double) and the clipped uint8
// image in the reference's interleaved [n][m][3] layout.
void launch_grid_finish(const GridLaunch& L, const GridGeom& G,
                        const uint8_t* mask, const float* g, const float* x,
                        uint8_t* img, double* parts, cudaStream_t st);

}  // namespace fpie
