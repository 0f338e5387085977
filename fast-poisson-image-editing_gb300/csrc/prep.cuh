// GPU-side construction of the grid solver's inputs from the three uint8
// images (prep.cu), shared by the grid solver, the equation solver and the
// batched form.
#pragma once

#include "common.cuh"

namespace fpie {

struct PrepArgs {
  GridGeom G;
  const uint8_t* m01;
  int mw, x0, y0;  // mask width, crop origin in mask coordinates
  const uint8_t* src;
  int sw, sx, sy;  // source width, crop origin in source coordinates
  const uint8_t* tgt;
  int tw, tx, ty;  // target width, crop origin in target coordinates
  int mode;        // gradient: 0 'src', 1 'avg', 2 'max'
};

// Thresholds the mask (3 channels: channel sum >= 384; 1 channel: >= 128),
// clears its 1-pixel frame into m01 and folds the set pixels' bounding box
// into box = {row min, row max, col min, col max} (atomics; box must hold
// {INT_MAX, -1, INT_MAX, -1} before).
void launch_prep_mask(const uint8_t* mask, int mh, int mw, int mch, uint8_t* m01, int* box,
                      cudaStream_t st);
// Writes mask, both state buffers and grad of the crop in the planar padded
// layout (interior only: the halo keeps what it holds).
void launch_prep_grid(const PrepArgs& a, uint8_t* mask, float* xa, float* xb, float* g,
                      cudaStream_t st);

}  // namespace fpie
