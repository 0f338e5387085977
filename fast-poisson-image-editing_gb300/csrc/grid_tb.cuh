// Temporally blocked grid sweep variants (grid_tb.cu).
#pragma once

#include <vector>

#include "common.cuh"

namespace fpie {

struct TbVariant {
  const char* name;
  int rows_per_thread, warps, depth;  // R, W, K (sweeps per launch)
  int tile_h, tile_w;                 // output tile: W*R - 2*apron rows, 128 - 2*apron columns
  int apron = 0;                      // region border around the tile (K, or 2K for red-black)
  bool red_black = false;             // red-black sweeps (EquSolver order), not Jacobi
  // Runs ksweeps (<= depth) sweeps xin -> xout on every active tile.
  void (*launch)(const GridGeom& G, const uint8_t* mask, const float* g,
                 const float* xin, float* xout, const uint8_t* active,
                 int tiles_x, int tiles, int ksweeps, cudaStream_t st);
  // One-time host set-up (shared-memory opt-in); call before any capture.
  void (*prepare)();
};

const std::vector<TbVariant>& tb_variants();

// Packed temporally blocked sweeps on a low-precision correction e
// (e' = (r + sum of neighbours' e) / 4 on masked pixels, FP32 arithmetic).
struct MixedVariant {
  const char* name;
  int depth, tile_h, tile_w;
  using Launch = void (*)(const GridGeom& G, const uint8_t* mask, const float* r,
                          const void* ein, void* eout, const uint8_t* active, int tiles_x,
                          int tiles, int ksweeps, int zero_start, cudaStream_t st);
  Launch launch_fp16, launch_bf16;
  // First launch of a cycle with the refine step fused in (tbp_fold_body):
  // xn = x + elast (elast NULL: no fold), r = FP32 residual of xn; writes
  // xn (tile interiors) to xout, r to rout, and the correction after
  // ksweeps sweeps from 0 to eout.
  using Fold = void (*)(const GridGeom& G, const uint8_t* mask, const float* g, const float* xin,
                        const void* elast, float* xout, float* rout, void* eout,
                        const uint8_t* active, int tiles_x, int tiles, int ksweeps,
                        cudaStream_t st);
  Fold fold_fp16, fold_bf16;
};

const std::vector<MixedVariant>& mixed_variants();

// Flags tiles (tile_h x tile_w, row-major, tiles_x per row): 0 = no masked
// pixel in the tile, 2 = the tile and its k-pixel apron fully masked, 1 = other.
void launch_tile_flags(const GridGeom& G, const uint8_t* mask, int th, int tw, int k,
                       int tiles_x, int tiles, uint8_t* flags, cudaStream_t st);

// Largest tile apron and tile extents any variant needs; the grid allocation
// reserves this much beyond the crop so no variant reads outside it.
constexpr int kMaxTileH = 256;
constexpr int kMaxTileW = 128;

}  // namespace fpie
