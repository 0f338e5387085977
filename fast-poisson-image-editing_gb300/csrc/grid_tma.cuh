// Persistent TMA-prefetch grid sweep (grid_tma.cu).
#pragma once

#include "common.cuh"

namespace fpie {

// Tile extents and sweeps per launch (same as the packed p16w8k16 variant,
// so its tile flags are shared).
int tma_tile_h();
int tma_tile_w();
int tma_depth();

// Shared-memory opt-in on the current device; call before any launch or
// capture.
void prepare_tma();

// Persistent CTAs for `items` (tile, channel) items: min(items, SMs x
// resident CTAs per SM).
int tma_ctas(int items);

// Builds the active-tile list of `flags` (tiles + 1 ints: the count, then
// the active tile indices in order); once per mask, before launch_tma.
void launch_tma_list(const uint8_t* flags, int tiles, int* list, cudaStream_t st);

// ksweeps (1..16) sweeps xin -> xout on every tile of `list`, `ctas`
// persistent CTAs taking the (tile, channel) items round-robin.  A wait for
// a region copy that fails wait_limit checks sets *error to 1 (the sweeps
// of that CTA's remaining items are then missing).
void launch_tma(const GridGeom& G, const uint8_t* mask, const float* g, const float* xin,
                float* xout, const uint8_t* flags, const int* list, int tiles_x, int tiles,
                int ksweeps, int* error, long long wait_limit, int ctas, cudaStream_t st);

}  // namespace fpie
