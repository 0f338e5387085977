// Dependency-flow grid sweep: a whole step in one cooperative launch
// (grid_flow.cu).
#pragma once

#include "common.cuh"

namespace fpie {

// Tile extents and sweeps per level (those of the packed p16w8k16 variant,
// so its tile flags and active-tile list are shared).
int flow_tile_h();
int flow_tile_w();
int flow_depth();
int flow_rb_depth();  // red-black sweeps per level (same tiles and apron)

// CTAs of a launch: every SM's share, all co-resident.
int flow_ctas();

// Per-mask tables from the active-tile list `list` (count + indices, as
// built by launch_tma_list) and the tile flags: inv (tiles ints) and rec
// (tiles x flow_rec_bytes(): each active tile's index, flag and the done
// offsets of its 3x3 neighbourhood).
void launch_flow_tables(const int* list, const uint8_t* flags, int tiles_x, int tiles, int* inv,
                        void* rec, cudaStream_t st);
size_t flow_rec_bytes();

// `sweeps` sweeps on every active tile, from buffer `parity` of {x0, x1};
// the result is in buffer (parity + ceil(sweeps / 16)) & 1 (red_black:
// red-black sweeps, ceil(sweeps / 8)).  done (3 ints per active tile) must
// be zero.  A neighbourhood wait that exceeds spin_limit polls sets *error
// to 1 and the launch stops early.
void launch_flow(const GridGeom& G, const uint8_t* mask, const float* g, float* x0, float* x1,
                 int parity, const int* list, const void* rec, int* done, int tiles_x, int tiles,
                 int sweeps, int* error, long long spin_limit, int ctas, cudaStream_t st,
                 bool red_black = false);

// The mixed forms (FP16 / BF16 correction, FP32 residual every 64 sweeps)
// as one launch: the level schedule of the batched kernel (mixed_levels),
// items scheduled like launch_flow.  The folded state ends in buffer
// (parity + flow_mixed_flips(sweeps)) & 1; e0/e1/r are the solver's
// correction and residual planes.
void launch_flow_mixed(const GridGeom& G, const uint8_t* mask, const float* g, float* x0, float* x1,
                       int parity, bool bf16, void* e0, void* e1, float* r, const int* list,
                       const void* rec, int* done, int tiles_x, int tiles, int sweeps, int* error,
                       long long spin_limit, int ctas, cudaStream_t st);
int flow_mixed_flips(int sweeps);

}  // namespace fpie
