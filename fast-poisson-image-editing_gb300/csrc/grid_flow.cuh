// Dependency-flow grid sweep: a whole step in one cooperative launch
// (grid_flow.cu).
#pragma once

#include "common.cuh"

namespace fpie {

// Tile extents for a temporal depth (sweeps per level): 16, the packed
// p16w8k16 variant's tiles (every form), or 12 (FP32 Jacobi sweeps only).
bool flow_depth_ok(int depth);
int flow_tile_h(int depth);
int flow_tile_w(int depth);
int flow_depth();  // 16: the mixed and red-black forms' depth
int flow_rb_depth();  // red-black sweeps per level (same tiles and apron)

// CTAs of a launch: every SM's share, all co-resident.
int flow_ctas();

// Per-mask tables of the depth-`depth` tiling from the active-tile list
// `list` (count + indices, as built by launch_tma_list), the tile flags and
// the code plane (launch_grid_code, built before): inv (tiles ints) and rec
// (tiles x flow_rec_bytes(): each active tile's index, sweep body and the
// done offsets of its 3x3 neighbourhood).
void launch_flow_tables(const GridGeom& G, const uint8_t* code, int depth, const int* list,
                        const uint8_t* flags, int tiles_x, int tiles, int* inv, void* rec,
                        cudaStream_t st);
size_t flow_rec_bytes();

// The code plane of the FP32 flow sweeps (G.plane bytes): per pixel bit 0 =
// masked, bit 1 = pinned (unmasked with a masked 4-neighbour, so it must
// keep its value); the other unmasked pixels are 0.
void launch_grid_code(const GridGeom& G, const uint8_t* mask, uint8_t* code, cudaStream_t st);

// `sweeps` sweeps on every active tile of the depth-`depth` tiling (with
// pin_bodies, Jacobi sweeps of regions whose pinned pixels lie in one
// column group or few pair rows read the code plane, launch_grid_code, and
// select only there; else every unmasked pixel keeps its value by the
// mask), from
// buffer `parity` of {x0, x1}; the result is in buffer
// (parity + ceil(sweeps / depth)) & 1 (red_black: red-black sweeps at depth
// 16, ceil(sweeps / 8)).  done (3 ints per active tile) must
// be zero.  A neighbourhood wait that exceeds spin_limit polls sets *error
// to 1 and the launch stops early.
void launch_flow(const GridGeom& G, const uint8_t* mask, const uint8_t* code, const float* g,
                 float* x0, float* x1, int parity, const int* list, const void* rec, int* done,
                 int tiles_x, int tiles, int sweeps, int* error, long long spin_limit, int ctas,
                 cudaStream_t st, bool red_black = false, int depth = 16,
                 bool pin_bodies = false);

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
