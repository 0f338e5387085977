// Resident (one cooperative launch per step) grid sweep, grid_resident.cu.
#pragma once

#include "common.cuh"

namespace fpie {

int resident_tile_h();
int resident_tile_w();
int resident_depth();
// CTAs that can be co-resident on the current device (cooperative limit).
int resident_max_ctas();
// ctas: (tile*3 + channel, flag) per CTA; nbrs: 8 neighbour CTA indices per
// CTA (-1 = none); period / error: device counters, zeroed by the caller.
void launch_resident(const GridGeom& G, const uint8_t* mask, const float* g, float* buf0,
                     float* buf1, const int2* ctas, const int* nbrs, int nctas, int tiles_x,
                     int sweeps, int* period, int* error, long long spin_limit, cudaStream_t st);

}  // namespace fpie
