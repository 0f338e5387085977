// Registry of the temporally blocked grid sweep variants and the tile-flag
// kernel they share.
//
// A variant (grid_tbp.cu: packed FP32x2 row pairs) handles one channel plane
// of one tile per CTA: it loads a 128-column x (W*R)-row region -- the tile
// plus a K-pixel apron on every side -- into registers, sweeps it K times
// (left/right neighbours from the adjacent lanes by warp shuffles, up/down
// neighbours from the warps above/below through shared memory, one barrier
// per sweep), and writes back the tile interior: after k <= K sweeps every
// pixel at least K away from the region border is exact.  Arithmetic per
// pixel is the one-sweep kernel's (numpy order), so results are
// bit-identical for any K.  HBM traffic per launch: x, grad and mask of the
// region once in, the tile's x once out.
//
// Variants measured and removed (slower on every measured shape, kept out of
// the library): the scalar one-value-per-lane "r" family (best r16w8k16:
// 1.49 us/sweep on square800 against 1.32 for the packed p16w8k16), the
// shallower and shared-grad packed ones (p8w12k8, p16w8k4, p12w12k8s,
// p8w16k8s), and a one-launch kernel with tiles resident in registers for
// the whole step (1.76 us/sweep: its per-period neighbour waits cost more
// than the reloads they saved).
#include "common.cuh"
#include "grid_tb.cuh"

namespace fpie {

// flags[t] = 0: tile t's interior (clipped to the crop) has no masked pixel;
// 2: every pixel of its region (interior plus a k-pixel apron, padding
// included) is masked; 1: otherwise.
__global__ void grid_tile_flags_kernel(GridGeom G, const uint8_t* __restrict__ mask,
                                       int th, int tw, int k, int tiles_x,
                                       uint8_t* __restrict__ flags) {
  const int t = blockIdx.x;
  const int ty = t / tiles_x, tx = t - ty * tiles_x;
  const int r0 = ty * th, c0 = tx * tw;
  const int r1 = min(r0 + th, G.n), c1 = min(c0 + tw, G.m);
  int any = 0;
  for (int q = threadIdx.x; q < (r1 - r0) * (c1 - c0); q += blockDim.x) {
    const int i = r0 + q / (c1 - c0), j = c0 + q % (c1 - c0);
    any |= mask[G.at(i, j)];
  }
  // Region rows/cols may reach past the crop into the zero padding.
  const int R0 = r0 - k, C0 = c0 - k, RH = th + 2 * k, RW = tw + 2 * k;
  int all = 1;
  for (int q = threadIdx.x; q < RH * RW; q += blockDim.x) {
    const int i = R0 + q / RW, j = C0 + q % RW;
    all &= (i >= 0 && i < G.n && j >= 0 && j < G.m) ? (int)mask[G.at(i, j)] : 0;
  }
  any = __syncthreads_or(any);
  all = __syncthreads_and(all);
  if (threadIdx.x == 0) flags[t] = any ? (all ? 2 : 1) : 0;
}

void append_packed_variants(std::vector<TbVariant>& v);  // grid_tbp.cu

const std::vector<TbVariant>& tb_variants() {
  static const std::vector<TbVariant> v = [] {
    std::vector<TbVariant> t;
    append_packed_variants(t);
    return t;
  }();
  return v;
}

void launch_tile_flags(const GridGeom& G, const uint8_t* mask, int th, int tw, int k,
                       int tiles_x, int tiles, uint8_t* flags, cudaStream_t st) {
  grid_tile_flags_kernel<<<tiles, 256, 0, st>>>(G, mask, th, tw, k, tiles_x, flags);
}

}  // namespace fpie
