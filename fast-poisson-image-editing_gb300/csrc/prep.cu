// GPU-side construction of the grid solver's inputs from the three images.
//
// Same results as the host path (GridProcessor.reset, fpie/process.py:422-487),
// bit for bit:
//   * mask: a 3-channel mask is "on" when its channel mean is >= 128, i.e.
//     when the channel sum is >= 384 (exact for uint8); a 1-channel mask when
//     its value is >= 128; the outer 1-pixel frame is cleared;
//   * crop: the set pixels' bounding box grown by one pixel;
//   * grad: for every set pixel, mix(C-U) + mix(C-D) + mix(C-L) + mix(C-R)
//     accumulated from 0 in that order, where mix is 'src' (a), 'avg'
//     ((a+b)/2) or 'max' (b if |a| < |b| else a), a the source difference
//     and b the target difference, all in float32 (every intermediate is a
//     small integer or half-integer, so the sums are exact); 0 elsewhere.
// The outputs go straight into the solver's planar padded layout.
#include <algorithm>

#include "common.cuh"

namespace fpie {

__global__ void prep_mask_kernel(const uint8_t* __restrict__ mask, int mh, int mw, int mch,
                                 uint8_t* __restrict__ m01, int* __restrict__ box) {
  int rmin = INT_MAX, rmax = -1, cmin = INT_MAX, cmax = -1;
  const long long total = (long long)mh * mw;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < total;
       p += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(p / mw), j = (int)(p % mw);
    bool on;
    if (mch == 3)
      on = (int)mask[p * 3] + mask[p * 3 + 1] + mask[p * 3 + 2] >= 384;
    else
      on = mask[p] >= 128;
    on = on && i > 0 && i < mh - 1 && j > 0 && j < mw - 1;
    m01[p] = on;
    if (on) {
      rmin = min(rmin, i);
      rmax = max(rmax, i);
      cmin = min(cmin, j);
      cmax = max(cmax, j);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    rmin = min(rmin, __shfl_down_sync(0xffffffffu, rmin, o));
    rmax = max(rmax, __shfl_down_sync(0xffffffffu, rmax, o));
    cmin = min(cmin, __shfl_down_sync(0xffffffffu, cmin, o));
    cmax = max(cmax, __shfl_down_sync(0xffffffffu, cmax, o));
  }
  if ((threadIdx.x & 31) == 0 && rmax >= 0) {
    atomicMin(box + 0, rmin);
    atomicMax(box + 1, rmax);
    atomicMin(box + 2, cmin);
    atomicMax(box + 3, cmax);
  }
}

__device__ __forceinline__ float mix_term(float a, float b, int mode) {
  if (mode == 0) return a;                             // 'src'
  if (mode == 1) return __fmul_rn(__fadd_rn(a, b), 0.5f);  // 'avg': (a+b)/2, exact here
  return fabsf(a) < fabsf(b) ? b : a;                  // 'max'
}

struct PrepArgs {
  GridGeom G;
  const uint8_t* m01;
  int mw, x0, y0;  // mask width, crop origin in mask coordinates
  const uint8_t* src;
  int sw, sx, sy;  // source width, crop origin in source coordinates
  const uint8_t* tgt;
  int tw, tx, ty;  // target width, crop origin in target coordinates
  int mode;
};

__global__ void prep_grid_kernel(PrepArgs A, uint8_t* __restrict__ mask, float* __restrict__ xa,
                                 float* __restrict__ xb, float* __restrict__ g) {
  const GridGeom& G = A.G;
  const long long total = (long long)G.n * G.m;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(q / G.m), j = (int)(q % G.m);
    const long long p = G.at(i, j);
    const bool on = A.m01[(long long)(A.x0 + i) * A.mw + (A.y0 + j)] != 0;
    mask[p] = on;
    const long long sc = ((long long)(A.sx + i) * A.sw + (A.sy + j)) * 3;
    const long long tc = ((long long)(A.tx + i) * A.tw + (A.ty + j)) * 3;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float t = (float)A.tgt[tc + c];
      xa[c * G.plane + p] = t;
      xb[c * G.plane + p] = t;
      float acc = 0.0f;
      if (on) {  // set pixels are never on the crop border: all 4 neighbours exist
        const float s0 = (float)A.src[sc + c];
        const long long su = sc - (long long)A.sw * 3, sd = sc + (long long)A.sw * 3;
        const long long tu = tc - (long long)A.tw * 3, td = tc + (long long)A.tw * 3;
        acc = __fadd_rn(acc, mix_term(s0 - A.src[su + c], t - A.tgt[tu + c], A.mode));
        acc = __fadd_rn(acc, mix_term(s0 - A.src[sd + c], t - A.tgt[td + c], A.mode));
        acc = __fadd_rn(acc, mix_term(s0 - A.src[sc - 3 + c], t - A.tgt[tc - 3 + c], A.mode));
        acc = __fadd_rn(acc, mix_term(s0 - A.src[sc + 3 + c], t - A.tgt[tc + 3 + c], A.mode));
      }
      g[c * G.plane + p] = acc;
    }
  }
}

void launch_prep_mask(const uint8_t* mask, int mh, int mw, int mch, uint8_t* m01, int* box,
                      cudaStream_t st) {
  const long long total = (long long)mh * mw;
  const int blocks = (int)std::max<long long>(1, std::min<long long>((total + 255) / 256, 152 * 16));
  prep_mask_kernel<<<blocks, 256, 0, st>>>(mask, mh, mw, mch, m01, box);
}

void launch_prep_grid(const PrepArgs& a, uint8_t* mask, float* xa, float* xb, float* g,
                      cudaStream_t st) {
  const long long total = (long long)a.G.n * a.G.m;
  const int blocks = (int)std::max<long long>(1, std::min<long long>((total + 255) / 256, 152 * 32));
  prep_grid_kernel<<<blocks, 256, 0, st>>>(a, mask, xa, xb, g);
}

}  // namespace fpie
