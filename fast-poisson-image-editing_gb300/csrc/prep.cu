// GPU-side construction of the grid solver's inputs from the three images.
//
// Same results as the host path (GridProcessor.reset, fpie/process.py:321-386),
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
#include "prep.cuh"

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
  const int blocks = stride_blocks(total, 256, 16);
  prep_mask_kernel<<<blocks, 256, 0, st>>>(mask, mh, mw, mch, m01, box);
}

void launch_prep_grid(const PrepArgs& a, uint8_t* mask, float* xa, float* xb, float* g,
                      cudaStream_t st) {
  const long long total = (long long)a.G.n * a.G.m;
  const int blocks = stride_blocks(total, 256, 32);
  prep_grid_kernel<<<blocks, 256, 0, st>>>(a, mask, xa, xb, g);
}

}  // namespace fpie

// ---- equation form ---------------------------------------------------------------
// ids: 1-based row-major ranks of the set pixels of the crop (the reference's
// partition + ids[mask == 0] = 0, fpie/process.py:180-190), by a three-step
// scan over blocks of kScanTile pixels.  Red-black numbering (the OpenMP
// EquSolver's partition, fpie/core/openmp/equ.cc:22-56): the same scan over
// the cells with odd row + col of the crop, then over the even ones, whose
// ranks continue after the odd count.
namespace fpie {

constexpr int kScanTile = 1024;  // 256 threads x 4 pixels

struct CropView {
  const uint8_t* m01;
  int mw, x0, y0, n, m;
  int parity = -1;  // 0 / 1: only the cells with that parity of row + col count as set
  __device__ __forceinline__ int at(long long q) const {
    const int i = (int)(q / m), j = (int)(q % m);
    if (parity >= 0 && ((i + j) & 1) != parity) return 0;
    return m01[(long long)(x0 + i) * mw + (y0 + j)];
  }
};

__global__ void __launch_bounds__(256) scan_count_kernel(CropView V, int* __restrict__ counts) {
  const long long total = (long long)V.n * V.m;
  const long long start = (long long)blockIdx.x * kScanTile;
  int c = 0;
  for (int k = threadIdx.x; k < kScanTile; k += blockDim.x)
    if (start + k < total) c += V.at(start + k) != 0;
  __shared__ int warp_sum[8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < 8; ++w) s += warp_sum[w];
    counts[blockIdx.x] = s;
  }
}

// One block: exclusive scan of the block counts in place; total at counts[nb].
__global__ void __launch_bounds__(1024) scan_offsets_kernel(int* __restrict__ counts, int nb) {
  __shared__ int carry;
  __shared__ int sh[1024];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += 1024) {
    const int k = base + threadIdx.x;
    const int v = k < nb ? counts[k] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {  // inclusive Hillis-Steele scan
      const int t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
      __syncthreads();
      sh[threadIdx.x] += t;
      __syncthreads();
    }
    if (k < nb) counts[k] = carry + sh[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += sh[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) counts[nb] = carry;
}

// base: added to every rank (NULL: 0); keep_others: leave the ids of cells
// that do not count as set (second pass of the red-black numbering).
__global__ void __launch_bounds__(256) scan_ids_kernel(CropView V, const int* __restrict__ offsets,
                                                      int* __restrict__ ids,
                                                      const int* __restrict__ base,
                                                      bool keep_others) {
  const long long total = (long long)V.n * V.m;
  const long long start = (long long)blockIdx.x * kScanTile + threadIdx.x * 4;
  int on[4], c = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    on[k] = start + k < total ? V.at(start + k) != 0 : 0;
    c += on[k];
  }
  // exclusive scan of c over the block
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int incl = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  __shared__ int warp_tot[8];
  if (lane == 31) warp_tot[w] = incl;
  __syncthreads();
  int before = 0;
  for (int k = 0; k < w; ++k) before += warp_tot[k];
  int rank = (base ? *base : 0) + offsets[blockIdx.x] + before + incl - c;
#pragma unroll
  for (int k = 0; k < 4; ++k)
    if (start + k < total && (on[k] || !keep_others)) ids[start + k] = on[k] ? ++rank : 0;
}

// counts[nb] = odd + even unknowns, counts[nb + 1] = odd ones.
__global__ void rb_total_kernel(int* counts, int nb) { counts[nb] += counts[nb + 1]; }

struct EquPrepArgs {
  CropView V;
  const int* ids;  // crop-sized
  const uint8_t* src;
  int sw, sx, sy;
  const uint8_t* tgt;
  int tw, tx, ty;
  int mode;
  long long np;    // plane stride of X/B
};

__device__ __forceinline__ float mix_term2(float a, float b, int mode) {
  if (mode == 0) return a;
  if (mode == 1) return __fmul_rn(__fadd_rn(a, b), 0.5f);
  return fabsf(a) < fabsf(b) ? b : a;
}

// Row id of every set pixel: A = ids of (up, down, left, right), X = target,
// B = grad (L, R, U, D order) + target values of unset neighbours (U, L, R,
// D order), and the pixel's target coordinates (fpie/process.py:227-269).
__global__ void equ_build_kernel(EquPrepArgs P, int4* __restrict__ A, float* __restrict__ x0,
                                 float* __restrict__ x1, float* __restrict__ b,
                                 int* __restrict__ rows, int* __restrict__ cols) {
  const CropView& V = P.V;
  const long long total = (long long)V.n * V.m;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int id = P.ids[q];
    if (!id) continue;
    const int i = (int)(q / V.m), j = (int)(q % V.m);
    // set pixels are never on the crop border: all four neighbours exist
    const int iu = P.ids[q - V.m], idn = P.ids[q + V.m], il = P.ids[q - 1], ir = P.ids[q + 1];
    A[id] = make_int4(iu, idn, il, ir);
    rows[id - 1] = P.tx + i;
    cols[id - 1] = P.ty + j;
    const long long sc = ((long long)(P.sx + i) * P.sw + (P.sy + j)) * 3;
    const long long tc = ((long long)(P.tx + i) * P.tw + (P.ty + j)) * 3;
    const long long srow = (long long)P.sw * 3, trow = (long long)P.tw * 3;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float s0 = (float)P.src[sc + c], t0 = (float)P.tgt[tc + c];
      const float tu = P.tgt[tc - trow + c], td = P.tgt[tc + trow + c];
      const float tl = P.tgt[tc - 3 + c], tr = P.tgt[tc + 3 + c];
      float gsum = __fadd_rn(mix_term2(s0 - P.src[sc - 3 + c], t0 - tl, P.mode),
                             mix_term2(s0 - P.src[sc + 3 + c], t0 - tr, P.mode));
      gsum = __fadd_rn(gsum, mix_term2(s0 - P.src[sc - srow + c], t0 - tu, P.mode));
      gsum = __fadd_rn(gsum, mix_term2(s0 - P.src[sc + srow + c], t0 - td, P.mode));
      float bv = gsum;
      if (!iu) bv = __fadd_rn(bv, tu);
      if (!il) bv = __fadd_rn(bv, tl);
      if (!ir) bv = __fadd_rn(bv, tr);
      if (!idn) bv = __fadd_rn(bv, td);
      x0[c * P.np + id] = t0;
      x1[c * P.np + id] = t0;
      b[c * P.np + id] = bv;
    }
  }
}

int launch_equ_ids(const uint8_t* m01, int mw, int x0, int y0, int n, int m, int* counts,
                   int* ids, cudaStream_t st, bool red_black) {
  CropView V{m01, mw, x0, y0, n, m};
  const long long total = (long long)n * m;
  const int nb = (int)((total + kScanTile - 1) / kScanTile);
  if (!red_black) {
    scan_count_kernel<<<nb, 256, 0, st>>>(V, counts);
    scan_offsets_kernel<<<1, 1024, 0, st>>>(counts, nb);
    scan_ids_kernel<<<nb, 256, 0, st>>>(V, counts, ids, nullptr, false);
    return nb;
  }
  V.parity = 1;  // odd cells: ids 1.., every other cell 0
  scan_count_kernel<<<nb, 256, 0, st>>>(V, counts);
  scan_offsets_kernel<<<1, 1024, 0, st>>>(counts, nb);
  scan_ids_kernel<<<nb, 256, 0, st>>>(V, counts, ids, nullptr, false);
  FPIE_CUDA(cudaMemcpyAsync(counts + nb + 1, counts + nb, sizeof(int), cudaMemcpyDeviceToDevice, st));
  V.parity = 0;  // even cells: ids after the odd count
  scan_count_kernel<<<nb, 256, 0, st>>>(V, counts);
  scan_offsets_kernel<<<1, 1024, 0, st>>>(counts, nb);
  scan_ids_kernel<<<nb, 256, 0, st>>>(V, counts, ids, counts + nb + 1, true);
  rb_total_kernel<<<1, 1, 0, st>>>(counts, nb);
  return nb;
}

void launch_equ_build(const uint8_t* m01, int mw, int x0, int y0, int n, int m, const int* ids,
                      const uint8_t* src, int sw, int sx, int sy, const uint8_t* tgt, int tw,
                      int tx, int ty, int mode, long long np, int4* A, float* xa, float* xb,
                      float* b, int* rows, int* cols, cudaStream_t st) {
  EquPrepArgs P{{m01, mw, x0, y0, n, m}, ids, src, sw, sx, sy, tgt, tw, tx, ty, mode, np};
  const long long total = (long long)n * m;
  const int blocks = stride_blocks(total, 256, 32);
  equ_build_kernel<<<blocks, 256, 0, st>>>(P, A, xa, xb, b, rows, cols);
}

}  // namespace fpie
