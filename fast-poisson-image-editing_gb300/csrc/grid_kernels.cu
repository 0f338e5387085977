// Grid sweep and finish kernels (FP32, one sweep per launch).
//
// Each thread owns four horizontally adjacent pixels of one row (one float4
// per channel plane).  A warp covers 128 consecutive columns, so every
// plane access is a 512-byte coalesced run; the left/right neighbours of the
// group's end pixels come from two scalar loads that hit the same L1 lines.
// Groups with no masked pixel do nothing: their values never change and both
// state buffers already hold them.
#include "grid_kernels.cuh"

namespace fpie {

constexpr int kSweepBX = 64, kSweepBY = 4;

__global__ void __launch_bounds__(kSweepBX * kSweepBY)
grid_sweep_kernel(GridGeom G, const uint8_t* __restrict__ mask,
                  const float* __restrict__ g, const float* __restrict__ xin,
                  float* __restrict__ xout) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;  // 4-column group
  const int i = blockIdx.y * blockDim.y + threadIdx.y;  // crop row
  if (i >= G.n || 4 * q >= G.m) return;
  const long long p = G.at(i, 4 * q);
  const uint32_t mk = *reinterpret_cast<const uint32_t*>(mask + p);
  if (mk == 0u) return;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float* xc = xin + c * G.plane;
    const float4 ce = ld4(xc + p);
    const float4 up = ld4(xc + p - G.pitch);
    const float4 dn = ld4(xc + p + G.pitch);
    const float lf = __ldg(xc + p - 1);
    const float rt = __ldg(xc + p + 4);
    const float4 gg = ld4(g + c * G.plane + p);
    float4 o;
    o.x = (mk & 0x000000ffu) ? jacobi5(gg.x, up.x, dn.x, lf, ce.y) : ce.x;
    o.y = (mk & 0x0000ff00u) ? jacobi5(gg.y, up.y, dn.y, ce.x, ce.z) : ce.y;
    o.z = (mk & 0x00ff0000u) ? jacobi5(gg.z, up.z, dn.z, ce.y, ce.w) : ce.z;
    o.w = (mk & 0xff000000u) ? jacobi5(gg.w, up.w, dn.w, ce.z, rt) : ce.w;
    *reinterpret_cast<float4*>(xout + c * G.plane + p) = o;
  }
}

__global__ void __launch_bounds__(kSweepBX * kSweepBY)
grid_finish_kernel(GridGeom G, const uint8_t* __restrict__ mask,
                   const float* __restrict__ g, const float* __restrict__ x,
                   uint8_t* __restrict__ img, double* __restrict__ parts) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  double acc[3] = {0.0, 0.0, 0.0};
  if (i < G.n && 4 * q < G.m) {
    const long long p = G.at(i, 4 * q);
    const uint32_t mk = *reinterpret_cast<const uint32_t*>(mask + p);
    const int jn = min(4, G.m - 4 * q);
    uint8_t* out = img + ((long long)i * G.m + 4 * q) * 3;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float* xc = x + c * G.plane;
      const float4 ce = ld4(xc + p);
      if (mk) {
        const float4 up = ld4(xc + p - G.pitch);
        const float4 dn = ld4(xc + p + G.pitch);
        const float lf = __ldg(xc + p - 1);
        const float rt = __ldg(xc + p + 4);
        const float4 gg = ld4(g + c * G.plane + p);
        // Per-pixel |r| is exact float32 (numpy order); the sums are double.
        if (mk & 0x000000ffu) acc[c] += fabsf(grid_res(ce.x, gg.x, up.x, dn.x, lf, ce.y));
        if (mk & 0x0000ff00u) acc[c] += fabsf(grid_res(ce.y, gg.y, up.y, dn.y, ce.x, ce.z));
        if (mk & 0x00ff0000u) acc[c] += fabsf(grid_res(ce.z, gg.z, up.z, dn.z, ce.y, ce.w));
        if (mk & 0xff000000u) acc[c] += fabsf(grid_res(ce.w, gg.w, up.w, dn.w, ce.z, rt));
      }
      const float v[4] = {ce.x, ce.y, ce.z, ce.w};
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (k < jn) out[k * 3 + c] = clip_u8(v[k]);
    }
  }
  block_sum3(acc[0], acc[1], acc[2]);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    const long long b = blockIdx.y * (long long)gridDim.x + blockIdx.x;
    parts[3 * b + 0] = acc[0];
    parts[3 * b + 1] = acc[1];
    parts[3 * b + 2] = acc[2];
  }
}

GridLaunch grid_launch(const GridGeom& G) {
  GridLaunch L;
  const int groups = (G.m + 3) / 4;
  L.sweep_block = dim3(kSweepBX, kSweepBY);
  L.sweep_grid = dim3((groups + kSweepBX - 1) / kSweepBX, (G.n + kSweepBY - 1) / kSweepBY);
  L.finish_block = L.sweep_block;
  L.finish_grid = L.sweep_grid;
  L.nparts = (int)(L.finish_grid.x * L.finish_grid.y);
  return L;
}

void launch_grid_sweep(const GridLaunch& L, const GridGeom& G,
                       const uint8_t* mask, const float* g, const float* xin,
                       float* xout, cudaStream_t st) {
  grid_sweep_kernel<<<L.sweep_grid, L.sweep_block, 0, st>>>(G, mask, g, xin, xout);
}

void launch_grid_finish(const GridLaunch& L, const GridGeom& G,
                        const uint8_t* mask, const float* g, const float* x,
                        uint8_t* img, double* parts, cudaStream_t st) {
  grid_finish_kernel<<<L.finish_grid, L.finish_block, 0, st>>>(G, mask, g, x, img, parts);
}

}  // namespace fpie
