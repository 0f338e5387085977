// Mixed-precision iterative refinement for the grid form.
//
// The FP32 solution x is kept; every cycle
//   1. refine: x <- x + e (e: the correction, FP16 or BF16), then the FP32
//      residual r = grad + up + down + left + right - 4x on masked pixels,
//      with its per-channel max |r| and sum |r| reduced in FP64;
//   2. inner: Jacobi sweeps on the correction equation 4e - sum(e_nb) = r,
//      e starting at 0 and kept at 0 on unmasked pixels, FP32 arithmetic,
//      e stored in FP16/BF16 between launches (grid_tbp.cu, storage type TS).
// The FP64 norms are the only FP64 arithmetic; they decide convergence.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "common.cuh"
#include "grid_mixed.cuh"

namespace fpie {

template <typename TS>
__device__ __forceinline__ float to_f(TS v);
template <>
__device__ __forceinline__ float to_f<__half>(__half v) { return __half2float(v); }
template <>
__device__ __forceinline__ float to_f<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <>
__device__ __forceinline__ float to_f<float>(float v) { return v; }

template <typename TS>
__device__ __forceinline__ float4 ld4_any(const TS* p) {
  return make_float4(to_f(p[0]), to_f(p[1]), to_f(p[2]), to_f(p[3]));
}

// Block-wide max and sum of three doubles each; valid in thread 0.
__device__ __forceinline__ void block_maxsum3(double (&mx)[3], double (&sm)[3]) {
  __shared__ double sh[6][32];
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = (blockDim.x * blockDim.y) >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      mx[c] = fmax(mx[c], __shfl_down_sync(0xffffffffu, mx[c], o));
      sm[c] += __shfl_down_sync(0xffffffffu, sm[c], o);
    }
  if (lane == 0)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      sh[c][warp] = mx[c];
      sh[3 + c][warp] = sm[c];
    }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      mx[c] = lane < nwarps ? sh[c][lane] : 0.0;
      sm[c] = lane < nwarps ? sh[3 + c][lane] : 0.0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        mx[c] = fmax(mx[c], __shfl_down_sync(0xffffffffu, mx[c], o));
        sm[c] += __shfl_down_sync(0xffffffffu, sm[c], o);
      }
  }
}

// Thread = 4 adjacent pixels of one row, all channels (the one-sweep
// kernel's geometry).  e == nullptr: no fold (x is already current);
// r == nullptr: the residual is only reduced, not stored; parts == nullptr:
// no norm partials (the refinement cycles do not need them).
template <typename TS>
__global__ void __launch_bounds__(256)
grid_refine_kernel(GridGeom G, const uint8_t* __restrict__ mask, const float* __restrict__ g,
                   const float* __restrict__ xin, const TS* __restrict__ e,
                   float* __restrict__ xout, float* __restrict__ r,
                   double* __restrict__ parts) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  double mx[3] = {0.0, 0.0, 0.0}, sm[3] = {0.0, 0.0, 0.0};
  if (i < G.n && 4 * q < G.m) {
    const long long p = G.at(i, 4 * q);
    const uint32_t mk = *reinterpret_cast<const uint32_t*>(mask + p);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const long long o = c * G.plane + p;
      float4 ce = ld4(xin + o), up = ld4(xin + o - G.pitch), dn = ld4(xin + o + G.pitch);
      float lf = __ldg(xin + o - 1), rt = __ldg(xin + o + 4);
      if (e) {
        const float4 ec = ld4_any(e + o), eu = ld4_any(e + o - G.pitch), ed = ld4_any(e + o + G.pitch);
        ce = make_float4(__fadd_rn(ce.x, ec.x), __fadd_rn(ce.y, ec.y), __fadd_rn(ce.z, ec.z), __fadd_rn(ce.w, ec.w));
        up = make_float4(__fadd_rn(up.x, eu.x), __fadd_rn(up.y, eu.y), __fadd_rn(up.z, eu.z), __fadd_rn(up.w, eu.w));
        dn = make_float4(__fadd_rn(dn.x, ed.x), __fadd_rn(dn.y, ed.y), __fadd_rn(dn.z, ed.z), __fadd_rn(dn.w, ed.w));
        lf = __fadd_rn(lf, to_f(e[o - 1]));
        rt = __fadd_rn(rt, to_f(e[o + 4]));
        if (mk) *reinterpret_cast<float4*>(xout + o) = ce;
      }
      if (mk || r) {
        const float gv[4] = {__ldg(g + o), __ldg(g + o + 1), __ldg(g + o + 2), __ldg(g + o + 3)};
        const float xv[6] = {lf, ce.x, ce.y, ce.z, ce.w, rt};
        const float uv[4] = {up.x, up.y, up.z, up.w}, dv[4] = {dn.x, dn.y, dn.z, dn.w};
        float rr[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const bool on = (mk >> (8 * k)) & 0xffu;
          const float v = on ? -grid_res(xv[k + 1], gv[k], uv[k], dv[k], xv[k], xv[k + 2]) : 0.0f;
          rr[k] = v;
          mx[c] = fmax(mx[c], (double)fabsf(v));
          sm[c] += (double)fabsf(v);
        }
        if (r) *reinterpret_cast<float4*>(r + o) = make_float4(rr[0], rr[1], rr[2], rr[3]);
      }
    }
  }
  if (parts == nullptr) return;  // uniform: a kernel argument
  block_maxsum3(mx, sm);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    const long long b = blockIdx.y * (long long)gridDim.x + blockIdx.x;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      parts[6 * b + c] = mx[c];
      parts[6 * b + 3 + c] = sm[c];
    }
  }
}

__global__ void __launch_bounds__(256)
norms_finalize_kernel(const double* __restrict__ parts, int nparts, double* __restrict__ out) {
  double mx[3] = {0.0, 0.0, 0.0}, sm[3] = {0.0, 0.0, 0.0};
  for (int k = threadIdx.x; k < nparts; k += blockDim.x)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      mx[c] = fmax(mx[c], parts[6 * k + c]);
      sm[c] += parts[6 * k + 3 + c];
    }
  block_maxsum3(mx, sm);
  if (threadIdx.x == 0)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      out[c] = mx[c];
      out[3 + c] = sm[c];
    }
}

void launch_refine(int precision, dim3 grid, dim3 block, const GridGeom& G, const uint8_t* mask,
                   const float* g, const float* xin, const void* e, float* xout, float* r,
                   double* parts, cudaStream_t st) {
  if (precision == FPIE_MIXED_BF16)
    grid_refine_kernel<__nv_bfloat16><<<grid, block, 0, st>>>(
        G, mask, g, xin, static_cast<const __nv_bfloat16*>(e), xout, r, parts);
  else if (precision == FPIE_MIXED_FP16)
    grid_refine_kernel<__half><<<grid, block, 0, st>>>(G, mask, g, xin,
                                                       static_cast<const __half*>(e), xout, r, parts);
  else
    grid_refine_kernel<float><<<grid, block, 0, st>>>(G, mask, g, xin,
                                                      static_cast<const float*>(e), xout, r, parts);
}

void launch_norms_finalize(const double* parts, int nparts, double* out, cudaStream_t st) {
  norms_finalize_kernel<<<1, 256, 0, st>>>(parts, nparts, out);
}

}  // namespace fpie
