// FP32 pipe throughput probe: the denominator of the sweep kernels' compute
// roofline.
//
// The sweep kernels are bound by FP32 issue, not by memory: every pixel
// update is four additions and one multiplication per channel, issued as
// packed FP32x2 instructions (two values per lane).  This probe measures
// how many such operations per second the device sustains when nothing
// else competes: every thread advances eight independent chains of packed
// operations (enough independent work to cover the pipe latency at 64
// warps per SM), the launch is timed with CUDA events on the caller's
// stream, and the rate counts one operation per value (a packed add is two
// operations, as the sweep's additions are counted).
#include <algorithm>

#include "common.cuh"

namespace fpie {

namespace {

constexpr int kChains = 8;
constexpr int kUnroll = 4;

// KIND 0: packed add (__fadd2_rn), 1: packed multiply (__fmul2_rn), 2: packed
// fused multiply-add (__ffma2_rn), 3: scalar add.
template <int KIND>
__global__ void __launch_bounds__(256) probe_fp32_kernel(int iters, float* sink) {
  const float s = 1.0f + 1e-7f * (float)(threadIdx.x & 7);
  float2 a[kChains];
#pragma unroll
  for (int j = 0; j < kChains; ++j) a[j] = make_float2(s * (float)(j + 1), s * (float)(j + 2));
  const float2 b = make_float2(1e-7f, 2e-7f);
  const float2 m = make_float2(0.9999999f, 1.0000001f);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
#pragma unroll
      for (int j = 0; j < kChains; ++j) {
        if (KIND == 0) a[j] = __fadd2_rn(a[j], b);
        if (KIND == 1) a[j] = __fmul2_rn(a[j], m);
        if (KIND == 2) a[j] = __ffma2_rn(a[j], m, b);
        if (KIND == 3) {
          a[j].x = __fadd_rn(a[j].x, b.x);
          a[j].y = __fadd_rn(a[j].y, b.y);
        }
      }
    }
  }
  float acc = 0.f;
#pragma unroll
  for (int j = 0; j < kChains; ++j) acc += a[j].x + a[j].y;
  // Never true for these inputs; keeps the chains from being removed.
  if (acc == -1.0f) sink[blockIdx.x] = acc;
}

}  // namespace

}  // namespace fpie

using namespace fpie;

extern "C" {

int fpie_probe_fp32_rate(void* stream, int kind, int iters, double* ops_per_s) {
  return guarded([&] {
    FPIE_REQUIRE(ops_per_s != nullptr, FPIE_ERR_ARG, "null output pointer");
    FPIE_REQUIRE(kind >= 0 && kind <= 3, FPIE_ERR_ARG, "kind must be 0..3");
    FPIE_REQUIRE(iters >= 1 && iters <= (1 << 24), FPIE_ERR_ARG, "iters out of range");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    int dev = 0, sms = 0;
    FPIE_CUDA(cudaGetDevice(&dev));
    FPIE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, threads = 256;
    float* sink = nullptr;
    FPIE_CUDA(cudaMallocAsync(&sink, sizeof(float) * blocks, st));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float ms = 0.f;
    try {
      FPIE_CUDA(cudaEventCreate(&e0));
      FPIE_CUDA(cudaEventCreate(&e1));
      auto launch = [&](int n) {
        switch (kind) {
          case 0: probe_fp32_kernel<0><<<blocks, threads, 0, st>>>(n, sink); break;
          case 1: probe_fp32_kernel<1><<<blocks, threads, 0, st>>>(n, sink); break;
          case 2: probe_fp32_kernel<2><<<blocks, threads, 0, st>>>(n, sink); break;
          default: probe_fp32_kernel<3><<<blocks, threads, 0, st>>>(n, sink); break;
        }
        FPIE_CUDA(cudaGetLastError());
      };
      launch(std::max(1, iters / 8));  // warm-up: clocks up, code loaded
      FPIE_CUDA(cudaEventRecord(e0, st));
      launch(iters);
      FPIE_CUDA(cudaEventRecord(e1, st));
      FPIE_CUDA(cudaEventSynchronize(e1));
      FPIE_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    } catch (...) {
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
      cudaFreeAsync(sink, st);
      throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    FPIE_CUDA(cudaFreeAsync(sink, st));
    FPIE_REQUIRE(ms > 0.f, FPIE_ERR_STATE, "probe launch took no measurable time");
    // Operations per launch: every thread, every iteration, kUnroll x kChains
    // packed instructions of two values each.
    const double ops = (double)blocks * threads * iters * kUnroll * kChains * 2.0;
    *ops_per_s = ops / (ms * 1e-3);
  });
}

}  // extern "C"
