// Grid step that allocates nothing: fpie_grid_step_noalloc.
//
// For callers that cannot allocate device memory at the point where they
// need a Poisson step: hosts whose device memory belongs to their own pool
// allocator (memory taken behind its back breaks its accounting), and
// latency-critical loops where cudaMalloc/cudaFree (which may synchronize
// the device) are not acceptable.  They pass every input and
// output buffer; the one buffer the step needs beyond those -- the second
// Jacobi state and the residual partials -- is a fixed array in the
// library's device image, sized for grids of at most kNoAllocMaxPixels
// pixels (3 MiB + 24 KiB, held on every GPU that loads the library until
// the process exits).
//
// Layout is the reference's own ([n][m][3] float32 state, [n][m] int32
// mask), so a caller needs no conversion.  Arithmetic is the numpy
// backend's order, exactly as in the solver objects' kernels, so the state
// and image after k sweeps are bit-identical to GridSolver's; err sums the
// same per-pixel terms in double in another fixed order (256-pixel blocks),
// so it agrees with GridSolver's to float rounding.
//
// The scratch array is shared by every call on a device and keeps the last
// call's contents; everything a call reads from it is written by that call
// first.  Calls whose GPU work overlaps (two streams, or two host threads)
// race on it and must be serialized by the caller.
#include <mutex>

#include "common.cuh"

namespace fpie {

constexpr int kNoAllocMaxPixels = 1 << 18;  // 262,144 pixels, e.g. 512 x 512
constexpr int kNoAllocBlock = 256;
constexpr int kNoAllocMaxParts = kNoAllocMaxPixels / kNoAllocBlock;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) float g_noalloc_state[3 * kNoAllocMaxPixels];
static __device__ __align__(256) double g_noalloc_parts[3 * kNoAllocMaxParts];

// One sweep in the interleaved layout; unmasked pixels are copied so the
// output buffer holds the full state.  Neighbours outside the grid read 0.
__global__ void __launch_bounds__(kNoAllocBlock)
noalloc_sweep_kernel(int n, int m, const int32_t* __restrict__ mask,
                     const float* __restrict__ grad,
                     const float* __restrict__ xin, float* __restrict__ xout) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n * m) return;
  const int i = p / m, j = p - i * m;
  const bool on = mask[p] != 0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float xc = xin[p * 3 + c];
    float o = xc;
    if (on) {
      const float u = i > 0 ? xin[(p - m) * 3 + c] : 0.0f;
      const float d = i < n - 1 ? xin[(p + m) * 3 + c] : 0.0f;
      const float l = j > 0 ? xin[(p - 1) * 3 + c] : 0.0f;
      const float r = j < m - 1 ? xin[(p + 1) * 3 + c] : 0.0f;
      o = jacobi5(grad[p * 3 + c], u, d, l, r);
    }
    xout[p * 3 + c] = o;
  }
}

// Per-block sums of |residual| (numpy order) into parts; clipped image.
__global__ void __launch_bounds__(kNoAllocBlock)
noalloc_finish_kernel(int n, int m, const int32_t* __restrict__ mask,
                      const float* __restrict__ grad, const float* __restrict__ x,
                      uint8_t* __restrict__ img, double* __restrict__ parts) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[3] = {0.0, 0.0, 0.0};
  if (p < n * m) {
    const int i = p / m, j = p - i * m;
    const bool on = mask[p] != 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float xc = x[p * 3 + c];
      if (on) {
        const float u = i > 0 ? x[(p - m) * 3 + c] : 0.0f;
        const float d = i < n - 1 ? x[(p + m) * 3 + c] : 0.0f;
        const float l = j > 0 ? x[(p - 1) * 3 + c] : 0.0f;
        const float r = j < m - 1 ? x[(p + 1) * 3 + c] : 0.0f;
        acc[c] = fabsf(grid_res(xc, grad[p * 3 + c], u, d, l, r));
      }
      if (img) img[p * 3 + c] = clip_u8(xc);
    }
  }
  block_sum3(acc[0], acc[1], acc[2]);
  if (threadIdx.x == 0) {
    parts[3 * blockIdx.x + 0] = acc[0];
    parts[3 * blockIdx.x + 1] = acc[1];
    parts[3 * blockIdx.x + 2] = acc[2];
  }
}

namespace {

struct NoAllocScratch {
  float* state = nullptr;
  double* parts = nullptr;
};

std::mutex g_noalloc_mu;
NoAllocScratch g_noalloc_dev[kNoAllocMaxDevices];

// Device addresses of the scratch arrays on the current device.  The first
// call on a device resolves them (cudaGetSymbolAddress, which also loads the
// library's module on that device) and loads the kernels, so later calls do
// no set-up; that first call should come before any stream capture.  The
// addresses are kept for the life of the process, so the entry point must
// not be used across a cudaDeviceReset of the device (the module would be
// loaded again at other addresses).
NoAllocScratch noalloc_scratch() {
  int dev = 0;
  FPIE_CUDA(cudaGetDevice(&dev));
  FPIE_REQUIRE(dev >= 0 && dev < kNoAllocMaxDevices, FPIE_ERR_ARG,
               "device ordinal beyond the no-allocation entry point's table");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  NoAllocScratch& s = g_noalloc_dev[dev];
  if (s.state == nullptr) {
    float* st = nullptr;
    double* pa = nullptr;
    FPIE_CUDA(cudaGetSymbolAddress((void**)&st, g_noalloc_state));
    FPIE_CUDA(cudaGetSymbolAddress((void**)&pa, g_noalloc_parts));
    cudaFuncAttributes attr;
    FPIE_CUDA(cudaFuncGetAttributes(&attr, noalloc_sweep_kernel));
    FPIE_CUDA(cudaFuncGetAttributes(&attr, noalloc_finish_kernel));
    s.state = st;
    s.parts = pa;
  }
  return s;
}

}  // namespace
}  // namespace fpie

using namespace fpie;

extern "C" int fpie_grid_step_noalloc(int n, int m, const int32_t* mask,
                                      float* x, const float* grad,
                                      int iteration, uint8_t* img, float* err,
                                      void* stream) {
  return guarded([&] {
    FPIE_REQUIRE(n >= 1 && m >= 1, FPIE_ERR_ARG, "grid must be at least 1x1");
    FPIE_REQUIRE((long long)n * m <= kNoAllocMaxPixels, FPIE_ERR_ARG,
                 "grid of " + std::to_string((long long)n * m) +
                     " pixels exceeds the no-allocation limit of " +
                     std::to_string(kNoAllocMaxPixels) + " pixels");
    FPIE_REQUIRE(mask && x && grad, FPIE_ERR_ARG, "null input array");
    const NoAllocScratch s = noalloc_scratch();
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int px = n * m;
    const int blocks = (px + kNoAllocBlock - 1) / kNoAllocBlock;
    float* bufs[2] = {x, s.state};
    int cur = 0;
    for (int k = 0; k < iteration; ++k, cur ^= 1) {
      noalloc_sweep_kernel<<<blocks, kNoAllocBlock, 0, st>>>(n, m, mask, grad,
                                                             bufs[cur], bufs[cur ^ 1]);
      FPIE_CUDA(cudaGetLastError());
    }
    if (cur == 1)  // an odd count left the state in the scratch array
      FPIE_CUDA(cudaMemcpyAsync(x, s.state, (size_t)px * 3 * sizeof(float),
                                cudaMemcpyDeviceToDevice, st));
    if (img || err) {
      noalloc_finish_kernel<<<blocks, kNoAllocBlock, 0, st>>>(n, m, mask, grad, x,
                                                              img, s.parts);
      FPIE_CUDA(cudaGetLastError());
      if (err) {
        launch_finalize(s.parts, blocks, err, st);
        FPIE_CUDA(cudaGetLastError());
      }
    }
  });
}
