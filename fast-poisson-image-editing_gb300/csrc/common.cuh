// Shared definitions of the fpie_gb300 CUDA backend: error plumbing, the
// solver handle, and the small device helpers every kernel uses.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>

#include "fpie_gb300.h"

namespace fpie {

// ---- error reporting ------------------------------------------------------
void set_error(const std::string& msg);
void clear_error();

struct Error {
  int code;
  std::string msg;
};

#define FPIE_CUDA(call)                                                     \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) {                                                \
      throw ::fpie::Error{FPIE_ERR_CUDA, std::string(#call) + ": " +        \
                                             cudaGetErrorString(e_)};       \
    }                                                                       \
  } while (0)

#define FPIE_REQUIRE(cond, code, msg)                   \
  do {                                                  \
    if (!(cond)) throw ::fpie::Error{(code), (msg)};    \
  } while (0)

// Runs `body` and converts exceptions to a status code + last-error string.
template <class F>
int guarded(F&& body) {
  try {
    clear_error();
    body();
    return FPIE_OK;
  } catch (const Error& e) {
    set_error(e.msg);
    return e.code;
  } catch (const std::exception& e) {
    set_error(e.what());
    return FPIE_ERR_STATE;
  }
}

// Blocks for a grid-stride loop over `total` elements, `threads` per block:
// one block per `threads` elements, at most `per_sm` blocks per SM of the
// current device (its multiprocessor count is read once per device), at
// least 1.
int stride_blocks(long long total, int threads, int per_sm);

// Stream-ordered device scratch that is released on every exit path,
// exceptions included (cudaFreeAsync on the stream it was allocated on).
// The library's stream-ordered scratch pool on the current device.  Unlike
// the device's default pool (release threshold 0: freed memory goes back to
// the driver at every synchronize, and the next reset maps it again), it
// keeps up to 4 GiB of freed scratch for reuse.
cudaMemPool_t scratch_pool();

struct AsyncScratch {
  void* ptr = nullptr;
  cudaStream_t stream = nullptr;
  AsyncScratch(size_t bytes, cudaStream_t st) : stream(st) {
    FPIE_CUDA(cudaMallocFromPoolAsync(&ptr, bytes, scratch_pool(), st));
  }
  ~AsyncScratch() {
    if (ptr) cudaFreeAsync(ptr, stream);
  }
  AsyncScratch(const AsyncScratch&) = delete;
  AsyncScratch& operator=(const AsyncScratch&) = delete;
  char* bytes() const { return static_cast<char*>(ptr); }
};

// ---- grid geometry ----------------------------------------------------------
// The grid state lives in HBM as three planar float32 channel planes with a
// zero halo of kPad rows above and kPad columns left of the crop, and
// kPad + slack rows/columns below and right of it.
// Rows are `pitch` floats apart, pitch a multiple of 32 (128 bytes), so the
// first crop column of every row is 16-byte aligned.  The halo lets every
// tile (including its temporal-blocking apron) be read without bounds checks.
constexpr int kPad = 32;

struct GridGeom {
  int n, m;          // crop rows, columns
  int pitch;         // floats per padded row
  int rows;          // n + 2*kPad + kSlackRows
  long long plane;   // floats per channel plane (pitch * rows)
  __host__ __device__ long long at(int i, int j) const {
    return (long long)(i + kPad) * pitch + (j + kPad);
  }
};

// Rows/columns reserved past the crop's far edges beyond kPad, so that the
// last tile of any temporally blocked variant (tile up to 224 rows / 120
// columns plus its apron) reads and writes inside the allocation.
constexpr int kSlackRows = 256;
constexpr int kSlackCols = 128;

inline GridGeom make_geom(int n, int m) {
  GridGeom g;
  g.n = n;
  g.m = m;
  g.pitch = ((m + 2 * kPad + kSlackCols) + 31) / 32 * 32;
  g.rows = n + 2 * kPad + kSlackRows;
  g.plane = (long long)g.pitch * g.rows;
  return g;
}

// ---- device helpers -----------------------------------------------------------
// The update keeps the numpy backend's evaluation order exactly:
// ((((g + up) + down) + left) + right) * 0.25  (x/4 and x*0.25 round alike).
// __fadd_rn/__fmul_rn are never contracted into FMAs.
__device__ __forceinline__ float jacobi5(float g, float u, float d, float l,
                                         float r) {
  return __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(g, u), d), l), r),
                   0.25f);
}

// Grid residual in the numpy backend's order: 4x - g - up - down - left - right.
__device__ __forceinline__ float grid_res(float x, float g, float u, float d,
                                          float l, float r) {
  float t = __fsub_rn(__fmul_rn(4.0f, x), g);
  t = __fsub_rn(t, u);
  t = __fsub_rn(t, d);
  t = __fsub_rn(t, l);
  return __fsub_rn(t, r);
}

// Clamp to [0,255] and truncate, as the reference's uint8 store does.
__device__ __forceinline__ uint8_t clip_u8(float v) {
  v = fminf(fmaxf(v, 0.0f), 255.0f);
  return (uint8_t)__float2int_rz(v);
}

__device__ __forceinline__ float4 ld4(const float* p) {
  return __ldg(reinterpret_cast<const float4*>(p));
}

// Block-wide sum of three doubles; the result is valid in thread 0.
// blockDim.x * blockDim.y must be a multiple of 32 and at most 1024.
__device__ __forceinline__ void block_sum3(double& a, double& b, double& c) {
  __shared__ double sh[3][32];
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int nwarps = (blockDim.x * blockDim.y) >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
    c += __shfl_down_sync(0xffffffffu, c, o);
  }
  if (lane == 0) {
    sh[0][warp] = a;
    sh[1][warp] = b;
    sh[2][warp] = c;
  }
  __syncthreads();
  if (warp == 0) {
    a = lane < nwarps ? sh[0][lane] : 0.0;
    b = lane < nwarps ? sh[1][lane] : 0.0;
    c = lane < nwarps ? sh[2][lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
      c += __shfl_down_sync(0xffffffffu, c, o);
    }
  }
}

// Sums `nparts` per-block partials (3 doubles each) into err[3] (float) in a
// fixed order, so the result does not depend on block scheduling.
void launch_finalize(const double* parts, int nparts, float* err,
                     cudaStream_t st);

// ---- solver handle -----------------------------------------------------------
struct Solver {
  int kind = 0;  // 1 = equ, 2 = grid
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;  // where work is enqueued
  long long launches = 0;
  int precision = FPIE_FP32;
  virtual ~Solver() {}
  // Raises the error a kernel recorded in device memory (e.g. a bounded wait
  // that timed out); called after the stream has been synchronised.
  virtual void check_async() {}
  void activate() const { FPIE_CUDA(cudaSetDevice(device)); }
};

Solver* new_equ_solver(int block_size);
Solver* new_grid_solver(int grid_x, int grid_y);

inline Solver* check_handle(fpie_solver* s, int kind) {
  FPIE_REQUIRE(s != nullptr, FPIE_ERR_ARG, "null solver handle");
  Solver* h = reinterpret_cast<Solver*>(s);
  if (kind) FPIE_REQUIRE(h->kind == kind, FPIE_ERR_ARG, "wrong solver kind for this call");
  h->activate();
  return h;
}

// Launch-configuration check: every launch is followed by this, so a bad
// configuration surfaces as an error status at the call that caused it.
inline void post_launch(Solver* s, int n = 1) {
  s->launches += n;
  FPIE_CUDA(cudaGetLastError());
}

}  // namespace fpie
