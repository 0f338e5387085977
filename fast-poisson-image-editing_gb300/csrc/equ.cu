// EquSolver backend: Jacobi on the relabelled unknowns through the int32
// neighbour table A (row 0 is the constant-0 unknown absent neighbours use).
//
// Replaces fpie/core/cuda/equ.cu (CudaEquSolver) behind the plugin surface
// of fpie/core/base_solver.h:12-75.  Strict Jacobi with two state buffers,
// the numpy backend's order of additions (fpie/np_solver.py:31-54), planar
// channel arrays, a deterministic residual reduction, checked CUDA calls,
// and neighbour indices validated before any kernel reads through them.
#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace fpie {

void launch_prep_mask(const uint8_t* mask, int mh, int mw, int mch, uint8_t* m01, int* box,
                      cudaStream_t st);
int launch_equ_ids(const uint8_t* m01, int mw, int x0, int y0, int n, int m, int* counts,
                   int* ids, cudaStream_t st);
void launch_equ_build(const uint8_t* m01, int mw, int x0, int y0, int n, int m, const int* ids,
                      const uint8_t* src, int sw, int sx, int sy, const uint8_t* tgt, int tw,
                      int tx, int ty, int mode, long long np, int4* A, float* xa, float* xb,
                      float* b, int* rows, int* cols, cudaStream_t st);

// X[c][i] planes, `np` floats apart (N rounded up to 32).
struct EquGeom {
  int N;
  long long np;
};

__global__ void equ_pack_kernel(EquGeom E, const float* __restrict__ X,
                                const float* __restrict__ B,
                                float* __restrict__ x0, float* __restrict__ x1,
                                float* __restrict__ b) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < E.N;
       i += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      x0[c * E.np + i] = X[i * 3 + c];
      x1[c * E.np + i] = X[i * 3 + c];
      b[c * E.np + i] = B[i * 3 + c];
    }
  }
}

// Counts A entries outside [0, N) so no sweep ever gathers out of bounds.
__global__ void equ_check_kernel(EquGeom E, const int4* __restrict__ A,
                                 unsigned int* __restrict__ bad) {
  unsigned int nbad = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < E.N;
       i += (long long)gridDim.x * blockDim.x) {
    const int4 a = A[i];
    nbad += (unsigned)(a.x < 0 || a.x >= E.N) + (unsigned)(a.y < 0 || a.y >= E.N) +
            (unsigned)(a.z < 0 || a.z >= E.N) + (unsigned)(a.w < 0 || a.w >= E.N);
  }
  if (nbad) atomicAdd(bad, nbad);
}

__global__ void equ_unpack_kernel(EquGeom E, const float* __restrict__ x,
                                  float* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < E.N;
       i += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int c = 0; c < 3; ++c) out[i * 3 + c] = x[c * E.np + i];
  }
}

// One sweep over all rows (row 0 included, as in the numpy backend; with the
// processor's inputs it stays 0).  The neighbour gathers are mostly
// contiguous: left/right are i-1/i+1 and up/down one masked row away.
__global__ void equ_sweep_kernel(EquGeom E, const int4* __restrict__ A,
                                 const float* __restrict__ b,
                                 const float* __restrict__ xin,
                                 float* __restrict__ xout) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E.N) return;
  const int4 a = __ldg(A + i);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float* xc = xin + c * E.np;
    float s = __fadd_rn(__ldg(b + c * E.np + i), __ldg(xc + a.x));
    s = __fadd_rn(s, __ldg(xc + a.y));
    s = __fadd_rn(s, __ldg(xc + a.z));
    s = __fadd_rn(s, __ldg(xc + a.w));
    xout[c * E.np + i] = __fmul_rn(s, 0.25f);
  }
}

// Residual partials (B + sum X[A] - 4X, numpy order) and the clipped image.
__global__ void __launch_bounds__(256)
equ_finish_kernel(EquGeom E, const int4* __restrict__ A,
                  const float* __restrict__ b, const float* __restrict__ x,
                  uint8_t* __restrict__ img, double* __restrict__ parts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[3] = {0.0, 0.0, 0.0};
  if (i < E.N) {
    const int4 a = __ldg(A + i);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float* xc = x + c * E.np;
      float s = __fadd_rn(__ldg(b + c * E.np + i), __ldg(xc + a.x));
      s = __fadd_rn(s, __ldg(xc + a.y));
      s = __fadd_rn(s, __ldg(xc + a.z));
      s = __fadd_rn(s, __ldg(xc + a.w));
      const float xi = xc[i];
      acc[c] = fabsf(__fsub_rn(s, __fmul_rn(4.0f, xi)));
      img[(long long)i * 3 + c] = clip_u8(xi);
    }
  }
  block_sum3(acc[0], acc[1], acc[2]);
  if (threadIdx.x == 0) {
    parts[3 * (long long)blockIdx.x + 0] = acc[0];
    parts[3 * (long long)blockIdx.x + 1] = acc[1];
    parts[3 * (long long)blockIdx.x + 2] = acc[2];
  }
}

static int conv_blocks(long long total) {
  long long b = (total + 255) / 256;
  return (int)std::max<long long>(1, std::min<long long>(b, 152 * 32));
}

struct EquSolverImpl : Solver {
  int block = 256;
  bool ready = false;
  EquGeom E{0, 0};
  int4* A = nullptr;
  float* x[2] = {nullptr, nullptr};
  float* b = nullptr;
  int cur = 0;
  uint8_t* d_img = nullptr;
  double* d_part = nullptr;
  float* d_err = nullptr;
  unsigned int* d_bad = nullptr;
  uint8_t* h_img = nullptr;
  float* h_err = nullptr;
  unsigned int* h_bad = nullptr;
  int nparts = 0;
  static constexpr int kChunk = 64;
  cudaGraphExec_t chunk[2] = {nullptr, nullptr};

  explicit EquSolverImpl(int block_size) {
    kind = 1;
    if (block_size >= 32 && block_size <= 1024 && block_size % 32 == 0) block = block_size;
    FPIE_CUDA(cudaGetDevice(&device));
    FPIE_CUDA(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking));
    stream = own_stream;
    FPIE_CUDA(cudaMallocHost(&h_err, 3 * sizeof(float)));
    FPIE_CUDA(cudaMallocHost(&h_bad, sizeof(unsigned int)));
    FPIE_CUDA(cudaMalloc(&d_bad, sizeof(unsigned int)));
  }

  ~EquSolverImpl() override {
    release();
    cudaFree(d_rows);
    cudaFree(d_cols);
    cudaFree(d_bad);
    if (h_err) cudaFreeHost(h_err);
    if (h_bad) cudaFreeHost(h_bad);
    if (own_stream) cudaStreamDestroy(own_stream);
  }

  void drop_graphs() {
    for (auto& e : chunk) {
      if (e) cudaGraphExecDestroy(e);
      e = nullptr;
    }
  }

  void release() {
    cudaStreamSynchronize(stream);  // NULL (legacy default stream) included
    drop_graphs();
    cudaFree(A);
    cudaFree(x[0]);
    cudaFree(x[1]);
    cudaFree(b);
    cudaFree(d_img);
    cudaFree(d_part);
    cudaFree(d_err);
    if (h_img) cudaFreeHost(h_img);
    A = nullptr;
    x[0] = x[1] = b = nullptr;
    d_img = nullptr;
    d_part = nullptr;
    d_err = nullptr;
    h_img = nullptr;
    ready = false;
  }

  void allocate(int N) {
    FPIE_REQUIRE(N >= 1, FPIE_ERR_ARG, "N must be at least 1");
    FPIE_REQUIRE(N <= (1 << 29), FPIE_ERR_ARG, "N too large");
    if (A && E.N == N) {  // same size: keep buffers and captured graphs
      cur = 0;
      ready = false;
      return;
    }
    release();
    E.N = N;
    E.np = ((long long)N + 31) / 32 * 32;
    nparts = (N + 255) / 256;
    const size_t pb = (size_t)E.np * 3 * sizeof(float);
    FPIE_CUDA(cudaMalloc(&A, (size_t)N * sizeof(int4)));
    FPIE_CUDA(cudaMalloc(&x[0], pb));
    FPIE_CUDA(cudaMalloc(&x[1], pb));
    FPIE_CUDA(cudaMalloc(&b, pb));
    FPIE_CUDA(cudaMalloc(&d_img, (size_t)N * 3));
    FPIE_CUDA(cudaMalloc(&d_part, (size_t)nparts * 3 * sizeof(double)));
    FPIE_CUDA(cudaMalloc(&d_err, 3 * sizeof(float)));
    FPIE_CUDA(cudaMallocHost(&h_img, (size_t)N * 3));
    FPIE_CUDA(cudaMemsetAsync(x[0], 0, pb, stream));
    FPIE_CUDA(cudaMemsetAsync(x[1], 0, pb, stream));
    FPIE_CUDA(cudaMemsetAsync(b, 0, pb, stream));
    cur = 0;
  }

  // Packs X/B and validates A (already in device memory at this->A).
  void pack_and_check(const float* dX, const float* dB) {
    equ_pack_kernel<<<conv_blocks(E.N), 256, 0, stream>>>(E, dX, dB, x[0], x[1], b);
    post_launch(this);
    FPIE_CUDA(cudaMemsetAsync(d_bad, 0, sizeof(unsigned int), stream));
    equ_check_kernel<<<conv_blocks(E.N), 256, 0, stream>>>(E, A, d_bad);
    post_launch(this);
    FPIE_CUDA(cudaMemcpyAsync(h_bad, d_bad, sizeof(unsigned int), cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
    if (*h_bad) {
      release();
      throw Error{FPIE_ERR_ARG, "A holds " + std::to_string(*h_bad) +
                                    " neighbour indices outside [0, N)"};
    }
    ready = true;
  }

  void reset_host(int N, const int32_t* hA, const float* hX, const float* hB) {
    FPIE_REQUIRE(hA && hX && hB, FPIE_ERR_ARG, "null input array");
    allocate(N);
    AsyncScratch scratch((size_t)N * 24, stream);
    float* stage = reinterpret_cast<float*>(scratch.bytes());
    FPIE_CUDA(cudaMemcpyAsync(A, hA, (size_t)N * 16, cudaMemcpyHostToDevice, stream));
    FPIE_CUDA(cudaMemcpyAsync(stage, hX, (size_t)N * 12, cudaMemcpyHostToDevice, stream));
    FPIE_CUDA(cudaMemcpyAsync(stage + (size_t)N * 3, hB, (size_t)N * 12, cudaMemcpyHostToDevice, stream));
    pack_and_check(stage, stage + (size_t)N * 3);
    FPIE_CUDA(cudaStreamSynchronize(stream));
  }

  void reset_device(int N, const int32_t* dA, const float* dX, const float* dB) {
    FPIE_REQUIRE(dA && dX && dB, FPIE_ERR_ARG, "null input array");
    allocate(N);
    FPIE_CUDA(cudaMemcpyAsync(A, dA, (size_t)N * 16, cudaMemcpyDeviceToDevice, stream));
    pack_and_check(dX, dB);
  }

  int* d_rows = nullptr;  // target coordinates of unknowns 1..N-1 (GPU reset)
  int* d_cols = nullptr;

  // GPU-side counterpart of EquProcessor.reset (fpie/process.py:293-372):
  // ids, A, X, B and the unknowns' target coordinates from the uint8 images.
  // box_out: crop on the target (row0, row1, col0, col1); returns N.
  int reset_images(const uint8_t* src, int sh, int sw, const uint8_t* msk, int mh, int mw, int mch,
                   const uint8_t* tgt, int th, int tw, int s_row, int s_col, int t_row, int t_col,
                   int mode, bool on_device, int* box_out) {
    FPIE_REQUIRE(src && msk && tgt && box_out, FPIE_ERR_ARG, "null input array");
    FPIE_REQUIRE(sh > 0 && sw > 0 && mh > 0 && mw > 0 && th > 0 && tw > 0, FPIE_ERR_ARG, "empty image");
    FPIE_REQUIRE(mch == 1 || mch == 3, FPIE_ERR_ARG, "mask must have 1 or 3 channels");
    FPIE_REQUIRE(mode >= 0 && mode <= 2, FPIE_ERR_ARG, "gradient mode must be 0 (src), 1 (avg), 2 (max)");
    const size_t sb = (size_t)sh * sw * 3, mb = (size_t)mh * mw * mch, tb = (size_t)th * tw * 3;
    const size_t mpx = (size_t)mh * mw;
    const size_t head = on_device ? 0 : (sb + mb + tb + 15) / 16 * 16;
    // staging: images (host path) | box (16 B) | m01 | crop ids (<= mpx ints) | block counts
    const size_t nb_max = (mpx + 1023) / 1024 + 2;
    const size_t bytes = head + 16 + (mpx + 15) / 16 * 16 + mpx * 4 + nb_max * 4;
    AsyncScratch scratch(bytes, stream);
    char* stage = scratch.bytes();
    const uint8_t *dsrc = src, *dmsk = msk, *dtgt = tgt;
    if (!on_device) {
      FPIE_CUDA(cudaMemcpyAsync(stage, src, sb, cudaMemcpyHostToDevice, stream));
      FPIE_CUDA(cudaMemcpyAsync(stage + sb, msk, mb, cudaMemcpyHostToDevice, stream));
      FPIE_CUDA(cudaMemcpyAsync(stage + sb + mb, tgt, tb, cudaMemcpyHostToDevice, stream));
      dsrc = reinterpret_cast<uint8_t*>(stage);
      dmsk = reinterpret_cast<uint8_t*>(stage + sb);
      dtgt = reinterpret_cast<uint8_t*>(stage + sb + mb);
    }
    int* dbox = reinterpret_cast<int*>(stage + head);
    uint8_t* m01 = reinterpret_cast<uint8_t*>(stage + head + 16);
    int* ids = reinterpret_cast<int*>(stage + head + 16 + (mpx + 15) / 16 * 16);
    int* counts = ids + mpx;
    int hbox[4] = {INT32_MAX, -1, INT32_MAX, -1};
    FPIE_CUDA(cudaMemcpyAsync(dbox, hbox, sizeof(hbox), cudaMemcpyHostToDevice, stream));
    launch_prep_mask(dmsk, mh, mw, mch, m01, dbox, stream);
    post_launch(this);
    FPIE_CUDA(cudaMemcpyAsync(hbox, dbox, sizeof(hbox), cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
    if (hbox[1] < 0)
      throw Error{FPIE_ERR_ARG, "the mask selects no pixel (after clearing its 1-pixel frame)"};
    const int x0 = hbox[0] - 1, x1 = hbox[1] + 2, y0 = hbox[2] - 1, y1 = hbox[3] + 2;
    const bool fits = s_row + x0 >= 0 && s_col + y0 >= 0 && s_row + x1 <= sh && s_col + y1 <= sw &&
                      t_row + x0 >= 0 && t_col + y0 >= 0 && t_row + x1 <= th && t_col + y1 <= tw;
    if (!fits)
      throw Error{FPIE_ERR_ARG, "the mask's crop at the given offsets leaves the source or target image"};
    const int n = x1 - x0, m = y1 - y0;
    const int nb = launch_equ_ids(m01, mw, x0, y0, n, m, counts, ids, stream);
    post_launch(this, 3);
    int unknowns = 0;
    FPIE_CUDA(cudaMemcpyAsync(&unknowns, counts + nb, sizeof(int), cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
    const int N = unknowns + 1;
    allocate(N);
    cudaFree(d_rows);
    cudaFree(d_cols);
    d_rows = d_cols = nullptr;
    FPIE_CUDA(cudaMalloc(&d_rows, sizeof(int) * std::max(unknowns, 1)));
    FPIE_CUDA(cudaMalloc(&d_cols, sizeof(int) * std::max(unknowns, 1)));
    FPIE_CUDA(cudaMemsetAsync(A, 0, sizeof(int4) * N, stream));
    FPIE_CUDA(cudaMemsetAsync(x[0], 0, (size_t)E.np * 3 * sizeof(float), stream));
    FPIE_CUDA(cudaMemsetAsync(x[1], 0, (size_t)E.np * 3 * sizeof(float), stream));
    FPIE_CUDA(cudaMemsetAsync(b, 0, (size_t)E.np * 3 * sizeof(float), stream));
    launch_equ_build(m01, mw, x0, y0, n, m, ids, dsrc, sw, s_row + x0, s_col + y0, dtgt, tw,
                     t_row + x0, t_col + y0, mode, E.np, A, x[0], x[1], b, d_rows, d_cols, stream);
    post_launch(this);
    ready = true;
    box_out[0] = t_row + x0;
    box_out[1] = t_row + x1;
    box_out[2] = t_col + y0;
    box_out[3] = t_col + y1;
    if (!on_device) FPIE_CUDA(cudaStreamSynchronize(stream));
    return N;
  }

  void get_index(int32_t* rows, int32_t* cols) {
    FPIE_REQUIRE(rows && cols, FPIE_ERR_ARG, "null output array");
    FPIE_REQUIRE(ready && d_rows, FPIE_ERR_STATE, "no index: the solver was not reset from images");
    FPIE_CUDA(cudaMemcpyAsync(rows, d_rows, sizeof(int) * (E.N - 1), cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaMemcpyAsync(cols, d_cols, sizeof(int) * (E.N - 1), cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
  }

  void get_inputs(int32_t* Aout, float* Bout) {
    FPIE_REQUIRE(Aout && Bout, FPIE_ERR_ARG, "null output array");
    FPIE_REQUIRE(ready, FPIE_ERR_STATE, "no state before reset");
    std::vector<float> hb((size_t)E.np * 3);
    FPIE_CUDA(cudaMemcpyAsync(Aout, A, sizeof(int4) * E.N, cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaMemcpyAsync(hb.data(), b, sizeof(float) * hb.size(), cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
    for (int i = 0; i < E.N; ++i)
      for (int c = 0; c < 3; ++c) Bout[(size_t)i * 3 + c] = hb[(size_t)c * E.np + i];
  }

  void sweep_once(cudaStream_t st, int from) {
    equ_sweep_kernel<<<(E.N + block - 1) / block, block, 0, st>>>(E, A, b, x[from], x[from ^ 1]);
  }

  void capture_chunk(int start) {
    cudaStream_t cs = nullptr;
    cudaGraph_t graph = nullptr;
    FPIE_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      int c = start;
      for (int k = 0; k < kChunk; ++k, c ^= 1) sweep_once(cs, c);
      e = cudaStreamEndCapture(cs, &graph);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&chunk[start], graph, 0);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    FPIE_CUDA(e);
  }

  void run_sweeps(int iters) {
    FPIE_REQUIRE(ready, FPIE_ERR_STATE, "step called before reset");
    while (iters >= kChunk) {
      if (!chunk[cur]) capture_chunk(cur);
      FPIE_CUDA(cudaGraphLaunch(chunk[cur], stream));
      post_launch(this, kChunk);
      iters -= kChunk;
    }
    for (; iters > 0; --iters) {
      sweep_once(stream, cur);
      post_launch(this);
      cur ^= 1;
    }
  }

  void finish(uint8_t* img, float* err) {
    equ_finish_kernel<<<nparts, 256, 0, stream>>>(E, A, b, x[cur], img ? img : d_img, d_part);
    post_launch(this);
    launch_finalize(d_part, nparts, err ? err : d_err, stream);
    post_launch(this);
  }

  void step_host(int iteration, uint8_t* img_out, float* err_out) {
    FPIE_REQUIRE(img_out && err_out, FPIE_ERR_ARG, "null output array");
    if (!ready) {
      err_out[0] = err_out[1] = err_out[2] = 0.0f;
      return;
    }
    run_sweeps(iteration);
    finish(d_img, d_err);
    const size_t bytes = (size_t)E.N * 3;
    FPIE_CUDA(cudaMemcpyAsync(h_img, d_img, bytes, cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaMemcpyAsync(h_err, d_err, 3 * sizeof(float), cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
    std::memcpy(img_out, h_img, bytes);
    std::memcpy(err_out, h_err, 3 * sizeof(float));
  }

  void get_state(float* out) {
    FPIE_REQUIRE(out, FPIE_ERR_ARG, "null output array");
    FPIE_REQUIRE(ready, FPIE_ERR_STATE, "no state before reset");
    AsyncScratch scratch((size_t)E.N * 12, stream);
    float* tmp = reinterpret_cast<float*>(scratch.bytes());
    equ_unpack_kernel<<<conv_blocks(E.N), 256, 0, stream>>>(E, x[cur], tmp);
    post_launch(this);
    FPIE_CUDA(cudaMemcpyAsync(out, tmp, (size_t)E.N * 12, cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
  }
};

Solver* new_equ_solver(int block_size) { return new EquSolverImpl(block_size); }

static EquSolverImpl* equ_of(fpie_solver* s) {
  return static_cast<EquSolverImpl*>(check_handle(s, 1));
}

void grid_sweeps(Solver* s, int iters);
void grid_get_state(Solver* s, float* out);
void grid_set_precision(Solver* s, int p);

}  // namespace fpie

using namespace fpie;

extern "C" {

int fpie_equ_partition(fpie_solver* s, const int32_t* mask, int n, int m,
                       int32_t* ids_out) {
  return guarded([&] {
    equ_of(s);
    FPIE_REQUIRE(mask && ids_out, FPIE_ERR_ARG, "null array");
    FPIE_REQUIRE(n >= 0 && m >= 0, FPIE_ERR_ARG, "negative mask shape");
    int32_t cnt = 0;
    const long long total = (long long)n * m;
    for (long long k = 0; k < total; ++k) ids_out[k] = mask[k] > 0 ? ++cnt : 0;
  });
}

int fpie_equ_reset(fpie_solver* s, int N, const int32_t* A, const float* X,
                   const float* B) {
  return guarded([&] { equ_of(s)->reset_host(N, A, X, B); });
}

int fpie_equ_step(fpie_solver* s, int iteration, uint8_t* x_out, float* err_out) {
  return guarded([&] { equ_of(s)->step_host(iteration, x_out, err_out); });
}

int fpie_equ_reset_device(fpie_solver* s, int N, const int32_t* A,
                          const float* X, const float* B) {
  return guarded([&] { equ_of(s)->reset_device(N, A, X, B); });
}

int fpie_equ_reset_images(fpie_solver* s, const uint8_t* src, int src_h, int src_w,
                          const uint8_t* mask, int mask_h, int mask_w, int mask_channels,
                          const uint8_t* tgt, int tgt_h, int tgt_w, int src_row, int src_col,
                          int tgt_row, int tgt_col, int gradient, int on_device, int* box,
                          int* N_out) {
  return guarded([&] {
    const int N = equ_of(s)->reset_images(src, src_h, src_w, mask, mask_h, mask_w, mask_channels,
                                          tgt, tgt_h, tgt_w, src_row, src_col, tgt_row, tgt_col,
                                          gradient, on_device != 0, box);
    if (N_out) *N_out = N;
  });
}

int fpie_equ_get_index(fpie_solver* s, int32_t* rows, int32_t* cols) {
  return guarded([&] { equ_of(s)->get_index(rows, cols); });
}

int fpie_equ_get_inputs(fpie_solver* s, int32_t* A, float* B) {
  return guarded([&] { equ_of(s)->get_inputs(A, B); });
}

int fpie_equ_step_device(fpie_solver* s, int iteration, uint8_t* x, float* err) {
  return guarded([&] {
    EquSolverImpl* h = equ_of(s);
    h->run_sweeps(iteration);
    if (x || err) h->finish(x, err);
  });
}

int fpie_sweeps(fpie_solver* s, int iteration) {
  return guarded([&] {
    Solver* h = check_handle(s, 0);
    if (h->kind == 1)
      static_cast<EquSolverImpl*>(h)->run_sweeps(iteration);
    else
      grid_sweeps(h, iteration);
  });
}

int fpie_get_state(fpie_solver* s, float* out) {
  return guarded([&] {
    Solver* h = check_handle(s, 0);
    if (h->kind == 1)
      static_cast<EquSolverImpl*>(h)->get_state(out);
    else
      grid_get_state(h, out);
  });
}

int fpie_set_precision(fpie_solver* s, int precision) {
  return guarded([&] {
    Solver* h = check_handle(s, 0);
    if (h->kind == 2) {
      grid_set_precision(h, precision);
      return;
    }
    FPIE_REQUIRE(precision == FPIE_FP32, FPIE_ERR_ARG,
                 "EquSolver supports FPIE_FP32 only; the mixed forms are grid solvers");
    h->precision = precision;
  });
}

}  // extern "C"
