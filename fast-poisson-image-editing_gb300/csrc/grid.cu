// GridSolver backend: masked 4-neighbour Jacobi on the cropped image.
//
// Replaces fpie/core/cuda/grid.cu (CudaGridSolver) behind the same plugin
// surface (fpie/core/base_solver.h:77-152).  Differences by design:
//  * strict Jacobi with two state buffers (the numpy backend's semantics,
//    fpie/np_solver.py:79-101), not an in-place chaotic sweep;
//  * planar, padded channel planes in HBM (see GridGeom) instead of
//    interleaved float3, so every access is an aligned, coalesced vector;
//  * the sweep loop is replayed from captured CUDA graphs in chunks;
//  * a deterministic two-level residual reduction (no cross-block race);
//  * every CUDA call is checked.
#include <algorithm>
#include <cstring>
#include <map>
#include <tuple>
#include <mutex>
#include <utility>

#include "common.cuh"
#include "grid_kernels.cuh"
#include "grid_mixed.cuh"
#include "grid_flow.cuh"
#include "grid_tma.cuh"
#include "grid_tb.cuh"
#include "prep.cuh"

namespace fpie {

__global__ void grid_inputs_unpack_kernel(GridGeom G, const uint8_t* __restrict__ mask,
                                          const float* __restrict__ g,
                                          int32_t* __restrict__ mask_out,
                                          float* __restrict__ grad_out) {
  const long long total = (long long)G.n * G.m;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(idx / G.m), j = (int)(idx % G.m);
    const long long p = G.at(i, j);
    mask_out[idx] = mask[p];
#pragma unroll
    for (int c = 0; c < 3; ++c) grad_out[idx * 3 + c] = g[c * G.plane + p];
  }
}

// ---- layout conversion kernels ------------------------------------------------

// An equation system that is a 4-neighbour raster stencil, on the grid:
// unknown i (1..N-1) at crop pixel pos[i] (row-major, G.m per row) gets its
// X as state and its B as "grad"; every other pixel stays 0 and unmasked,
// which is what the system's constant row 0 contributes to a gather.
// X and B are planar (channel c at c * np).
__global__ void grid_from_equ_kernel(GridGeom G, int N, const int* __restrict__ pos,
                                     const float* __restrict__ xe, const float* __restrict__ be,
                                     long long np, uint8_t* __restrict__ mask,
                                     float* __restrict__ x0, float* __restrict__ x1,
                                     float* __restrict__ g) {
  for (long long i = 1 + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    const int p = pos[i];
    const long long q = G.at(p / G.m, p % G.m);
    mask[q] = 1;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float v = xe[c * np + i];
      x0[c * G.plane + q] = v;
      x1[c * G.plane + q] = v;
      g[c * G.plane + q] = be[c * np + i];
    }
  }
}

// The unknowns' state back into planar X (row 0 untouched).
__global__ void grid_to_equ_kernel(GridGeom G, int N, const int* __restrict__ pos,
                                   const float* __restrict__ x, float* __restrict__ xe,
                                   long long np) {
  for (long long i = 1 + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    const int p = pos[i];
    const long long q = G.at(p / G.m, p % G.m);
#pragma unroll
    for (int c = 0; c < 3; ++c) xe[c * np + i] = x[c * G.plane + q];
  }
}

__global__ void grid_pack_kernel(GridGeom G, const int32_t* __restrict__ mk,
                                 const float* __restrict__ t,
                                 const float* __restrict__ gr,
                                 uint8_t* __restrict__ mask,
                                 float* __restrict__ x0, float* __restrict__ x1,
                                 float* __restrict__ g) {
  const long long total = (long long)G.n * G.m;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       idx < total; idx += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(idx / G.m), j = (int)(idx % G.m);
    const long long p = G.at(i, j);
    mask[p] = mk[idx] != 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float v = t[idx * 3 + c];
      x0[c * G.plane + p] = v;
      x1[c * G.plane + p] = v;
      g[c * G.plane + p] = gr[idx * 3 + c];
    }
  }
}

__global__ void grid_unpack_kernel(GridGeom G, const float* __restrict__ x,
                                   float* __restrict__ out) {
  const long long total = (long long)G.n * G.m;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       idx < total; idx += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(idx / G.m), j = (int)(idx % G.m);
    const long long p = G.at(i, j);
#pragma unroll
    for (int c = 0; c < 3; ++c) out[idx * 3 + c] = x[c * G.plane + p];
  }
}

static int conv_blocks(long long total) { return stride_blocks(total, 256, 32); }

// ---- the solver object ----------------------------------------------------------

struct GridSolverImpl : Solver {
  int grid_x, grid_y;
  int N_user = 0;
  bool ready = false;
  GridGeom G{};
  float* x[2] = {nullptr, nullptr};
  float* g = nullptr;
  uint8_t* mask = nullptr;
  int cur = 0;
  uint8_t* d_img = nullptr;
  double* d_part = nullptr;
  float* d_err = nullptr;
  float* h_err = nullptr;
  int* h_box = nullptr;  // pinned, for the GPU-side reset's bounding box
  GridLaunch L{};
  static constexpr int kChunk = 64;  // sweeps per captured graph (even)
  cudaGraphExec_t chunk[2] = {nullptr, nullptr};

  // Bounded device waits (the flow kernel's neighbourhood waits, the TMA
  // kernel's copy waits) give up after spin_limit rounds and set d_wait_err.
  long long spin_limit = 1LL << 26;  // x ~64 ns sleeps: a few seconds at most
  int* d_wait_err = nullptr;
  int* h_wait_err = nullptr;  // pinned

  // ---- persistent TMA-prefetch kernel (variant index kTma; by name only) -----
  static constexpr int kTma = -3;
  int* tma_list = nullptr;   // active-tile list (count + indices)
  int tma_list_cap = 0;
  int tma_grid = 0;          // persistent CTAs for the current tiling

  // ---- dependency-flow kernel (FP32: variants kFlow, kFlow12, kFlowP,
  // kFlow12P; mixed: mvariant kFlow) ----------------------------------------------
  // Its tables depend only on the geometry, the mask and the depth.
  static constexpr int kFlow = -4;     // depth 16 ("p16w8k16d")
  static constexpr int kFlow12 = -5;   // depth 12 ("p16w8k12d"), FP32 Jacobi only
  static constexpr int kFlowP = -6;    // depth 16 with pinned-boundary bodies ("p16w8k16dp")
  static constexpr int kFlow12P = -7;  // depth 12 with them ("p16w8k12dp")
  static bool is_flow(int v) { return v == kFlow || v == kFlow12 || v == kFlowP || v == kFlow12P; }
  // Depth of the flow launches the current settings make, and whether they
  // use the pinned-boundary bodies (FP32 Jacobi only).
  int flow_k() const {
    return precision == FPIE_FP32 && (variant == kFlow12 || variant == kFlow12P) ? 12
                                                                                : flow_depth();
  }
  bool flow_pin() const {
    return precision == FPIE_FP32 && !red_black && (variant == kFlowP || variant == kFlow12P);
  }
  uint8_t* ft_flags = nullptr;  // tile flags for the flow tiling
  uint8_t* code = nullptr;      // masked / pinned bits per pixel (launch_grid_code)
  int* ft_list = nullptr;       // active-tile list (count + indices)
  int* flow_inv = nullptr;      // tile -> active-list index
  void* flow_rec = nullptr;     // per active tile: index, flag, neighbourhood
  int* flow_done = nullptr;     // levels finished per (active tile, channel)
  int flow_cap = 0;             // tiles the arrays hold
  int ft_tiles_x = 0, ft_tiles = 0;
  int ft_k = 0;  // depth the tables were built for
  bool ft_ok = false;
  int flow_grid = 0;

  // Reads and clears the wait-error flag (a flow-kernel neighbourhood wait
  // or a TMA copy wait that gave up); call after the stream has been
  // synchronised.
  void check_waits() {
    if (!d_wait_err) return;
    FPIE_CUDA(cudaMemcpyAsync(h_wait_err, d_wait_err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
    if (*h_wait_err) {
      *h_wait_err = 0;
      FPIE_CUDA(cudaMemsetAsync(d_wait_err, 0, sizeof(int), stream));
      FPIE_CUDA(cudaStreamSynchronize(stream));
      throw Error{FPIE_ERR_TIMEOUT, "sweep kernel: a bounded device wait gave up"};
    }
  }
  void check_async() override { check_waits(); }

  // All `iters` sweeps in one launch of the dependency-flow kernel.  A wait
  // that timed out is reported at the next host synchronisation.
  void run_flow(int iters) {
    ensure_flow_tables();
    FPIE_CUDA(cudaMemsetAsync(flow_done, 0, (size_t)ft_tiles * 3 * sizeof(int), stream));
    launch_flow(G, mask, code, g, x[0], x[1], cur, ft_list, flow_rec, flow_done, ft_tiles_x,
                ft_tiles, iters, d_wait_err, spin_limit, flow_grid, stream, red_black, ft_k,
                flow_pin());
    post_launch(this);
    const int per_level = red_black ? flow_rb_depth() : ft_k;
    const int levels = (iters + per_level - 1) / per_level;
    if (levels & 1) cur ^= 1;
  }

  // The mixed forms as one flow launch (cycles of 64 sweeps and the final
  // fold, like run_mixed's launch sequence with a 16-sweep kernel).
  void run_flow_mixed(int iters) {
    ensure_mixed();
    ensure_flow_tables();
    FPIE_CUDA(cudaMemsetAsync(flow_done, 0, (size_t)ft_tiles * 3 * sizeof(int), stream));
    launch_flow_mixed(G, mask, g, x[0], x[1], cur, precision == FPIE_MIXED_BF16, e[0], e[1], r,
                      ft_list, flow_rec, flow_done, ft_tiles_x, ft_tiles, iters, d_wait_err,
                      spin_limit, flow_grid, stream);
    post_launch(this);
    if (flow_mixed_flips(iters) & 1) cur ^= 1;
    e_pending = false;
  }

  // ---- mixed-precision refinement state (allocated on first use) -----------
  static constexpr int kRefine = 64;  // inner sweeps per refinement cycle
  void* e[2] = {nullptr, nullptr};    // correction, FP16 or BF16 planes
  float* r = nullptr;                 // FP32 residual planes
  double* d_part6 = nullptr;          // per-block max|r|, sum|r| (double)
  double* d_norm = nullptr;           // [max x3, sum x3]
  double* h_norm = nullptr;           // pinned copy
  uint8_t* mflags = nullptr;
  int mflags_cap = 0, mtiles_x = 0, mtiles = 0;
  bool mflags_ok = false;
  int mvariant = 0;
  bool mtuned = false;
  int e_prec = -1;                    // precision the e buffers were sized for
  cudaGraphExec_t cycle[2] = {nullptr, nullptr};

  GridSolverImpl(int gx, int gy) : grid_x(gx), grid_y(gy) {
    kind = 2;
    FPIE_CUDA(cudaGetDevice(&device));
    FPIE_CUDA(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking));
    stream = own_stream;
    FPIE_CUDA(cudaMallocHost(&h_err, 3 * sizeof(float)));
  }

  ~GridSolverImpl() override {
    release();
    if (h_err) cudaFreeHost(h_err);
    if (h_norm) cudaFreeHost(h_norm);
    if (h_box) cudaFreeHost(h_box);
    if (own_stream) cudaStreamDestroy(own_stream);
  }

  void drop_graphs() {
    for (auto& gx : chunk) {
      if (gx) cudaGraphExecDestroy(gx);
      gx = nullptr;
    }
    for (auto& gx : cycle) {
      if (gx) cudaGraphExecDestroy(gx);
      gx = nullptr;
    }
  }

  void release_mixed() {
    cudaFree(e[0]);
    cudaFree(e[1]);
    cudaFree(r);
    cudaFree(d_part6);
    cudaFree(d_norm);
    cudaFree(mflags);
    e[0] = e[1] = nullptr;
    r = nullptr;
    d_part6 = d_norm = nullptr;
    mflags = nullptr;
    mflags_cap = 0;
    mflags_ok = false;
    e_prec = -1;
  }

  void release() {
    cudaStreamSynchronize(stream);  // NULL (legacy default stream) included
    drop_graphs();
    cudaFree(x[0]);
    cudaFree(x[1]);
    cudaFree(g);
    cudaFree(mask);
    cudaFree(code);
    cudaFree(d_img);
    cudaFree(d_part);
    cudaFree(d_err);
    cudaFree(flags);
    flags = nullptr;
    flags_cap = 0;
    flags_ok = false;
    release_mixed();
    cudaFree(d_wait_err);
    cudaFree(tma_list);
    cudaFree(flow_inv);
    cudaFree(flow_done);
    cudaFree(flow_rec);
    cudaFree(ft_flags);
    cudaFree(ft_list);
    flow_inv = nullptr;
    flow_done = nullptr;
    flow_rec = nullptr;
    ft_flags = nullptr;
    ft_list = nullptr;
    flow_cap = 0;
    ft_ok = false;
    if (h_wait_err) cudaFreeHost(h_wait_err);
    d_wait_err = nullptr;
    h_wait_err = nullptr;
    tma_list = nullptr;
    tma_list_cap = 0;
    x[0] = x[1] = g = nullptr;
    mask = nullptr;
    code = nullptr;
    d_img = nullptr;
    d_part = nullptr;
    d_err = nullptr;
    ready = false;
  }

  void allocate(int n, int m) {
    FPIE_REQUIRE(n >= 1 && m >= 1, FPIE_ERR_ARG, "grid must be at least 1x1");
    FPIE_REQUIRE((long long)n * m <= (1LL << 31) / 4, FPIE_ERR_ARG,
                 "grid too large (n*m*3 must fit in int32 indexing of the image)");
    if (x[0] && G.n == n && G.m == m) {
      // Same geometry: keep the buffers (and the captured sweep graphs, whose
      // pointers stay valid).  The halo is still zero; the interior is
      // rewritten by the pack kernel.
      cur = 0;
      ready = false;
      flags_ok = false;  // the new mask may activate other tiles
      mflags_ok = false;
      ft_ok = false;
      return;
    }
    release();
    if (!pinned) tuned = false;
    G = make_geom(n, m);
    L = grid_launch(G);
    FPIE_REQUIRE(L.sweep_grid.y <= 65535, FPIE_ERR_ARG, "grid has too many rows");
    const size_t pb = (size_t)G.plane * sizeof(float);
    FPIE_CUDA(cudaMalloc(&x[0], 3 * pb));
    FPIE_CUDA(cudaMalloc(&x[1], 3 * pb));
    FPIE_CUDA(cudaMalloc(&g, 3 * pb));
    FPIE_CUDA(cudaMalloc(&mask, (size_t)G.plane));
    FPIE_CUDA(cudaMalloc(&code, (size_t)G.plane));
    FPIE_CUDA(cudaMalloc(&d_img, (size_t)n * m * 3));
    FPIE_CUDA(cudaMalloc(&d_part, (size_t)L.nparts * 3 * sizeof(double)));
    FPIE_CUDA(cudaMalloc(&d_err, 3 * sizeof(float)));
    FPIE_CUDA(cudaMemsetAsync(x[0], 0, 3 * pb, stream));
    FPIE_CUDA(cudaMemsetAsync(x[1], 0, 3 * pb, stream));
    FPIE_CUDA(cudaMemsetAsync(g, 0, 3 * pb, stream));
    FPIE_CUDA(cudaMemsetAsync(mask, 0, (size_t)G.plane, stream));
    cur = 0;
  }

  void pack(const int32_t* dmask, const float* dtgt, const float* dgrad) {
    const long long total = (long long)G.n * G.m;
    grid_pack_kernel<<<conv_blocks(total), 256, 0, stream>>>(
        G, dmask, dtgt, dgrad, mask, x[0], x[1], g);
    post_launch(this);
    ready = true;
  }

  void reset_host(int N, int n, int m, const int32_t* hm, const float* ht,
                  const float* hg) {
    FPIE_REQUIRE(hm && ht && hg, FPIE_ERR_ARG, "null input array");
    allocate(n, m);
    N_user = N;
    const size_t px = (size_t)n * m;
    const size_t bytes = px * 4 + 2 * px * 12;
    AsyncScratch scratch(bytes, stream);
    char* stage = scratch.bytes();
    int32_t* sm = reinterpret_cast<int32_t*>(stage);
    float* st = reinterpret_cast<float*>(stage + px * 4);
    float* sg = reinterpret_cast<float*>(stage + px * 16);
    FPIE_CUDA(cudaMemcpyAsync(sm, hm, px * 4, cudaMemcpyHostToDevice, stream));
    FPIE_CUDA(cudaMemcpyAsync(st, ht, px * 12, cudaMemcpyHostToDevice, stream));
    FPIE_CUDA(cudaMemcpyAsync(sg, hg, px * 12, cudaMemcpyHostToDevice, stream));
    pack(sm, st, sg);
    // The caller may reuse its arrays as soon as reset returns.
    FPIE_CUDA(cudaStreamSynchronize(stream));
  }

  // Loads an equation system that is a 4-neighbour raster stencil (see
  // grid_from_equ_kernel); the sweeps are then bit-identical to the
  // system's gather sweeps.
  void reset_from_equ(int n, int m, int N, const int* pos, const float* xe, const float* be,
                      long long np) {
    allocate(n, m);
    N_user = n * m;
    const size_t pb = (size_t)G.plane * 3 * sizeof(float);
    FPIE_CUDA(cudaMemsetAsync(x[0], 0, pb, stream));
    FPIE_CUDA(cudaMemsetAsync(x[1], 0, pb, stream));
    FPIE_CUDA(cudaMemsetAsync(g, 0, pb, stream));
    FPIE_CUDA(cudaMemsetAsync(mask, 0, (size_t)G.plane, stream));
    if (N > 1) {
      grid_from_equ_kernel<<<conv_blocks(N), 256, 0, stream>>>(G, N, pos, xe, be, np, mask, x[0],
                                                               x[1], g);
      post_launch(this);
    }
    ready = true;
  }

  void to_equ(int N, const int* pos, float* xe, long long np) {
    FPIE_REQUIRE(ready, FPIE_ERR_STATE, "no state before reset");
    if (N <= 1) return;
    grid_to_equ_kernel<<<conv_blocks(N), 256, 0, stream>>>(G, N, pos, x[cur], xe, np);
    post_launch(this);
  }

  void reset_device(int n, int m, const int32_t* dm, const float* dt,
                    const float* dg) {
    FPIE_REQUIRE(dm && dt && dg, FPIE_ERR_ARG, "null input array");
    allocate(n, m);
    N_user = n * m;
    pack(dm, dt, dg);
  }

  // Builds the solver inputs on the GPU from the three uint8 images
  // (prep.cu), the device counterpart of GridProcessor.reset.  box_out
  // receives the crop on the target (row0, row1, col0, col1).
  void reset_images(const uint8_t* src, int sh, int sw, const uint8_t* msk, int mh, int mw,
                    int mch, const uint8_t* tgt, int th, int tw, int s_row, int s_col,
                    int t_row, int t_col, int mode, bool on_device, int* box_out) {
    FPIE_REQUIRE(src && msk && tgt && box_out, FPIE_ERR_ARG, "null input array");
    FPIE_REQUIRE(sh > 0 && sw > 0 && mh > 0 && mw > 0 && th > 0 && tw > 0, FPIE_ERR_ARG,
                 "empty image");
    FPIE_REQUIRE(mch == 1 || mch == 3, FPIE_ERR_ARG, "mask must have 1 or 3 channels");
    FPIE_REQUIRE(mode >= 0 && mode <= 2, FPIE_ERR_ARG,
                 "gradient mode must be 0 (src), 1 (avg), 2 (max)");
    const size_t sb = (size_t)sh * sw * 3, mb = (size_t)mh * mw * mch, tb = (size_t)th * tw * 3;
    const size_t mpx = (size_t)mh * mw;
    const size_t head = on_device ? 0 : (sb + mb + tb + 15) / 16 * 16;
    AsyncScratch scratch(head + 16 + mpx, stream);
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
    if (!h_box) FPIE_CUDA(cudaMallocHost(&h_box, 4 * sizeof(int)));
    h_box[0] = INT32_MAX;
    h_box[1] = -1;
    h_box[2] = INT32_MAX;
    h_box[3] = -1;
    FPIE_CUDA(cudaMemcpyAsync(dbox, h_box, 4 * sizeof(int), cudaMemcpyHostToDevice, stream));
    launch_prep_mask(dmsk, mh, mw, mch, m01, dbox, stream);
    post_launch(this);
    FPIE_CUDA(cudaMemcpyAsync(h_box, dbox, 4 * sizeof(int), cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
    const int b0 = h_box[0], b1 = h_box[1], b2 = h_box[2], b3 = h_box[3];
    if (b1 < 0)
      throw Error{FPIE_ERR_ARG, "the mask selects no pixel (after clearing its 1-pixel frame)"};
    const int x0 = b0 - 1, x1 = b1 + 2, y0 = b2 - 1, y1 = b3 + 2;
    const bool fits = s_row + x0 >= 0 && s_col + y0 >= 0 && s_row + x1 <= sh && s_col + y1 <= sw &&
                      t_row + x0 >= 0 && t_col + y0 >= 0 && t_row + x1 <= th && t_col + y1 <= tw;
    if (!fits)
      throw Error{FPIE_ERR_ARG,
                  "the mask's crop at the given offsets leaves the source or target image"};
    allocate(x1 - x0, y1 - y0);
    N_user = G.n * G.m;
    PrepArgs a{G, m01, mw, x0, y0, dsrc, sw, s_row + x0, s_col + y0, dtgt, tw, t_row + x0,
               t_col + y0, mode};
    launch_prep_grid(a, mask, x[0], x[1], g, stream);
    post_launch(this);
    ready = true;
    flags_ok = false;
    mflags_ok = false;
    ft_ok = false;
    box_out[0] = t_row + x0;
    box_out[1] = t_row + x1;
    box_out[2] = t_col + y0;
    box_out[3] = t_col + y1;
    if (!on_device) FPIE_CUDA(cudaStreamSynchronize(stream));
  }

  void get_inputs(int32_t* mask_out, float* grad_out) {
    FPIE_REQUIRE(mask_out && grad_out, FPIE_ERR_ARG, "null output array");
    FPIE_REQUIRE(ready, FPIE_ERR_STATE, "no state before reset");
    const long long total = (long long)G.n * G.m;
    AsyncScratch scratch(total * 16, stream);
    char* tmp = scratch.bytes();
    grid_inputs_unpack_kernel<<<conv_blocks(total), 256, 0, stream>>>(
        G, mask, g, reinterpret_cast<int32_t*>(tmp), reinterpret_cast<float*>(tmp + total * 4));
    post_launch(this);
    FPIE_CUDA(cudaMemcpyAsync(mask_out, tmp, total * 4, cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaMemcpyAsync(grad_out, tmp + total * 4, total * 12, cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
  }

  // ---- sweep kernels ---------------------------------------------------------
  // variant: -1 = one sweep per launch (grid_sweep_kernel), k >= 0 = the k-th
  // temporally blocked variant.  All give bit-identical states.
  int variant = default_variant();
  bool tuned = false;       // kernel chosen by the autotuner (or pinned)
  bool pinned = false;      // chosen explicitly with fpie_grid_set_kernel
  uint8_t* flags = nullptr;  // active-tile flags of `variant`
  int flags_cap = 0, tiles_x = 0, tiles = 0;
  bool flags_ok = false;

  // The kernel used before (or without) autotuning: the packed 16-row,
  // 8-warp, 16-sweep variant, fastest on both benchmark shapes measured.
  static int default_variant() {
    for (size_t k = 0; k < tb_variants().size(); ++k)
      if (std::string(tb_variants()[k].name) == "p16w8k16") return (int)k;
    return 0;
  }

  int depth() const {
    if (variant == kTma) return tma_depth();
    if (is_flow(variant)) return flow_k();
    return variant < 0 ? 1 : tb_variants()[variant].depth;
  }

  void ensure_flags() {
    if (is_flow(variant)) {
      ensure_flow_tables();
      return;
    }
    // sweep1: no flags
    if (flags_ok || (variant < 0 && variant != kTma)) return;
    const bool tma = variant == kTma;
    const bool listed = tma;  // kernels that take the active-tile list
    const int th = tma ? tma_tile_h() : tb_variants()[variant].tile_h;
    const int tw = tma ? tma_tile_w() : tb_variants()[variant].tile_w;
    const int kd = tma ? tma_depth() : tb_variants()[variant].apron;
    tiles_x = (G.m + tw - 1) / tw;
    tiles = tiles_x * ((G.n + th - 1) / th);
    if (tiles > flags_cap) {
      cudaFree(flags);
      flags = nullptr;
      FPIE_CUDA(cudaMalloc(&flags, tiles));
      flags_cap = tiles;
    }
    if (listed) {
      prepare_tma();
      tma_grid = tma_ctas(tiles * 3);
      ensure_wait_flag();
      if (tiles + 1 > tma_list_cap) {
        cudaFree(tma_list);
        tma_list = nullptr;
        FPIE_CUDA(cudaMalloc(&tma_list, (size_t)(tiles + 1) * sizeof(int)));
        tma_list_cap = tiles + 1;
      }
    } else {
      tb_variants()[variant].prepare();
    }
    launch_tile_flags(G, mask, th, tw, kd, tiles_x, tiles, flags, stream);
    post_launch(this);
    if (listed) {
      launch_tma_list(flags, tiles, tma_list, stream);
      post_launch(this);
    }
    flags_ok = true;
  }

  void ensure_wait_flag() {
    if (d_wait_err) return;
    FPIE_CUDA(cudaMalloc(&d_wait_err, sizeof(int)));
    FPIE_CUDA(cudaMallocHost(&h_wait_err, sizeof(int)));
    *h_wait_err = 0;
    FPIE_CUDA(cudaMemsetAsync(d_wait_err, 0, sizeof(int), stream));
  }

  // Flags, active-tile list, records and counters of the flow tiling.
  void ensure_flow_tables() {
    const int kd = flow_k();
    if (ft_ok && ft_k == kd) return;
    const int th = flow_tile_h(kd), tw = flow_tile_w(kd);
    ft_tiles_x = (G.m + tw - 1) / tw;
    ft_tiles = ft_tiles_x * ((G.n + th - 1) / th);
    if (ft_tiles > flow_cap) {
      cudaFree(flow_inv);
      cudaFree(flow_done);
      cudaFree(flow_rec);
      cudaFree(ft_flags);
      cudaFree(ft_list);
      flow_inv = flow_done = ft_list = nullptr;
      flow_rec = nullptr;
      ft_flags = nullptr;
      FPIE_CUDA(cudaMalloc(&ft_flags, (size_t)ft_tiles));
      FPIE_CUDA(cudaMalloc(&ft_list, (size_t)(ft_tiles + 1) * sizeof(int)));
      FPIE_CUDA(cudaMalloc(&flow_inv, (size_t)ft_tiles * sizeof(int)));
      FPIE_CUDA(cudaMalloc(&flow_done, (size_t)ft_tiles * 3 * sizeof(int)));
      FPIE_CUDA(cudaMalloc(&flow_rec, (size_t)ft_tiles * flow_rec_bytes()));
      flow_cap = ft_tiles;
    }
    flow_grid = flow_ctas();
    ensure_wait_flag();
    launch_tile_flags(G, mask, th, tw, kd, ft_tiles_x, ft_tiles, ft_flags, stream);
    post_launch(this);
    launch_tma_list(ft_flags, ft_tiles, ft_list, stream);
    post_launch(this);
    launch_grid_code(G, mask, code, stream);
    post_launch(this);
    launch_flow_tables(G, code, kd, ft_list, ft_flags, ft_tiles_x, ft_tiles, flow_inv, flow_rec,
                       stream);
    post_launch(this, 3);
    ft_k = kd;
    ft_ok = true;
  }

  void select_variant(int v) {
    if (v != variant) {
      drop_graphs();
      flags_ok = false;
    }
    variant = v;
  }

  // Red-black sweeps instead of Jacobi: only the EquSolver's red-black
  // order sets this, on the grid placement of its system.
  bool red_black = false;

  static int red_black_variant() {
    for (size_t k = 0; k < tb_variants().size(); ++k)
      if (tb_variants()[k].red_black) return (int)k;
    return -100;
  }

  void set_red_black(bool on) {
    if (on == red_black) return;
    FPIE_REQUIRE(!on || precision == FPIE_FP32, FPIE_ERR_STATE, "red-black sweeps are FP32 only");
    red_black = on;
    select_variant(on ? red_black_variant() : default_variant());
    pinned = tuned = false;
  }

  // k sweeps (k <= depth()) from buffer `from`; flips nothing (caller does).
  void launch_block(cudaStream_t st, int from, int k) {
    if (variant == kTma) {
      launch_tma(G, mask, g, x[from], x[from ^ 1], flags, tma_list, tiles_x, tiles, k, d_wait_err,
                 spin_limit, tma_grid, st);
    } else if (variant < 0) {
      launch_grid_sweep(L, G, mask, g, x[from], x[from ^ 1], st);
    } else {
      const TbVariant& v = tb_variants()[variant];
      v.launch(G, mask, g, x[from], x[from ^ 1], flags, tiles_x, tiles, k, st);
    }
  }

  void capture_chunk(int start) {
    cudaStream_t cs = nullptr;
    cudaGraph_t graph = nullptr;
    FPIE_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      int c = start;
      const int d = depth();
      for (int k = 0; k < kChunk; k += d, c ^= 1) launch_block(cs, c, d);
      e = cudaStreamEndCapture(cs, &graph);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&chunk[start], graph, 0);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    FPIE_CUDA(e);
  }

  // One graph replay = kChunk sweeps; the launch count is even, so the
  // current buffer is unchanged afterwards.
  void run_chunk() {
    ensure_flags();
    if (!chunk[cur]) capture_chunk(cur);
    FPIE_CUDA(cudaGraphLaunch(chunk[cur], stream));
    post_launch(this, kChunk / depth());
  }

  // Autotuner: times kChunk sweeps of every candidate (real sweeps, so the
  // state advances exactly as it would with any one kernel) and keeps the
  // fastest.  The choice is remembered per grid shape for this process.
  static std::mutex& tune_mutex() {
    static std::mutex mu;
    return mu;
  }
  static std::map<std::tuple<int, int, bool>, int>& tune_cache() {
    static std::map<std::tuple<int, int, bool>, int> c;
    return c;
  }
  static constexpr int kTuneReps = 2;

  int autotune(int iters) {
    {
      std::lock_guard<std::mutex> lk(tune_mutex());
      auto it = tune_cache().find({G.n, G.m, red_black});
      if (it != tune_cache().end()) {
        select_variant(it->second);
        tuned = true;
        return 0;
      }
    }
    // Candidates: four packed temporally blocked variants, then the flow
    // kernel below (two depths).  sweep1 (one sweep per launch, the baseline) and the TMA
    // kernel stay available by name but were never the fastest on a
    // measured shape; timing them would only lengthen the first step.
    static const char* const kTuned[] = {"p16w8k16", "p8w16k16", "p16w8k8", "p8w8k8"};
    std::vector<int> cands;
    for (int v = 0; v < (int)tb_variants().size(); ++v) {
      const TbVariant& tv = tb_variants()[v];
      bool take = tv.red_black;
      if (!red_black)
        for (const char* n : kTuned) take = take || std::string(tv.name) == n;
      if (take && tv.red_black == red_black) cands.push_back(v);
    }
    const int ncand = (int)cands.size();
    if (iters < (ncand + 1) * (kTuneReps + 1) * kChunk + kChunk) return 0;
    cudaEvent_t e0, e1;
    FPIE_CUDA(cudaEventCreate(&e0));
    FPIE_CUDA(cudaEventCreate(&e1));
    int best = default_variant(), used = 0;
    float best_ms = 1e30f;
    for (int v : cands) {
      select_variant(v);
      run_chunk();  // warm: flags, graph capture, first replay
      used += kChunk;
      for (int r = 0; r < kTuneReps; ++r) {
        FPIE_CUDA(cudaEventRecord(e0, stream));
        run_chunk();
        FPIE_CUDA(cudaEventRecord(e1, stream));
        FPIE_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        FPIE_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        used += kChunk;
        if (ms < best_ms) {
          best_ms = ms;
          best = v;
        }
      }
    }
    // The dependency-flow kernel runs a whole step per launch; timed on 4
    // chunks per launch so that its start and end (one level each) weigh as
    // little as in a real step.  For Jacobi sweeps both depths (which tiling
    // covers the grid with less work depends on its extents), each with and
    // without the pinned-boundary bodies (they pay off on straight mask
    // edges; the larger kernel runs curved ones slower).
    for (int fv : {kFlow, kFlow12, kFlowP, kFlow12P}) {
      if (fv != kFlow && red_black) continue;
      if (iters - used < (kTuneReps + 1) * 4 * kChunk) break;
      select_variant(fv);
      run_flow(4 * kChunk);
      used += 4 * kChunk;
      for (int r = 0; r < kTuneReps; ++r) {
        FPIE_CUDA(cudaEventRecord(e0, stream));
        run_flow(4 * kChunk);
        FPIE_CUDA(cudaEventRecord(e1, stream));
        FPIE_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        FPIE_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        used += 4 * kChunk;
        if (ms / 4 < best_ms) {
          best_ms = ms / 4;
          best = fv;
        }
      }
      check_waits();
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    select_variant(best);
    tuned = true;
    std::lock_guard<std::mutex> lk(tune_mutex());
    tune_cache()[{G.n, G.m, red_black}] = best;
    return used;
  }

  void run_sweeps(int iters) {
    FPIE_REQUIRE(ready, FPIE_ERR_STATE, "step called before reset");
    if (iters <= 0) return;
    if (precision != FPIE_FP32) {
      run_mixed(iters);
      return;
    }
    if (!tuned && !pinned) iters -= autotune(iters);
    if (is_flow(variant)) {
      if (iters > 0) run_flow(iters);
      return;
    }
    while (iters >= kChunk) {
      run_chunk();
      iters -= kChunk;
    }
    ensure_flags();
    while (iters > 0) {
      const int k = std::min(iters, depth());
      launch_block(stream, cur, k);
      post_launch(this);
      cur ^= 1;
      iters -= k;
    }
  }

  // ---- mixed precision ---------------------------------------------------------
  void ensure_mixed() {
    if (e[0] == nullptr || e_prec != precision) {
      release_mixed();
      const size_t eb = (size_t)G.plane * 3 * 2;  // FP16 / BF16
      FPIE_CUDA(cudaMalloc(&e[0], eb));
      FPIE_CUDA(cudaMalloc(&e[1], eb));
      FPIE_CUDA(cudaMalloc(&r, (size_t)G.plane * 3 * sizeof(float)));
      FPIE_CUDA(cudaMalloc(&d_part6, (size_t)L.nparts * 6 * sizeof(double)));
      FPIE_CUDA(cudaMalloc(&d_norm, 6 * sizeof(double)));
      FPIE_CUDA(cudaMemsetAsync(e[0], 0, eb, stream));
      FPIE_CUDA(cudaMemsetAsync(e[1], 0, eb, stream));
      FPIE_CUDA(cudaMemsetAsync(r, 0, (size_t)G.plane * 3 * sizeof(float), stream));
      e_prec = precision;
      drop_graphs();
    }
    if (!mflags_ok && mvariant >= 0) {
      const MixedVariant& v = mixed_variants()[mvariant];
      mtiles_x = (G.m + v.tile_w - 1) / v.tile_w;
      mtiles = mtiles_x * ((G.n + v.tile_h - 1) / v.tile_h);
      if (mtiles > mflags_cap) {
        cudaFree(mflags);
        mflags = nullptr;
        FPIE_CUDA(cudaMalloc(&mflags, mtiles));
        mflags_cap = mtiles;
      }
      launch_tile_flags(G, mask, v.tile_h, v.tile_w, v.depth, mtiles_x, mtiles, mflags, stream);
      post_launch(this);
      mflags_ok = true;
    }
  }

  void select_mixed(int v) {
    if (v != mvariant) {
      drop_graphs();
      mflags_ok = false;
    }
    mvariant = v;
  }

  // FP64 norms of the residual of x[cur] (no fold) into d_norm.
  void refine_norms(cudaStream_t st, float* rout) {
    launch_refine(precision, L.sweep_grid, L.sweep_block, G, mask, g, x[cur], nullptr,
                  nullptr, rout, d_part6, st);
    launch_norms_finalize(d_part6, L.nparts, d_norm, st);
  }

  // Pending correction: the last cycle's e (in e[e_last]) not yet added to x.
  bool e_pending = false;
  int e_last = 0;

  // One refinement cycle of c inner sweeps.  Its first launch folds the
  // pending correction into x (x[cur] + e -> x[cur ^ 1]), recomputes the
  // FP32 residual, and starts the new correction from 0 (tbp_fold_body);
  // the other launches continue the correction.
  void mixed_cycle(cudaStream_t st, int c) {
    const MixedVariant& v = mixed_variants()[mvariant];
    const bool bf = precision == FPIE_MIXED_BF16;
    const MixedVariant::Launch fn = bf ? v.launch_bf16 : v.launch_fp16;
    const MixedVariant::Fold fold = bf ? v.fold_bf16 : v.fold_fp16;
    const int k0 = std::min(c, v.depth);
    const int out0 = e_pending ? (e_last ^ 1) : 0;
    fold(G, mask, g, x[cur], e_pending ? e[e_last] : nullptr, x[cur ^ 1], r, e[out0], mflags,
         mtiles_x, mtiles, k0, st);
    if (e_pending) cur ^= 1;
    int last = out0;
    for (int done = k0, k = 0; done < c; done += k) {
      k = std::min(c - done, v.depth);
      fn(G, mask, r, e[last], e[last ^ 1], mflags, mtiles_x, mtiles, k, 0, st);
      last ^= 1;
    }
    e_last = last;
    e_pending = true;
  }

  // Adds the pending correction to x (end of a step).
  void mixed_flush(cudaStream_t st) {
    if (!e_pending) return;
    launch_refine(precision, L.sweep_grid, L.sweep_block, G, mask, g, x[cur], e[e_last],
                  x[cur ^ 1], nullptr, nullptr, st);
    cur ^= 1;
    e_pending = false;
  }

  int cycle_launches(int c) const {
    const int d = mixed_variants()[mvariant].depth;
    return (c + d - 1) / d;
  }

  // Full cycles with a pending correction replay captured graphs (one per
  // x parity; e_last is the same after every full cycle).
  void run_cycle_graph() {
    if (!e_pending) {  // the first cycle of a step has nothing to fold
      mixed_cycle(stream, kRefine);
      post_launch(this, cycle_launches(kRefine));
      return;
    }
    const int key = cur;
    if (!cycle[key]) {
      const int save_cur = cur, save_last = e_last;
      cudaStream_t cs = nullptr;
      cudaGraph_t graph = nullptr;
      FPIE_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      cudaError_t err = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
      if (err == cudaSuccess) {
        mixed_cycle(cs, kRefine);
        err = cudaStreamEndCapture(cs, &graph);
      }
      if (err == cudaSuccess) err = cudaGraphInstantiate(&cycle[key], graph, 0);
      if (graph) cudaGraphDestroy(graph);
      cudaStreamDestroy(cs);
      cur = save_cur;  // capturing only recorded the launches
      e_last = save_last;
      FPIE_CUDA(err);
    }
    FPIE_CUDA(cudaGraphLaunch(cycle[key], stream));
    post_launch(this, cycle_launches(kRefine));
    cur ^= 1;  // the cycle's fold moved x
  }

  int autotune_mixed(int iters) {
    const std::pair<int, int> key{G.n * 4 + precision, G.m};
    {
      std::lock_guard<std::mutex> lk(tune_mutex());
      auto it = mixed_tune_cache().find(key);
      if (it != mixed_tune_cache().end()) {
        select_mixed(it->second);
        mtuned = true;
        return 0;
      }
    }
    const int ncand = (int)mixed_variants().size();
    if (iters < ncand * (kTuneReps + 1) * kRefine + kRefine) return 0;
    cudaEvent_t e0, e1;
    FPIE_CUDA(cudaEventCreate(&e0));
    FPIE_CUDA(cudaEventCreate(&e1));
    int best = 0, used = 0;
    float best_ms = 1e30f;
    for (int v = 0; v < ncand; ++v) {
      select_mixed(v);
      ensure_mixed();
      run_cycle_graph();
      used += kRefine;
      for (int rep = 0; rep < kTuneReps; ++rep) {
        FPIE_CUDA(cudaEventRecord(e0, stream));
        run_cycle_graph();
        FPIE_CUDA(cudaEventRecord(e1, stream));
        FPIE_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        FPIE_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        used += kRefine;
        if (ms < best_ms) {
          best_ms = ms;
          best = v;
        }
      }
    }
    // The flow kernel: whole launches of 4 cycles, per 64 sweeps.
    if (iters - used >= (kTuneReps + 1) * 4 * kRefine) {
      if (e_pending) {  // fold the candidates' pending correction first
        mixed_flush(stream);
        post_launch(this);
      }
      select_mixed(kFlow);
      run_flow_mixed(4 * kRefine);
      used += 4 * kRefine;
      for (int rep = 0; rep < kTuneReps; ++rep) {
        FPIE_CUDA(cudaEventRecord(e0, stream));
        run_flow_mixed(4 * kRefine);
        FPIE_CUDA(cudaEventRecord(e1, stream));
        FPIE_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        FPIE_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        used += 4 * kRefine;
        if (ms / 4 < best_ms) {
          best_ms = ms / 4;
          best = kFlow;
        }
      }
      check_waits();
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    select_mixed(best);
    mtuned = true;
    std::lock_guard<std::mutex> lk(tune_mutex());
    mixed_tune_cache()[key] = best;
    return used;
  }

  static std::map<std::pair<int, int>, int>& mixed_tune_cache() {
    static std::map<std::pair<int, int>, int> c;
    return c;
  }

  void run_mixed(int iters) {
    ensure_mixed();
    e_pending = false;  // a step starts from a folded x
    if (!mtuned && !pinned) iters -= autotune_mixed(iters);
    if (mvariant == kFlow) {
      if (iters > 0) run_flow_mixed(iters);
      return;
    }
    ensure_mixed();
    while (iters >= kRefine) {
      run_cycle_graph();
      iters -= kRefine;
    }
    if (iters > 0) {
      mixed_cycle(stream, iters);
      post_launch(this, cycle_launches(iters));
    }
    mixed_flush(stream);
    post_launch(this);
  }

  void residual_norms(double* out) {
    FPIE_REQUIRE(out, FPIE_ERR_ARG, "null output array");
    FPIE_REQUIRE(ready, FPIE_ERR_STATE, "no state before reset");
    if (!d_part6) {
      FPIE_CUDA(cudaMalloc(&d_part6, (size_t)L.nparts * 6 * sizeof(double)));
      FPIE_CUDA(cudaMalloc(&d_norm, 6 * sizeof(double)));
    }
    if (!h_norm) FPIE_CUDA(cudaMallocHost(&h_norm, 6 * sizeof(double)));
    refine_norms(stream, nullptr);
    post_launch(this, 2);
    FPIE_CUDA(cudaMemcpyAsync(h_norm, d_norm, 6 * sizeof(double), cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
    std::memcpy(out, h_norm, 6 * sizeof(double));
  }

  // Sweeps in blocks of `check_every` until every channel's max |r| <= tol
  // or max_sweeps are done; returns the sweeps run.
  int solve(double tol, int max_sweeps, int check_every) {
    FPIE_REQUIRE(ready, FPIE_ERR_STATE, "solve called before reset");
    FPIE_REQUIRE(check_every > 0 && max_sweeps >= 0, FPIE_ERR_ARG, "bad solve limits");
    int done = 0;
    double nrm[6];
    residual_norms(nrm);
    while (done < max_sweeps && std::max(nrm[0], std::max(nrm[1], nrm[2])) > tol) {
      const int k = std::min(check_every, max_sweeps - done);
      run_sweeps(k);
      done += k;
      residual_norms(nrm);
    }
    return done;
  }

  void set_kernel(const std::string& name) {
    if (red_black && name != "auto") {
      const std::string launch = tb_variants()[red_black_variant()].name;
      FPIE_REQUIRE(name == launch || name == launch + "d", FPIE_ERR_ARG,
                   "red-black sweeps run on " + launch + " or " + launch + "d, not '" + name + "'");
      select_variant(name == launch ? red_black_variant() : kFlow);
      pinned = true;
      return;
    }
    if (name == "auto") {
      pinned = false;
      tuned = false;
      std::lock_guard<std::mutex> lk(tune_mutex());
      tune_cache().erase({G.n, G.m, red_black});
      return;
    }
    if (precision != FPIE_FP32) {
      int v = -100;
      if (name == "p16w8k16d") v = kFlow;
      for (size_t k = 0; k < mixed_variants().size(); ++k)
        if (name == mixed_variants()[k].name) v = (int)k;
      FPIE_REQUIRE(v != -100, FPIE_ERR_ARG, "unknown mixed-precision grid kernel '" + name + "'");
      select_mixed(v);
      pinned = true;
      return;
    }
    int v = -100;  // unknown
    if (name == "sweep1") v = -1;
    if (name == "p16w8k16t") v = kTma;
    if (name == "p16w8k16d") v = kFlow;
    if (name == "p16w8k12d") v = kFlow12;
    if (name == "p16w8k16dp") v = kFlowP;
    if (name == "p16w8k12dp") v = kFlow12P;
    for (size_t k = 0; k < tb_variants().size(); ++k)
      if (name == tb_variants()[k].name && !tb_variants()[k].red_black) v = (int)k;
    FPIE_REQUIRE(v != -100, FPIE_ERR_ARG, "unknown grid kernel '" + name + "'");
    select_variant(v);
    pinned = true;
  }

  std::string kernel_name() const {
    if (precision != FPIE_FP32)
      return mvariant == kFlow ? std::string("p16w8k16d") : std::string(mixed_variants()[mvariant].name);
    if (variant == kTma) return std::string("p16w8k16t");
    if (variant == kFlow && red_black) return std::string(tb_variants()[red_black_variant()].name) + "d";
    if (variant == kFlow) return std::string("p16w8k16d");
    if (variant == kFlow12) return std::string("p16w8k12d");
    if (variant == kFlowP) return std::string("p16w8k16dp");
    if (variant == kFlow12P) return std::string("p16w8k12dp");
    return variant < 0 ? std::string("sweep1") : std::string(tb_variants()[variant].name);
  }

  void set_precision(int p) {
    FPIE_REQUIRE(p == FPIE_FP32 || p == FPIE_MIXED_FP16 || p == FPIE_MIXED_BF16, FPIE_ERR_ARG,
                 "unknown precision");
    FPIE_REQUIRE(!red_black || p == FPIE_FP32, FPIE_ERR_STATE, "red-black sweeps are FP32 only");
    if (p != precision) {
      precision = p;
      pinned = false;
      drop_graphs();
    }
  }

  void finish(uint8_t* img, float* err) {
    launch_grid_finish(L, G, mask, g, x[cur], img ? img : d_img, d_part, stream);
    post_launch(this);
    launch_finalize(d_part, L.nparts, err ? err : d_err, stream);
    post_launch(this);
  }

  void step_host(int iteration, uint8_t* img_out, float* err_out) {
    FPIE_REQUIRE(img_out && err_out, FPIE_ERR_ARG, "null output array");
    if (!ready) {  // the reference returns an empty image before any reset
      err_out[0] = err_out[1] = err_out[2] = 0.0f;
      return;
    }
    run_sweeps(iteration);
    finish(d_img, d_err);
    const size_t bytes = (size_t)G.n * G.m * 3;
    // Straight into the caller's (pageable) array: measured on GB300 5x
    // faster than a pinned staging buffer plus a host copy.
    FPIE_CUDA(cudaMemcpyAsync(img_out, d_img, bytes, cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaMemcpyAsync(h_err, d_err, 3 * sizeof(float), cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
    check_waits();
    std::memcpy(err_out, h_err, 3 * sizeof(float));
  }

  void get_state(float* out) {
    FPIE_REQUIRE(out, FPIE_ERR_ARG, "null output array");
    FPIE_REQUIRE(ready, FPIE_ERR_STATE, "no state before reset");
    const long long total = (long long)G.n * G.m;
    AsyncScratch scratch(total * 12, stream);
    float* tmp = reinterpret_cast<float*>(scratch.bytes());
    grid_unpack_kernel<<<conv_blocks(total), 256, 0, stream>>>(G, x[cur], tmp);
    post_launch(this);
    FPIE_CUDA(cudaMemcpyAsync(out, tmp, total * 12, cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
    check_waits();
  }
};

Solver* new_grid_solver(int grid_x, int grid_y) {
  return new GridSolverImpl(grid_x, grid_y);
}

static GridSolverImpl* grid_of(fpie_solver* s) {
  return static_cast<GridSolverImpl*>(check_handle(s, 2));
}

}  // namespace fpie

using namespace fpie;

extern "C" {

int fpie_grid_reset(fpie_solver* s, int N, int n, int m, const int32_t* mask,
                    const float* tgt, const float* grad) {
  return guarded([&] { grid_of(s)->reset_host(N, n, m, mask, tgt, grad); });
}

int fpie_grid_step(fpie_solver* s, int iteration, uint8_t* img_out,
                   float* err_out) {
  return guarded([&] { grid_of(s)->step_host(iteration, img_out, err_out); });
}

int fpie_grid_reset_device(fpie_solver* s, int n, int m, const int32_t* mask,
                           const float* tgt, const float* grad) {
  return guarded([&] { grid_of(s)->reset_device(n, m, mask, tgt, grad); });
}

int fpie_grid_reset_images(fpie_solver* s, const uint8_t* src, int src_h, int src_w,
                           const uint8_t* mask, int mask_h, int mask_w, int mask_channels,
                           const uint8_t* tgt, int tgt_h, int tgt_w, int src_row, int src_col,
                           int tgt_row, int tgt_col, int gradient, int on_device, int* box) {
  return guarded([&] {
    grid_of(s)->reset_images(src, src_h, src_w, mask, mask_h, mask_w, mask_channels, tgt, tgt_h,
                             tgt_w, src_row, src_col, tgt_row, tgt_col, gradient, on_device != 0,
                             box);
  });
}

int fpie_grid_get_inputs(fpie_solver* s, int32_t* mask_out, float* grad_out) {
  return guarded([&] { grid_of(s)->get_inputs(mask_out, grad_out); });
}

int fpie_residual_norms(fpie_solver* s, double* out) {
  return guarded([&] { grid_of(s)->residual_norms(out); });
}

int fpie_grid_solve(fpie_solver* s, double tol, int max_sweeps, int check_every,
                    int* sweeps_done) {
  return guarded([&] {
    const int d = grid_of(s)->solve(tol, max_sweeps, check_every);
    if (sweeps_done) *sweeps_done = d;
  });
}

int fpie_grid_set_kernel(fpie_solver* s, const char* name) {
  return guarded([&] {
    FPIE_REQUIRE(name != nullptr, FPIE_ERR_ARG, "null kernel name");
    grid_of(s)->set_kernel(name);
  });
}

int fpie_grid_set_spin_limit(fpie_solver* s, long long spins) {
  return guarded([&] {
    FPIE_REQUIRE(spins >= 0, FPIE_ERR_ARG, "spin limit must be >= 0");
    GridSolverImpl* h = grid_of(s);
    if (spins != h->spin_limit) h->drop_graphs();  // captured TMA launches hold the limit
    h->spin_limit = spins;
  });
}

int fpie_grid_kernel(fpie_solver* s, char* buf, int len) {
  return guarded([&] {
    FPIE_REQUIRE(buf != nullptr && len > 0, FPIE_ERR_ARG, "null or empty buffer");
    const std::string k = grid_of(s)->kernel_name();
    std::snprintf(buf, (size_t)len, "%s", k.c_str());
  });
}

int fpie_grid_step_device(fpie_solver* s, int iteration, uint8_t* img,
                          float* err) {
  return guarded([&] {
    GridSolverImpl* h = grid_of(s);
    h->run_sweeps(iteration);
    if (img || err) h->finish(img, err);
  });
}

}  // extern "C"

namespace fpie {
// Kind-dispatching helpers used by the shared ABI calls in equ.cu.
void grid_sweeps(Solver* s, int iters) { static_cast<GridSolverImpl*>(s)->run_sweeps(iters); }
void grid_get_state(Solver* s, float* out) { static_cast<GridSolverImpl*>(s)->get_state(out); }
void grid_set_precision(Solver* s, int p) { static_cast<GridSolverImpl*>(s)->set_precision(p); }

// Used by the equation solver to run raster-stencil systems on a grid; each
// call enqueues on stream `st`.
void grid_reset_from_equ(Solver* s, cudaStream_t st, int n, int m, int N, const int* pos,
                         const float* xe, const float* be, long long np) {
  s->stream = st;
  static_cast<GridSolverImpl*>(s)->reset_from_equ(n, m, N, pos, xe, be, np);
}
void grid_to_equ(Solver* s, cudaStream_t st, int N, const int* pos, float* xe, long long np) {
  s->stream = st;
  static_cast<GridSolverImpl*>(s)->to_equ(N, pos, xe, np);
}
void grid_run(Solver* s, cudaStream_t st, int iters) {
  s->stream = st;
  static_cast<GridSolverImpl*>(s)->run_sweeps(iters);
}
void grid_pin_kernel(Solver* s, const std::string& name) {
  static_cast<GridSolverImpl*>(s)->set_kernel(name);
}
void grid_set_red_black(Solver* s, bool on) { static_cast<GridSolverImpl*>(s)->set_red_black(on); }
std::string grid_kernel_of(Solver* s) { return static_cast<GridSolverImpl*>(s)->kernel_name(); }
void grid_set_spin(Solver* s, long long spins) {
  GridSolverImpl* h = static_cast<GridSolverImpl*>(s);
  if (spins != h->spin_limit) h->drop_graphs();
  h->spin_limit = spins;
}
}  // namespace fpie
