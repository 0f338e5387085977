// EquSolver backend: Jacobi on the relabelled unknowns through the int32
// neighbour table A (row 0 is the constant-0 unknown absent neighbours use).
//
// Replaces fpie/core/cuda/equ.cu (CudaEquSolver) behind the plugin surface
// of fpie/core/base_solver.h:12-75.  Strict Jacobi with two state buffers,
// the numpy backend's order of additions (fpie/np_solver.py:31-54), planar
// channel arrays, a deterministic residual reduction, checked CUDA calls,
// and neighbour indices validated before any kernel reads through them.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "prep.cuh"

namespace fpie {

int launch_equ_ids(const uint8_t* m01, int mw, int x0, int y0, int n, int m, int* counts,
                   int* ids, cudaStream_t st, bool red_black);
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

// Half a red-black sweep (the reference's OpenMP EquSolver order,
// fpie/core/openmp/equ.cc:67-80, 109-118): rows lo..hi-1 updated in place as
// ((((B + X[U]) + X[D]) + X[L]) + X[R]) / 4.  Every neighbour of these rows
// is of the other colour or row 0 (checked at reset by equ_colour_kernel), so
// no thread of the launch writes a value another thread reads: the result is
// the reference's, whatever the thread order.  Plain loads: x is written
// during the launch (at other addresses).
__global__ void equ_rb_kernel(EquGeom E, const int4* __restrict__ A,
                              const float* __restrict__ b, float* x, int lo, int hi) {
  const int i = lo + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= hi) return;
  const int4 a = __ldg(A + i);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float* xc = x + c * E.np;
    float s = __fadd_rn(__ldg(b + c * E.np + i), xc[a.x]);
    s = __fadd_rn(s, xc[a.y]);
    s = __fadd_rn(s, xc[a.z]);
    s = __fadd_rn(s, xc[a.w]);
    x[c * E.np + i] = __fmul_rn(s, 0.25f);
  }
}

// Counts neighbour entries that break the red-black colouring: a row in
// 1..n_mid-1 (red) must only name rows in n_mid..N-1 or 0, a row in
// n_mid..N-1 (black) only rows in 1..n_mid-1 or 0.
__global__ void equ_colour_kernel(EquGeom E, const int4* __restrict__ A, int n_mid,
                                  unsigned int* __restrict__ bad) {
  unsigned int nbad = 0;
  for (long long i = 1 + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < E.N;
       i += (long long)gridDim.x * blockDim.x) {
    const int4 a = A[i];
    const bool red = i < n_mid;
    const int nb[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) nbad += (unsigned)(nb[k] != 0 && (nb[k] < n_mid) == red);
  }
  if (nbad) atomicAdd(bad, nbad);
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

static int conv_blocks(long long total) { return stride_blocks(total, 256, 32); }

Solver* new_grid_solver(int grid_x, int grid_y);
void grid_reset_from_equ(Solver* s, cudaStream_t st, int n, int m, int N, const int* pos,
                         const float* xe, const float* be, long long np);
void grid_to_equ(Solver* s, cudaStream_t st, int N, const int* pos, float* xe, long long np);
void grid_run(Solver* s, cudaStream_t st, int iters);
void grid_pin_kernel(Solver* s, const std::string& name);
std::string grid_kernel_of(Solver* s);
void grid_set_spin(Solver* s, long long spins);
void grid_set_red_black(Solver* s, bool on);

// Whether the system A (N x 4: up, down, left, right; 0 = the constant row)
// is a 4-neighbour raster stencil, i.e. its unknowns can be placed on a grid
// so that each one's grid neighbours are exactly its A entries (0 where the
// grid pixel holds no unknown).  EquProcessor builds such systems from a
// mask (fpie/process.py:252-266); then the equation sweep
// X' = ((((B + X[U]) + X[D]) + X[L]) + X[R]) / 4 is, operation for
// operation, the grid sweep with grad = B and 0 at every pixel that is not
// an unknown.  On success pos[i] (i >= 1) is unknown i's pixel, row-major in
// an n x m crop: connected components are placed one below the other, a row
// apart, inside a 1-pixel frame.  Row 0 must be the constant (all-zero A).
// n_mid > 0 (red-black order): every component is also placed so that its
// unknowns 1..n_mid-1 land on odd row + col and the others on even (one
// column further right if needed), the colouring the red-black grid kernel
// derives from a pixel's position.  The system must already be 2-coloured
// by n_mid (neighbours of different colours).
static bool raster_embed(int N, const int32_t* A, std::vector<int>& pos, int& n, int& m,
                         int n_mid = 0) {
  if (N < 2) return false;
  for (int k = 0; k < 4; ++k)
    if (A[k] != 0) return false;
  static const int dr[4] = {-1, 1, 0, 0}, dc[4] = {0, 0, -1, 1};
  std::vector<int> R(N, 0), C(N, 0);
  std::vector<char> seen(N, 0);
  std::vector<int> queue;
  queue.reserve(N);
  long long rows = 1;  // the top frame row
  long long width = 0;
  for (int s = 1; s < N; ++s) {
    if (seen[s]) continue;
    const size_t head = queue.size();
    queue.push_back(s);
    seen[s] = 1;
    int rmin = 0, rmax = 0, cmin = 0, cmax = 0;
    for (size_t q = head; q < queue.size(); ++q) {
      const int i = queue[q];
      for (int k = 0; k < 4; ++k) {
        const int j = A[4 * (size_t)i + k];
        if (j == 0) continue;
        if (j < 0 || j >= N) return false;
        const int rj = R[i] + dr[k], cj = C[i] + dc[k];
        if (!seen[j]) {
          seen[j] = 1;
          R[j] = rj;
          C[j] = cj;
          rmin = std::min(rmin, rj);
          rmax = std::max(rmax, rj);
          cmin = std::min(cmin, cj);
          cmax = std::max(cmax, cj);
          queue.push_back(j);
        } else if (R[j] != rj || C[j] != cj) {
          return false;
        }
      }
    }
    // The seed s sits at (rows - rmin, 1 - cmin); with a colouring, shift
    // the component right by one column if s would get the wrong parity.
    int shift = 0;
    if (n_mid > 0) {
      const bool odd = ((rows - rmin) + (1 - cmin)) % 2 != 0;
      if (odd != (s < n_mid)) shift = 1;
    }
    for (size_t q = head; q < queue.size(); ++q) {
      R[queue[q]] += (int)(rows - rmin);
      C[queue[q]] += 1 - cmin + shift;
    }
    rows += (long long)(rmax - rmin + 1) + 1;  // the component, then an empty row
    width = std::max(width, (long long)(cmax - cmin + 1) + 2 + shift);
    if (rows > (1LL << 30)) return false;
  }
  // The crop must stay comparable to the system (many scattered pieces would
  // make a mostly empty grid; the gather kernel is better there).
  if (rows * width > 8LL * N + (1LL << 20) || rows * width > (1LL << 31) / 4) return false;
  n = (int)rows;
  m = (int)width;
  std::vector<int> occ((size_t)n * m, 0);
  for (int i = 1; i < N; ++i) {
    int& o = occ[(size_t)R[i] * m + C[i]];
    if (o) return false;  // two unknowns on one pixel
    o = i;
  }
  for (int i = 1; i < N; ++i)
    for (int k = 0; k < 4; ++k)
      if (occ[(size_t)(R[i] + dr[k]) * m + (C[i] + dc[k])] != A[4 * (size_t)i + k]) return false;
  pos.assign(N, 0);
  for (int i = 1; i < N; ++i) pos[i] = R[i] * m + C[i];
  return true;
}

// Pixels of the unknowns from their target coordinates (the GPU-side reset
// knows them): pos[i] = (rows[i-1] - r0) * m + (cols[i-1] - c0).
__global__ void equ_pos_kernel(int N, const int* __restrict__ rows, const int* __restrict__ cols,
                               int r0, int c0, int m, int* __restrict__ pos) {
  for (long long i = 1 + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x)
    pos[i] = (rows[i - 1] - r0) * m + (cols[i - 1] - c0);
}

// Counts violations of a cached placement (pos, occ: unknown id per crop
// pixel, 0 elsewhere; m pixels per row) by the system now in A / x / b:
// row 0 must be the zero constant, and every unknown's four grid neighbours
// must be exactly its A entries -- the condition raster_embed establishes.
__global__ void equ_layout_check_kernel(EquGeom E, const int4* __restrict__ A,
                                        const float* __restrict__ x, const float* __restrict__ b,
                                        const int* __restrict__ pos, const int* __restrict__ occ,
                                        int m, unsigned int* __restrict__ bad) {
  unsigned int nbad = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < E.N;
       i += (long long)gridDim.x * blockDim.x) {
    const int4 a = A[i];
    if (i == 0) {
      nbad += (a.x | a.y | a.z | a.w) != 0;
      for (int c = 0; c < 3; ++c) nbad += (x[c * E.np] != 0.f) + (b[c * E.np] != 0.f);
      continue;
    }
    const int p = pos[i];
    nbad += (occ[p - m] != a.x) + (occ[p + m] != a.y) + (occ[p - 1] != a.z) + (occ[p + 1] != a.w);
  }
  if (nbad) atomicAdd(bad, nbad);
}

// A caller's placement: counts unknowns that do not own their pixel (two on
// one pixel) and, with a colouring (n_mid > 0), unknowns whose pixel has the
// wrong parity of row + col (1..n_mid-1 odd, the others even).
__global__ void equ_place_check_kernel(int N, const int* __restrict__ pos,
                                       const int* __restrict__ occ, int m, int n_mid,
                                       unsigned int* __restrict__ bad) {
  unsigned int nbad = 0;
  for (long long i = 1 + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    const int p = pos[i];
    nbad += occ[p] != (int)i;
    if (n_mid > 0) nbad += (((p / m + p % m) & 1) != 0) != (i < n_mid);
  }
  if (nbad) atomicAdd(bad, nbad);
}

__global__ void equ_occ_kernel(int N, const int* __restrict__ pos, int* __restrict__ occ) {
  for (long long i = 1 + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x)
    occ[pos[i]] = (int)i;
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
  float* h_err = nullptr;
  unsigned int* h_bad = nullptr;
  int nparts = 0;
  static constexpr int kChunk = 64;
  cudaGraphExec_t chunk[2] = {nullptr, nullptr};

  // ---- iteration order: FPIE_ORDER_JACOBI (numpy) or FPIE_ORDER_RED_BLACK
  // (the reference's OpenMP EquSolver).  n_mid: the first even id of the
  // last red-black partition (fpie/core/openmp/equ.cc:42); the state is
  // updated in place in x[cur].
  int order = FPIE_ORDER_JACOBI;
  int n_mid = 0;
  cudaGraphExec_t rb_chunk = nullptr;
  int rb_chunk_mid = -1;

  // ---- grid mode: systems that are a 4-neighbour raster stencil run on an
  // internal grid solver (its autotuned temporally blocked kernels); the
  // state lives there and is gathered back into x[cur] when needed.
  std::string kernel_req = "auto";  // "auto" | "gather" | a grid kernel name
  Solver* grid = nullptr;
  int* d_pos = nullptr;             // per unknown: its crop pixel
  int pos_cap = 0;
  bool use_grid = false;
  bool grid_newer = false;          // grid state ahead of x[cur]
  // The last placement found by the host search, kept to be re-checked on
  // the device at the next reset of a system of the same size.
  int* d_occ = nullptr;             // unknown id per crop pixel
  int lay_N = 0, lay_n = 0, lay_m = 0;
  int lay_mid = 0;                  // the colouring it was placed for (0: none)
  size_t occ_cap = 0;               // ints allocated at d_occ
  long long spin_limit = 1LL << 26;

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
    delete grid;
    cudaFree(d_pos);
    cudaFree(d_occ);
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
    if (rb_chunk) cudaGraphExecDestroy(rb_chunk);
    rb_chunk = nullptr;
    rb_chunk_mid = -1;
  }

  void set_order(int o) {
    FPIE_REQUIRE(o == FPIE_ORDER_JACOBI || o == FPIE_ORDER_RED_BLACK, FPIE_ERR_ARG,
                 "order must be FPIE_ORDER_JACOBI or FPIE_ORDER_RED_BLACK");
    if (o == order) return;
    cudaStreamSynchronize(stream);
    order = o;
    n_mid = 0;
    ready = false;  // the loaded system was numbered for the other order
    use_grid = false;
    grid_newer = false;
  }

  // ids of a partition: row-major (Jacobi), or odd row+col first, then even
  // (red-black; fpie/core/openmp/equ.cc:22-56), remembering n_mid.
  void partition(const int32_t* mask, int n, int m, int32_t* ids) {
    const long long total = (long long)n * m;
    int32_t cnt = 0;
    if (order == FPIE_ORDER_JACOBI) {
      for (long long k = 0; k < total; ++k) ids[k] = mask[k] > 0 ? ++cnt : 0;
      return;
    }
    for (int parity = 1; parity >= 0; --parity) {
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < m; ++j) {
          const long long k = (long long)i * m + j;
          if ((i + j) % 2 == parity) ids[k] = mask[k] > 0 ? ++cnt : 0;
        }
      if (parity == 1) n_mid = cnt + 1;
    }
  }

  // Red-black: the loaded system must follow the colouring of the last
  // partition, or the in-place halves would race.
  void check_colouring() {
    if (n_mid < 1 || n_mid > E.N) {
      release();
      throw Error{FPIE_ERR_STATE, "red-black order: call partition() on the system's mask before "
                                  "reset (n_mid = " + std::to_string(n_mid) + ", N = " +
                                  std::to_string(E.N) + ")"};
    }
    FPIE_CUDA(cudaMemsetAsync(d_bad, 0, sizeof(unsigned int), stream));
    equ_colour_kernel<<<conv_blocks(E.N), 256, 0, stream>>>(E, A, n_mid, d_bad);
    post_launch(this);
    FPIE_CUDA(cudaMemcpyAsync(h_bad, d_bad, sizeof(unsigned int), cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
    if (*h_bad) {
      release();
      throw Error{FPIE_ERR_ARG, "red-black order: A holds " + std::to_string(*h_bad) +
                                    " neighbour(s) of a row's own colour for the last partition"};
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
    A = nullptr;
    x[0] = x[1] = b = nullptr;
    d_img = nullptr;
    d_part = nullptr;
    d_err = nullptr;
    ready = false;
    use_grid = false;
    grid_newer = false;
  }

  void ensure_pos(int N) {
    if (N > pos_cap) {
      cudaFree(d_pos);
      d_pos = nullptr;
      FPIE_CUDA(cudaMalloc(&d_pos, sizeof(int) * (size_t)N));
      pos_cap = N;
    }
  }

  // Moves the system into grid mode at crop size n x m (d_pos filled).
  void enter_grid(int n, int m) {
    if (!grid) grid = new_grid_solver(8, 8);
    grid_set_spin(grid, spin_limit);
    grid_set_red_black(grid, order == FPIE_ORDER_RED_BLACK);
    if (kernel_req != "auto") grid_pin_kernel(grid, kernel_req);
    grid_reset_from_equ(grid, stream, n, m, E.N, d_pos, x[0], b, E.np);
    use_grid = true;
    grid_newer = false;
  }

  // Whether the last placement fits the system now loaded (device check).
  int colour_mid() const { return order == FPIE_ORDER_RED_BLACK ? n_mid : 0; }

  bool cached_layout_fits() {
    if (!d_occ || lay_N != E.N || lay_N < 2 || lay_mid != colour_mid()) return false;
    FPIE_CUDA(cudaMemsetAsync(d_bad, 0, sizeof(unsigned int), stream));
    equ_layout_check_kernel<<<conv_blocks(E.N), 256, 0, stream>>>(E, A, x[0], b, d_pos, d_occ,
                                                                   lay_m, d_bad);
    post_launch(this);
    FPIE_CUDA(cudaMemcpyAsync(h_bad, d_bad, sizeof(unsigned int), cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
    return *h_bad == 0;
  }

  // After a reset from host or device arrays: grid mode when the system is
  // a raster stencil (and the kernel choice allows it).  hA: the system's A
  // on the host, or NULL to fetch it from the device if the search is needed.
  void choose_mode(const int32_t* hA) {
    use_grid = false;
    if (order == FPIE_ORDER_RED_BLACK) {
      FPIE_REQUIRE(kernel_req == "auto" || kernel_req == "gather" || kernel_req.rfind("rb", 0) == 0,
                   FPIE_ERR_ARG,
                   "red-black order runs on its own kernels, not grid kernel '" + kernel_req + "'");
      check_colouring();
    }
    if (kernel_req == "gather") return;
    if (cached_layout_fits()) {
      enter_grid(lay_n, lay_m);
      return;
    }
    std::vector<int32_t> fetched;
    if (!hA) {
      fetched.resize((size_t)E.N * 4);
      FPIE_CUDA(cudaMemcpyAsync(fetched.data(), A, (size_t)E.N * 16, cudaMemcpyDeviceToHost, stream));
      FPIE_CUDA(cudaStreamSynchronize(stream));
      hA = fetched.data();
    }
    float row0[6];
    for (int c = 0; c < 3; ++c) {
      FPIE_CUDA(cudaMemcpyAsync(row0 + c, x[0] + c * E.np, 4, cudaMemcpyDeviceToHost, stream));
      FPIE_CUDA(cudaMemcpyAsync(row0 + 3 + c, b + c * E.np, 4, cudaMemcpyDeviceToHost, stream));
    }
    FPIE_CUDA(cudaStreamSynchronize(stream));
    bool zero_row0 = true;
    for (float v : row0) zero_row0 = zero_row0 && v == 0.f;
    std::vector<int> pos;
    int n = 0, m = 0;
    const bool ok = zero_row0 && raster_embed(E.N, hA, pos, n, m, colour_mid());
    if (!ok) {
      FPIE_REQUIRE(kernel_req == "auto", FPIE_ERR_ARG,
                   "grid kernel '" + kernel_req + "' needs a 4-neighbour raster system "
                   "(row 0 constant and zero; every unknown's up/down/left/right in A)");
      return;
    }
    ensure_pos(E.N);
    FPIE_CUDA(cudaMemcpyAsync(d_pos, pos.data(), sizeof(int) * (size_t)E.N, cudaMemcpyHostToDevice,
                              stream));
    cudaFree(d_occ);
    d_occ = nullptr;
    occ_cap = 0;
    lay_N = 0;
    FPIE_CUDA(cudaMalloc(&d_occ, sizeof(int) * (size_t)n * m));
    occ_cap = (size_t)n * m;
    FPIE_CUDA(cudaMemsetAsync(d_occ, 0, sizeof(int) * (size_t)n * m, stream));
    equ_occ_kernel<<<conv_blocks(E.N), 256, 0, stream>>>(E.N, d_pos, d_occ);
    post_launch(this);
    lay_N = E.N;
    lay_n = n;
    lay_m = m;
    lay_mid = colour_mid();
    enter_grid(n, m);
    FPIE_CUDA(cudaStreamSynchronize(stream));  // pos is a host vector
  }

  // After a reset with the caller's placement of the unknowns (pos[i] =
  // row * m + col in an n x m crop, as EquProcessor knows it): the placement
  // is checked on the device (every unknown alone on its pixel, its four
  // grid neighbours exactly its A entries, row 0 the zero constant, and in
  // red-black order the colour parity) instead of being searched for on the
  // host.  A placement that does not fit the system is an argument error.
  void choose_mode_placed(const int32_t* hpos, int n, int m) {
    use_grid = false;
    if (order == FPIE_ORDER_RED_BLACK) {
      FPIE_REQUIRE(kernel_req == "auto" || kernel_req == "gather" || kernel_req.rfind("rb", 0) == 0,
                   FPIE_ERR_ARG,
                   "red-black order runs on its own kernels, not grid kernel '" + kernel_req + "'");
      check_colouring();
    }
    if (kernel_req == "gather" || E.N < 2) return;
    FPIE_REQUIRE(n >= 3 && m >= 3 && (long long)n * m <= (1LL << 31) / 4, FPIE_ERR_ARG,
                 "placement crop must be at least 3 x 3 and below 2^29 pixels");
    for (int i = 1; i < E.N; ++i) {  // interior pixels only: the check reads all four neighbours
      const int p = hpos[i], r = p / m, c = p % m;
      FPIE_REQUIRE(p >= 0 && r >= 1 && r <= n - 2 && c >= 1 && c <= m - 2, FPIE_ERR_ARG,
                   "placement of unknown " + std::to_string(i) + " is not inside the crop's frame");
    }
    ensure_pos(E.N);
    FPIE_CUDA(cudaMemcpyAsync(d_pos, hpos, sizeof(int) * (size_t)E.N, cudaMemcpyHostToDevice, stream));
    lay_N = 0;
    if (!d_occ || occ_cap < (size_t)n * m) {
      cudaFree(d_occ);
      d_occ = nullptr;
      occ_cap = 0;
      FPIE_CUDA(cudaMalloc(&d_occ, sizeof(int) * (size_t)n * m));
      occ_cap = (size_t)n * m;
    }
    FPIE_CUDA(cudaMemsetAsync(d_occ, 0, sizeof(int) * (size_t)n * m, stream));
    equ_occ_kernel<<<conv_blocks(E.N), 256, 0, stream>>>(E.N, d_pos, d_occ);
    post_launch(this);
    FPIE_CUDA(cudaMemsetAsync(d_bad, 0, sizeof(unsigned int), stream));
    equ_place_check_kernel<<<conv_blocks(E.N), 256, 0, stream>>>(E.N, d_pos, d_occ, m, colour_mid(),
                                                                 d_bad);
    post_launch(this);
    equ_layout_check_kernel<<<conv_blocks(E.N), 256, 0, stream>>>(E, A, x[0], b, d_pos, d_occ, m,
                                                                   d_bad);
    post_launch(this);
    FPIE_CUDA(cudaMemcpyAsync(h_bad, d_bad, sizeof(unsigned int), cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
    if (*h_bad) {
      release();
      throw Error{FPIE_ERR_ARG, "the placement does not fit the system: " + std::to_string(*h_bad) +
                                    " mismatched unknowns or neighbours"};
    }
    lay_N = E.N;
    lay_n = n;
    lay_m = m;
    lay_mid = colour_mid();
    enter_grid(n, m);
  }

  void reset_host_placed(int N, const int32_t* hA, const float* hX, const float* hB,
                         const int32_t* hpos, int n, int m) {
    FPIE_REQUIRE(hA && hX && hB && hpos, FPIE_ERR_ARG, "null input array");
    allocate(N);
    AsyncScratch scratch((size_t)N * 24, stream);
    float* stage = reinterpret_cast<float*>(scratch.bytes());
    FPIE_CUDA(cudaMemcpyAsync(A, hA, (size_t)N * 16, cudaMemcpyHostToDevice, stream));
    FPIE_CUDA(cudaMemcpyAsync(stage, hX, (size_t)N * 12, cudaMemcpyHostToDevice, stream));
    FPIE_CUDA(cudaMemcpyAsync(stage + (size_t)N * 3, hB, (size_t)N * 12, cudaMemcpyHostToDevice, stream));
    pack_and_check(stage, stage + (size_t)N * 3);
    choose_mode_placed(hpos, n, m);
    FPIE_CUDA(cudaStreamSynchronize(stream));
  }

  // x[cur] up to date with the grid state.
  void sync_from_grid() {
    if (use_grid && grid_newer) {
      grid_to_equ(grid, stream, E.N, d_pos, x[cur], E.np);
      grid_newer = false;
    }
  }

  void check_async() override {
    if (grid) grid->check_async();
  }

  void set_kernel(const std::string& name) {
    kernel_req = name;
    if (grid && name != "auto" && name != "gather") grid_pin_kernel(grid, name);
    if (grid && name == "auto") grid_pin_kernel(grid, "auto");
  }

  std::string kernel_name() const {
    if (!use_grid) return order == FPIE_ORDER_RED_BLACK ? "red_black" : "gather";
    return "grid:" + grid_kernel_of(grid);
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
    choose_mode(hA);
    FPIE_CUDA(cudaStreamSynchronize(stream));
  }

  void reset_device(int N, const int32_t* dA, const float* dX, const float* dB) {
    FPIE_REQUIRE(dA && dX && dB, FPIE_ERR_ARG, "null input array");
    allocate(N);
    FPIE_CUDA(cudaMemcpyAsync(A, dA, (size_t)N * 16, cudaMemcpyDeviceToDevice, stream));
    pack_and_check(dX, dB);
    choose_mode(nullptr);
  }

  int* d_rows = nullptr;  // target coordinates of unknowns 1..N-1 (GPU reset)
  int* d_cols = nullptr;

  // GPU-side counterpart of EquProcessor.reset (fpie/process.py:192-271):
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
    const bool rb = order == FPIE_ORDER_RED_BLACK;
    const int nb = launch_equ_ids(m01, mw, x0, y0, n, m, counts, ids, stream, rb);
    post_launch(this, rb ? 7 : 3);
    int tallies[2] = {0, 0};  // unknowns, and (red-black) the odd ones
    FPIE_CUDA(cudaMemcpyAsync(tallies, counts + nb, (rb ? 2 : 1) * sizeof(int),
                              cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
    const int unknowns = tallies[0];
    if (rb) n_mid = tallies[1] + 1;
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
    use_grid = false;
    lay_N = 0;  // d_pos is rewritten below; the cached placement no longer matches d_occ
    if (kernel_req != "gather" && N > 1) {  // a mask's system: its pixels are known
      ensure_pos(N);
      equ_pos_kernel<<<conv_blocks(N), 256, 0, stream>>>(N, d_rows, d_cols, t_row + x0,
                                                          t_col + y0, m, d_pos);
      post_launch(this);
      enter_grid(n, m);
    }
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

  void rb_sweep_once(cudaStream_t st) {
    if (n_mid > 1)
      equ_rb_kernel<<<(n_mid - 1 + block - 1) / block, block, 0, st>>>(E, A, b, x[cur], 1, n_mid);
    if (E.N > n_mid)
      equ_rb_kernel<<<(E.N - n_mid + block - 1) / block, block, 0, st>>>(E, A, b, x[cur], n_mid, E.N);
  }

  void run_rb(int iters) {
    const int per = (n_mid > 1) + (E.N > n_mid);
    while (iters >= kChunk) {
      if (!rb_chunk || rb_chunk_mid != n_mid) {
        if (rb_chunk) cudaGraphExecDestroy(rb_chunk);
        rb_chunk = nullptr;
        cudaStream_t cs = nullptr;
        cudaGraph_t graph = nullptr;
        FPIE_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
          for (int k = 0; k < kChunk; ++k) rb_sweep_once(cs);
          e = cudaStreamEndCapture(cs, &graph);
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&rb_chunk, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        cudaStreamDestroy(cs);
        FPIE_CUDA(e);
        rb_chunk_mid = n_mid;
      }
      FPIE_CUDA(cudaGraphLaunch(rb_chunk, stream));
      post_launch(this, kChunk * per);
      iters -= kChunk;
    }
    for (; iters > 0; --iters) {
      rb_sweep_once(stream);
      post_launch(this, per);
    }
  }

  void run_sweeps(int iters) {
    FPIE_REQUIRE(ready, FPIE_ERR_STATE, "step called before reset");
    if (order == FPIE_ORDER_RED_BLACK && !use_grid) {
      run_rb(iters);
      return;
    }
    if (use_grid) {
      if (iters > 0) {
        grid_run(grid, stream, iters);
        grid_newer = true;
      }
      return;
    }
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
    sync_from_grid();
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
    // Straight into the caller's (pageable) array: measured on GB300 5x
    // faster than a pinned staging buffer plus a host copy.
    FPIE_CUDA(cudaMemcpyAsync(img_out, d_img, bytes, cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaMemcpyAsync(h_err, d_err, 3 * sizeof(float), cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
    check_async();
    std::memcpy(err_out, h_err, 3 * sizeof(float));
  }

  void get_state(float* out) {
    FPIE_REQUIRE(out, FPIE_ERR_ARG, "null output array");
    FPIE_REQUIRE(ready, FPIE_ERR_STATE, "no state before reset");
    sync_from_grid();
    AsyncScratch scratch((size_t)E.N * 12, stream);
    float* tmp = reinterpret_cast<float*>(scratch.bytes());
    equ_unpack_kernel<<<conv_blocks(E.N), 256, 0, stream>>>(E, x[cur], tmp);
    post_launch(this);
    FPIE_CUDA(cudaMemcpyAsync(out, tmp, (size_t)E.N * 12, cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
    check_async();
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
    EquSolverImpl* h = equ_of(s);
    FPIE_REQUIRE(mask && ids_out, FPIE_ERR_ARG, "null array");
    FPIE_REQUIRE(n >= 0 && m >= 0, FPIE_ERR_ARG, "negative mask shape");
    h->partition(mask, n, m, ids_out);
  });
}

int fpie_equ_set_order(fpie_solver* s, int order) {
  return guarded([&] { equ_of(s)->set_order(order); });
}

int fpie_equ_order(fpie_solver* s, int* order, int* n_mid) {
  return guarded([&] {
    FPIE_REQUIRE(order != nullptr, FPIE_ERR_ARG, "null output");
    const EquSolverImpl* h = equ_of(s);
    *order = h->order;
    if (n_mid) *n_mid = h->n_mid;
  });
}

int fpie_equ_reset(fpie_solver* s, int N, const int32_t* A, const float* X,
                   const float* B) {
  return guarded([&] { equ_of(s)->reset_host(N, A, X, B); });
}

int fpie_equ_reset_placed(fpie_solver* s, int N, const int32_t* A, const float* X, const float* B,
                          const int32_t* pos, int n, int m) {
  return guarded([&] { equ_of(s)->reset_host_placed(N, A, X, B, pos, n, m); });
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

int fpie_equ_set_kernel(fpie_solver* s, const char* name) {
  return guarded([&] {
    FPIE_REQUIRE(name != nullptr, FPIE_ERR_ARG, "null kernel name");
    equ_of(s)->set_kernel(name);
  });
}

int fpie_equ_kernel(fpie_solver* s, char* buf, int len) {
  return guarded([&] {
    FPIE_REQUIRE(buf != nullptr && len > 0, FPIE_ERR_ARG, "null or empty buffer");
    const std::string k = equ_of(s)->kernel_name();
    std::snprintf(buf, (size_t)len, "%s", k.c_str());
  });
}

int fpie_equ_raster_layout(int N, const int32_t* A, int32_t* pos, int* n, int* m) {
  return guarded([&] {
    FPIE_REQUIRE(A && pos && n && m, FPIE_ERR_ARG, "null argument");
    FPIE_REQUIRE(N >= 1, FPIE_ERR_ARG, "N must be at least 1");
    std::vector<int> p;
    int nn = 0, mm = 0;
    FPIE_REQUIRE(raster_embed(N, A, p, nn, mm), FPIE_ERR_ARG, "not a 4-neighbour raster system");
    pos[0] = -1;
    for (int i = 1; i < N; ++i) pos[i] = p[i];
    *n = nn;
    *m = mm;
  });
}

int fpie_equ_set_spin_limit(fpie_solver* s, long long spins) {
  return guarded([&] {
    FPIE_REQUIRE(spins >= 0, FPIE_ERR_ARG, "spin limit must be >= 0");
    EquSolverImpl* h = equ_of(s);
    h->spin_limit = spins;
    if (h->grid) grid_set_spin(h->grid, spins);
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
