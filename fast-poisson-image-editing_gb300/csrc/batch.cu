// Batched form: many paste jobs of uneven size in one persistent launch.
//
// Every job is a grid problem with its own padded planes (the GridSolver
// layout).  Its sweeps are cut into levels of K sweeps (the tile kernel's
// temporal depth); a work item is one (job, active tile, channel) at one
// level.  Items are queued level-major -- all jobs' level 0, then level 1,
// ... -- and a persistent kernel of (SMs x occupancy) CTAs pulls them with
// one atomic each.  Before running an item at level z a CTA waits until its
// job has finished every item of level z-1 (a per-job counter); items of
// other jobs keep the SMs busy meanwhile, which is what batching buys over
// one launch per job.  No deadlock is possible: an item is taken only by a
// running CTA, and every item it waits for was taken earlier by another
// running CTA that waits only for still earlier levels.  The wait is bounded
// anyway: past the spin limit the kernel records an error and every CTA
// leaves, and the host reports FPIE_ERR_TIMEOUT.
//
// Arithmetic per pixel is the grid kernels' (numpy order), so each job's
// result is bit-identical to a GridSolver run of the same sweeps, alone or
// in any mix.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "prep.cuh"
#include "grid_kernels.cuh"
#include "grid_mixed.cuh"
#include "grid_tbp.cuh"
#include "mixed_levels.cuh"

namespace fpie {

struct BJobDev {
  GridGeom G;
  const uint8_t* mask;
  const float* g;
  float* x[2];
  void* e[2];       // mixed forms: the correction (FP16 / BF16 planes)
  float* r;         // mixed forms: the FP32 residual planes
  int tiles_x;      // tiles per row of this job
  int ntiles;       // active tiles
  int tile_off;     // first entry of this job in the tile list
  int sweeps;       // sweeps in this launch
  int parity;       // buffer holding the state at level 0
};

struct BQueue {
  const BJobDev* jobs;
  const int* order;        // jobs sorted by level count, descending
  const long long* ct;     // ct[k] = items of sorted jobs [0, k)
  const long long* lo;     // lo[z] = items before level z; lo[nlevels] = total
  const int* act;          // act[z] = jobs (sorted prefix) still active at level z
  const int2* tiles;       // (tile index, flag) per job, concatenated
  int nlevels;
  int njobs;
  int ntiles;              // entries of `tiles`
  int smem_tables;         // job records and tile entries are copied to dynamic shared memory
  unsigned long long* next;
  int* done;
  int* error;
  long long spin_limit;
};

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

template <typename T>
__device__ __forceinline__ int upper_bound_idx(const T* a, int n, T v) {
  int lo = 0, hi = n;  // first index with a[i] > v
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] <= v) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Item bodies, out of line: inlined into the work loop, the compiler's
// register assignment needs several times the register moves per sweep of
// the same code in a launch-per-tile kernel (measured with instruction
// counters on the grid kernels).
template <int R, int W, int K, bool FULL, typename TS>
__device__ __noinline__ void batch_sweep_item(const GridGeom& G, const uint8_t* mask,
                                              const float* gc, const TS* xc, TS* oc,
                                              long long base, int ks, int lane, int w,
                                              float4 (&edge)[2][2][W][32]) {
  tbp_body<R, W, K, FULL, TS, false, true>(G, mask, gc, xc, oc, base, ks, lane, w, edge);
}

template <int R, int W, int K, bool FULL, typename TS, bool HASE>
__device__ __noinline__ void batch_fold_item(const GridGeom& G, const uint8_t* mask,
                                             const float* gc, const float* xin, const TS* elast,
                                             float* xout, float* rout, TS* eout, long long base,
                                             int ks, int lane, int w,
                                             float4 (&edge)[2][2][W][32]) {
  tbp_fold_body<R, W, K, FULL, TS, HASE, true>(G, mask, gc, xin, elast, xout, rout, eout, base,
                                               ks, lane, w, edge);
}

template <int R, int W, int K, typename TS>
__global__ void __launch_bounds__(W * 32)
batch_persistent_kernel(BQueue Q) {
  constexpr bool MIXED = !std::is_same<TS, float>::value;
  constexpr int TH = W * R - 2 * K;
  constexpr int TW = 128 - 2 * K;
  // The queue tables, in shared memory when they fit: decoding an item is
  // two binary searches, which through global memory would be ~20 dependent
  // L2 round trips on every item's critical path.
  constexpr int kSL = 640, kSJ = 320;
  __shared__ float4 edge[2][2][W][32];
  __shared__ long long s_lo[kSL + 1], s_ct[kSJ + 1];
  __shared__ int s_act[kSL], s_order[kSJ];
  __shared__ long long s_idx;
  __shared__ int s_stop;
  __shared__ int2 s_tf;
  // The current item's job record, copied by warp 0 (one round trip) so
  // that the CTA does not chase it field by field through global memory --
  // unless every job record (and tile entry) was copied to dynamic shared
  // memory at the start (Q.smem_tables), which takes both round trips off
  // every item's critical path.
  __shared__ __align__(16) BJobDev s_job;
  extern __shared__ __align__(16) unsigned char batch_dyn[];
  BJobDev* s_jobs = reinterpret_cast<BJobDev*>(batch_dyn);
  int2* s_tiles = reinterpret_cast<int2*>(batch_dyn + sizeof(BJobDev) * (size_t)Q.njobs);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const bool fits = Q.nlevels <= kSL && Q.njobs <= kSJ;
  if (fits) {
    for (int k = threadIdx.x; k <= Q.nlevels; k += blockDim.x) s_lo[k] = Q.lo[k];
    for (int k = threadIdx.x; k < Q.nlevels; k += blockDim.x) s_act[k] = Q.act[k];
    for (int k = threadIdx.x; k <= Q.njobs; k += blockDim.x) s_ct[k] = Q.ct[k];
    for (int k = threadIdx.x; k < Q.njobs; k += blockDim.x) s_order[k] = Q.order[k];
  }
  if (Q.smem_tables) {
    static_assert(sizeof(BJobDev) % 4 == 0, "job record in words");
    const int words = (int)(sizeof(BJobDev) / 4) * Q.njobs;
    const int* src = reinterpret_cast<const int*>(Q.jobs);
    int* dst = reinterpret_cast<int*>(s_jobs);
    for (int k = threadIdx.x; k < words; k += blockDim.x) dst[k] = src[k];
    for (int k = threadIdx.x; k < Q.ntiles; k += blockDim.x) s_tiles[k] = Q.tiles[k];
  }
  const long long* lo = fits ? s_lo : Q.lo;
  const long long* ct = fits ? s_ct : Q.ct;
  const int* act = fits ? s_act : Q.act;
  const int* order = fits ? s_order : Q.order;
  const long long total = Q.lo[Q.nlevels];
  if (threadIdx.x == 0) s_idx = (long long)atomicAdd(Q.next, 1ULL);
  __syncthreads();
  for (;;) {
    const long long idx = s_idx;
    if (idx >= total) break;
    const int z = upper_bound_idx(lo, Q.nlevels + 1, idx) - 1;
    const long long i = idx - lo[z];
    const int js = upper_bound_idx(ct, act[z] + 1, i) - 1;
    const int j = order[js];
    const int tc = (int)(i - ct[js]);
    const int ti = tc / 3, c = tc - 3 * ti;
    if (w == 0 && !Q.smem_tables) {
      const int* src = reinterpret_cast<const int*>(Q.jobs + j);
      int* dst = reinterpret_cast<int*>(&s_job);
      for (int k = lane; k < (int)(sizeof(BJobDev) / 4); k += 32) dst[k] = src[k];
      __syncwarp();
    }
    const BJobDev& J = Q.smem_tables ? s_jobs[j] : s_job;
    unsigned long long nxt = 0;
    if (threadIdx.x == 0) {
      s_tf = Q.smem_tables ? s_tiles[J.tile_off + ti] : Q.tiles[J.tile_off + ti];
      const int need = J.ntiles * 3 * z;
      long long spins = 0;
      int stop = 0;
      // Acquire loads: the read that sees the count orders the producers'
      // writes before everything this thread does next, and the CTA barrier
      // below carries that order to the other threads -- no separate fence.
      while (ld_acquire_gpu(Q.done + j) < need) {
        if (*(volatile int*)Q.error) { stop = 1; break; }
        if (++spins > Q.spin_limit) {
          atomicExch(Q.error, 1);
          stop = 1;
          break;
        }
        __nanosleep(128);
      }
      s_stop = stop;
      // The next item is taken now, so that the atomic's round trip
      // overlaps this item's sweeps.  (A CTA then holds two items; the
      // lowest unfinished item is always one being worked on, since a held
      // next item is higher than its CTA's current one, and it waits only
      // for lower items: no deadlock.)
      if (!stop) nxt = atomicAdd(Q.next, 1ULL);
    }
    __syncthreads();
    if (s_stop) break;
    const int2 tf = s_tf;
    const int ty = tf.x / J.tiles_x, tx = tf.x - ty * J.tiles_x;
    const long long base = J.G.at(ty * TH - K + w * R, tx * TW - K + 4 * lane);
    const long long co = c * J.G.plane;
    const float* gc = J.g + co;
    if (!MIXED) {
      const int pin = (J.parity + z) & 1;
      const float* xc = J.x[pin] + co;
      float* oc = J.x[pin ^ 1] + co;
      const int ks = min(K, J.sweeps - z * K);
      if (tf.y == 2)
        batch_sweep_item<R, W, K, true, float>(J.G, J.mask, gc, xc, oc, base, ks, lane, w, edge);
      else
        batch_sweep_item<R, W, K, false, float>(J.G, J.mask, gc, xc, oc, base, ks, lane, w, edge);
    } else {
      const MixedLevel L = mixed_level(z, J.sweeps, K);
      TS* e0 = static_cast<TS*>(J.e[0]);
      TS* e1 = static_cast<TS*>(J.e[1]);
      if (L.type == 0) {
        // x parity before this cycle's fold: one flip per earlier fold.
        const int xp = (J.parity + (L.cycle > 0 ? L.cycle - 1 : 0)) & 1;
        if (L.cycle > 0) {  // full previous cycles end in e[1]
          if (tf.y == 2)
            batch_fold_item<R, W, K, true, TS, true>(J.G, J.mask, gc, J.x[xp] + co, e1 + co,
                J.x[xp ^ 1] + co, J.r + co, e0 + co, base, L.k, lane, w, edge);
          else
            batch_fold_item<R, W, K, false, TS, true>(J.G, J.mask, gc, J.x[xp] + co, e1 + co,
                J.x[xp ^ 1] + co, J.r + co, e0 + co, base, L.k, lane, w, edge);
        } else {
          if (tf.y == 2)
            batch_fold_item<R, W, K, true, TS, false>(J.G, J.mask, gc, J.x[xp] + co, nullptr,
                nullptr, J.r + co, e0 + co, base, L.k, lane, w, edge);
          else
            batch_fold_item<R, W, K, false, TS, false>(J.G, J.mask, gc, J.x[xp] + co, nullptr,
                nullptr, J.r + co, e0 + co, base, L.k, lane, w, edge);
        }
      } else if (L.type == 1) {
        const TS* ein = ((L.pos - 1) & 1) ? e1 : e0;
        TS* eout = (L.pos & 1) ? e1 : e0;
        const float* rc = J.r + co;
        if (tf.y == 2)
          batch_sweep_item<R, W, K, true, TS>(J.G, J.mask, rc, ein + co, eout + co, base, L.k, lane, w, edge);
        else
          batch_sweep_item<R, W, K, false, TS>(J.G, J.mask, rc, ein + co, eout + co, base, L.k, lane, w, edge);
      } else {
        const int xp = (J.parity + L.cycle - 1) & 1;
        const TS* elast = (((L.nlast - 1) & 1) ? e1 : e0) + co;
        refine_tile<TS>(J.G, J.mask, gc, J.x[xp] + co, elast, J.x[xp ^ 1] + co, nullptr,
                        ty * TH, tx * TW, TH, TW);
      }
    }
    // The next index is published before the barrier below, which then
    // serves both purposes: every thread reads it at the top of the next
    // iteration (all reads of the current one happened before this item's
    // first barrier), and every thread's writes precede the release.
    if (threadIdx.x == 0) s_idx = (long long)nxt;
    // Release: the CTA barrier orders every thread's writes before the
    // release reduction, which makes them visible before the count.  Thread
    // 32 issues it, so that thread 0's next acquire does not queue behind it.
    __syncthreads();
    if (threadIdx.x == 32)
      asm volatile("red.release.gpu.global.add.s32 [%0], 1;" : : "l"(Q.done + j) : "memory");
  }
}

struct BatchVariant {
  const char* name;
  int rows, warps, depth, tile_h, tile_w;
  const void* kernel[3];  // by precision: FP32, mixed FP16, mixed BF16
  void (*launch[3])(int grid, const BQueue& q, cudaStream_t st);
  void (*prepare[3])();   // shared-memory opt-in, once per device before the first launch
};

// Dynamic shared memory of a launch: the job records and tile entries when
// they fit in kBatchSmemTables bytes, else none (read from global memory).
constexpr size_t kBatchSmemTables = 160 * 1024;

size_t batch_smem_bytes(int njobs, int ntiles) {
  const size_t b = sizeof(BJobDev) * (size_t)njobs + sizeof(int2) * (size_t)ntiles;
  return b <= kBatchSmemTables ? b : 0;
}

template <int R, int W, int K, typename TS>
void launch_batch(int grid, const BQueue& q, cudaStream_t st) {
  const size_t dyn = q.smem_tables ? batch_smem_bytes(q.njobs, q.ntiles) : 0;
  batch_persistent_kernel<R, W, K, TS><<<grid, W * 32, dyn, st>>>(q);
}

template <int R, int W, int K, typename TS>
void prepare_batch() {
  FPIE_CUDA(cudaFuncSetAttribute(batch_persistent_kernel<R, W, K, TS>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kBatchSmemTables));
}

template <int R, int W, int K>
BatchVariant make_bv(const char* name) {
  return BatchVariant{name, R, W, K, W * R - 2 * K, 128 - 2 * K,
                      {(const void*)&batch_persistent_kernel<R, W, K, float>,
                       (const void*)&batch_persistent_kernel<R, W, K, __half>,
                       (const void*)&batch_persistent_kernel<R, W, K, __nv_bfloat16>},
                      {&launch_batch<R, W, K, float>, &launch_batch<R, W, K, __half>,
                       &launch_batch<R, W, K, __nv_bfloat16>},
                      {&prepare_batch<R, W, K, float>, &prepare_batch<R, W, K, __half>,
                       &prepare_batch<R, W, K, __nv_bfloat16>}};
}

static const std::vector<BatchVariant>& batch_variants() {
  static const std::vector<BatchVariant> v = {
      make_bv<16, 8, 16>("p16w8k16"),
      make_bv<8, 16, 16>("p8w16k16"),
      make_bv<16, 8, 8>("p16w8k8"),
  };
  return v;
}

// ---- host side ---------------------------------------------------------------------

struct BatchJob {
  int n = 0, m = 0;
  GridGeom G{};
  GridLaunch L{};
  std::vector<uint8_t> hmask;  // 0/1 crop mask, for tile lists
  // Active-tile lists per batch variant, built on first use (the mask of a
  // job never changes).
  std::vector<std::vector<int2>> tiles_of;
  std::vector<int> tiles_x_of;
  float* x[2] = {nullptr, nullptr};
  float* g = nullptr;
  uint8_t* mask = nullptr;
  uint8_t* img = nullptr;
  double* parts = nullptr;  // per-block partials: 6 doubles each (norms need 6)
  float* err = nullptr;
  double* norm = nullptr;   // [max|r| x3, sum|r| x3] of the last norms() call
  void* e[2] = {nullptr, nullptr};  // mixed forms only
  float* r = nullptr;               // mixed forms only
  int cur = 0;
  int sweeps_total = 0, sweeps_done = 0;
  bool live = false;
  size_t bytes = 0;
};

__global__ void batch_pack_kernel(GridGeom G, const int32_t* __restrict__ mk,
                                  const float* __restrict__ t, const float* __restrict__ gr,
                                  uint8_t* __restrict__ mask, float* __restrict__ x0,
                                  float* __restrict__ x1, float* __restrict__ g) {
  const long long total = (long long)G.n * G.m;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(idx / G.m), j = (int)(idx % G.m);
    const long long p = G.at(i, j);
    mask[p] = mk[idx] != 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      x0[c * G.plane + p] = t[idx * 3 + c];
      x1[c * G.plane + p] = t[idx * 3 + c];
      g[c * G.plane + p] = gr[idx * 3 + c];
    }
  }
}

struct Batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<BatchJob> jobs;
  size_t budget = 0, used = 0;
  int variant = 0;
  bool tuned = false, pinned = false;
  long long launches = 0;
  long long spin_limit = 1LL << 25;  // x ~128 ns sleeps: a few seconds at most
  int sms = 0;
  // Images-in adds copy on a second stream (see add_images).
  cudaStream_t xfer = nullptr;
  cudaEvent_t xfer_done = nullptr;
  // Asynchronous runs: each launch's error flag lands in a pinned slot that
  // wait() checks; kMaxPending launches may be in flight.
  static constexpr int kMaxPending = 64;
  int* h_errs = nullptr;
  int n_pending = 0;
  // Asynchronous norms: one pinned array, filled by one copy per call.
  double* h_norms = nullptr;
  int h_norms_cap = 0, norms_count = -1;
  cudaEvent_t norms_done = nullptr;

  explicit Batch(size_t budget_bytes) : budget(budget_bytes) {
    FPIE_CUDA(cudaGetDevice(&device));
    FPIE_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    FPIE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  }
  ~Batch() {
    for (auto& j : jobs) free_job(j);
    cudaStreamSynchronize(stream);
    if (xfer) {
      cudaStreamSynchronize(xfer);
      cudaStreamDestroy(xfer);
    }
    if (xfer_done) cudaEventDestroy(xfer_done);
    if (norms_done) cudaEventDestroy(norms_done);
    cudaFreeHost(h_errs);
    cudaFreeHost(h_norms);
    cudaStreamDestroy(stream);
  }

  // Job buffers come from the library's stream-ordered pool on the batch's
  // stream, so that removing a job (cudaFreeAsync) never waits for the
  // device: the memory returns to the pool once the work queued before the
  // removal -- e.g. an epoch still running -- is done.
  template <typename T>
  void alloc(T** p, size_t bytes) {
    void* q = nullptr;
    FPIE_CUDA(cudaMallocFromPoolAsync(&q, bytes, scratch_pool(), stream));
    *p = static_cast<T*>(q);
  }
  void release(void* p) {
    if (p) cudaFreeAsync(p, stream);
  }

  int precision = FPIE_FP32;

  static size_t job_bytes(int n, int m, int precision = FPIE_FP32) {
    const GridGeom G = make_geom(n, m);
    const GridLaunch L = grid_launch(G);
    const size_t mixed = precision == FPIE_FP32 ? 0 : (size_t)G.plane * 3 * (2 * 2 + 4);
    return mixed + (size_t)G.plane * (9 * sizeof(float) + 1) + (size_t)n * m * 3 +
           (size_t)L.nparts * 6 * sizeof(double) + 3 * sizeof(float) + 6 * sizeof(double) +
           7 * 256;
  }

  void free_job(BatchJob& j) {
    release(j.x[0]);
    release(j.x[1]);
    release(j.g);
    release(j.mask);
    release(j.img);
    release(j.parts);
    release(j.err);
    release(j.norm);
    release(j.e[0]);
    release(j.e[1]);
    release(j.r);
    j.e[0] = j.e[1] = nullptr;
    j.r = nullptr;
    j.x[0] = j.x[1] = j.g = nullptr;
    j.mask = j.img = nullptr;
    j.parts = nullptr;
    j.err = nullptr;
    j.norm = nullptr;
    if (j.live) used -= j.bytes;
    j.live = false;
  }

  // A new job slot of an n x m grid with zeroed device buffers (stream-
  // ordered on the batch's stream); the caller fills mask, x and grad.
  int new_job(int n, int m, int iterations) {
    FPIE_REQUIRE(n >= 1 && m >= 1, FPIE_ERR_ARG, "bad job size");
    FPIE_REQUIRE(iterations >= 0, FPIE_ERR_ARG, "negative sweep count");
    FPIE_REQUIRE((long long)n * m <= (1LL << 29), FPIE_ERR_ARG, "job too large");
    const size_t need = job_bytes(n, m, precision);
    FPIE_REQUIRE(used + need <= budget, FPIE_ERR_STATE,
                 "job needs " + std::to_string(need) + " bytes; HBM budget left is " +
                     std::to_string(budget - used));
    int id = -1;
    for (size_t k = 0; k < jobs.size(); ++k)
      if (!jobs[k].live) { id = (int)k; break; }
    if (id < 0) { jobs.emplace_back(); id = (int)jobs.size() - 1; }
    BatchJob& j = jobs[id];
    j = BatchJob{};
    j.n = n;
    j.m = m;
    j.G = make_geom(n, m);
    j.L = grid_launch(j.G);
    j.sweeps_total = iterations;
    j.sweeps_done = 0;
    const size_t pb = (size_t)j.G.plane * sizeof(float);
    try {
      alloc(&j.x[0], 3 * pb);
      alloc(&j.x[1], 3 * pb);
      alloc(&j.g, 3 * pb);
      alloc(&j.mask, (size_t)j.G.plane);
      alloc(&j.img, (size_t)n * m * 3);
      alloc(&j.parts, (size_t)j.L.nparts * 6 * sizeof(double));
      alloc(&j.err, 3 * sizeof(float));
      alloc(&j.norm, 6 * sizeof(double));
      if (precision != FPIE_FP32) {
        const size_t eb = (size_t)j.G.plane * 3 * 2, rb = (size_t)j.G.plane * 3 * sizeof(float);
        alloc(&j.e[0], eb);
        alloc(&j.e[1], eb);
        alloc(&j.r, rb);
        FPIE_CUDA(cudaMemsetAsync(j.e[0], 0, eb, stream));
        FPIE_CUDA(cudaMemsetAsync(j.e[1], 0, eb, stream));
        FPIE_CUDA(cudaMemsetAsync(j.r, 0, rb, stream));
      }
      FPIE_CUDA(cudaMemsetAsync(j.x[0], 0, 3 * pb, stream));
      FPIE_CUDA(cudaMemsetAsync(j.x[1], 0, 3 * pb, stream));
      FPIE_CUDA(cudaMemsetAsync(j.g, 0, 3 * pb, stream));
      FPIE_CUDA(cudaMemsetAsync(j.mask, 0, (size_t)j.G.plane, stream));
    } catch (...) {
      free_job(j);
      throw;
    }
    j.live = true;
    j.bytes = need;
    used += need;
    return id;
  }

  int add(int n, int m, const int32_t* hm, const float* ht, const float* hg, int iterations) {
    FPIE_REQUIRE(hm && ht && hg, FPIE_ERR_ARG, "bad job arrays");
    const int id = new_job(n, m, iterations);
    BatchJob& j = jobs[id];
    j.hmask.resize((size_t)n * m);
    for (size_t k = 0; k < j.hmask.size(); ++k) j.hmask[k] = hm[k] != 0;
    try {
      const size_t px = (size_t)n * m;
      AsyncScratch scratch(px * 28, stream);
      char* stage = scratch.bytes();
      FPIE_CUDA(cudaMemcpyAsync(stage, hm, px * 4, cudaMemcpyHostToDevice, stream));
      FPIE_CUDA(cudaMemcpyAsync(stage + px * 4, ht, px * 12, cudaMemcpyHostToDevice, stream));
      FPIE_CUDA(cudaMemcpyAsync(stage + px * 16, hg, px * 12, cudaMemcpyHostToDevice, stream));
      const int blocks = stride_blocks(px, 256, 16);
      batch_pack_kernel<<<blocks, 256, 0, stream>>>(
          j.G, reinterpret_cast<int32_t*>(stage), reinterpret_cast<float*>(stage + px * 4),
          reinterpret_cast<float*>(stage + px * 16), j.mask, j.x[0], j.x[1], j.g);
      FPIE_CUDA(cudaGetLastError());
      ++launches;
      FPIE_CUDA(cudaStreamSynchronize(stream));  // the caller may reuse its arrays
    } catch (...) {
      free_job(j);
      throw;
    }
    return id;
  }

  // A job from the three uint8 images, as GridProcessor.reset builds it
  // (fpie/process.py:321-386): the mask is thresholded and its frame
  // cleared on the host (a pass over mh x mw bytes that gives the crop, and
  // the tile lists need the crop mask on the host anyway); the crop's
  // gradient mixing and the planar layout are built on the device by the
  // GPU-side reset's kernel (prep.cu).  The images are copied on a second
  // stream, so the copies do not wait for an epoch running on the batch's
  // stream; the build kernel is queued on the batch's stream after them.
  // box = the crop on the target (row0, row1, col0, col1).
  int add_images(const uint8_t* src, int sh, int sw, const uint8_t* msk, int mh, int mw,
                 int mch, const uint8_t* tgt, int th, int tw, int s_row, int s_col, int t_row,
                 int t_col, int mode, int iterations, int* box) {
    FPIE_REQUIRE(src && msk && tgt, FPIE_ERR_ARG, "null input array");
    FPIE_REQUIRE(sh > 0 && sw > 0 && mh > 0 && mw > 0 && th > 0 && tw > 0, FPIE_ERR_ARG,
                 "empty image");
    FPIE_REQUIRE(mch == 1 || mch == 3, FPIE_ERR_ARG, "mask must have 1 or 3 channels");
    FPIE_REQUIRE(mode >= 0 && mode <= 2, FPIE_ERR_ARG,
                 "gradient mode must be 0 (src), 1 (avg), 2 (max)");
    std::vector<uint8_t> m01((size_t)mh * mw);
    int b0 = INT32_MAX, b1 = -1, b2 = INT32_MAX, b3 = -1;
    for (int i = 0; i < mh; ++i)
      for (int k = 0; k < mw; ++k) {
        const size_t p = (size_t)i * mw + k;
        bool on = mch == 3 ? (int)msk[p * 3] + msk[p * 3 + 1] + msk[p * 3 + 2] >= 384
                           : msk[p] >= 128;
        on = on && i > 0 && i < mh - 1 && k > 0 && k < mw - 1;
        m01[p] = on;
        if (on) {
          b0 = std::min(b0, i);
          b1 = std::max(b1, i);
          b2 = std::min(b2, k);
          b3 = std::max(b3, k);
        }
      }
    if (b1 < 0) throw Error{FPIE_ERR_ARG, "the mask selects no pixel (after clearing its 1-pixel frame)"};
    const int x0 = b0 - 1, x1 = b1 + 2, y0 = b2 - 1, y1 = b3 + 2;
    const bool fits = s_row + x0 >= 0 && s_col + y0 >= 0 && s_row + x1 <= sh && s_col + y1 <= sw &&
                      t_row + x0 >= 0 && t_col + y0 >= 0 && t_row + x1 <= th && t_col + y1 <= tw;
    if (!fits)
      throw Error{FPIE_ERR_ARG,
                  "the mask's crop at the given offsets leaves the source or target image"};
    const int n = x1 - x0, m = y1 - y0;
    const int id = new_job(n, m, iterations);
    BatchJob& j = jobs[id];
    j.hmask.resize((size_t)n * m);
    for (int i = 0; i < n; ++i)
      std::memcpy(&j.hmask[(size_t)i * m], &m01[(size_t)(x0 + i) * mw + y0], (size_t)m);
    try {
      if (!xfer) {
        FPIE_CUDA(cudaStreamCreateWithFlags(&xfer, cudaStreamNonBlocking));
        FPIE_CUDA(cudaEventCreateWithFlags(&xfer_done, cudaEventDisableTiming));
      }
      const size_t sb = (size_t)sh * sw * 3, tb = (size_t)th * tw * 3, mb = (size_t)mh * mw;
      auto al = [](size_t x) { return (x + 255) / 256 * 256; };
      char* stage = nullptr;
      FPIE_CUDA(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&stage), al(sb) + al(tb) + al(mb),
                                        scratch_pool(), xfer));
      FPIE_CUDA(cudaMemcpyAsync(stage, src, sb, cudaMemcpyHostToDevice, xfer));
      FPIE_CUDA(cudaMemcpyAsync(stage + al(sb), tgt, tb, cudaMemcpyHostToDevice, xfer));
      FPIE_CUDA(cudaMemcpyAsync(stage + al(sb) + al(tb), m01.data(), mb, cudaMemcpyHostToDevice,
                                xfer));
      FPIE_CUDA(cudaEventRecord(xfer_done, xfer));
      FPIE_CUDA(cudaStreamWaitEvent(stream, xfer_done, 0));
      const uint8_t* dsrc = reinterpret_cast<uint8_t*>(stage);
      const uint8_t* dtgt = reinterpret_cast<uint8_t*>(stage + al(sb));
      const uint8_t* dm01 = reinterpret_cast<uint8_t*>(stage + al(sb) + al(tb));
      PrepArgs a{j.G, dm01, mw, x0, y0, dsrc, sw, s_row + x0, s_col + y0, dtgt, tw, t_row + x0,
                 t_col + y0, mode};
      launch_prep_grid(a, j.mask, j.x[0], j.x[1], j.g, stream);
      FPIE_CUDA(cudaGetLastError());
      ++launches;
      FPIE_CUDA(cudaFreeAsync(stage, stream));  // after the build kernel
      // The copies read host memory (the caller's images and m01, which goes
      // out of scope here): wait for them -- only for them, the second
      // stream holds nothing else -- so every host buffer may be reused.
      FPIE_CUDA(cudaStreamSynchronize(xfer));
    } catch (...) {
      free_job(j);
      throw;
    }
    if (box) {
      box[0] = t_row + x0;
      box[1] = t_row + x1;
      box[2] = t_col + y0;
      box[3] = t_col + y1;
    }
    return id;
  }

  BatchJob& job(int id) {
    FPIE_REQUIRE(id >= 0 && id < (int)jobs.size() && jobs[id].live, FPIE_ERR_ARG,
                 "no such job " + std::to_string(id));
    return jobs[id];
  }

  // (tile index, flag) of the active tiles of a job for every variant's
  // tiling: a tile is active if a masked pixel lies in it, and fully masked
  // (flag 2) if every pixel of its region (tile + depth on each side) lies
  // in the crop and is masked.  Counted with one summed-area table of the
  // mask, so each tile costs four lookups instead of a scan of its region.
  static void tile_lists(BatchJob& j) {
    const int n = j.n, m = j.m;
    const size_t w = (size_t)m + 1;
    std::vector<int> S((size_t)(n + 1) * w, 0);
    for (int i = 0; i < n; ++i) {
      int row = 0;
      for (int k = 0; k < m; ++k) {
        row += j.hmask[(size_t)i * m + k] ? 1 : 0;
        S[(size_t)(i + 1) * w + k + 1] = S[(size_t)i * w + k + 1] + row;
      }
    }
    // Masked pixels in rows [r0, r1) x columns [c0, c1), clipped to the crop.
    auto count = [&](int r0, int r1, int c0, int c1) -> long long {
      r0 = std::max(r0, 0), c0 = std::max(c0, 0), r1 = std::min(r1, n), c1 = std::min(c1, m);
      if (r0 >= r1 || c0 >= c1) return 0;
      return (long long)S[(size_t)r1 * w + c1] - S[(size_t)r0 * w + c1] - S[(size_t)r1 * w + c0] +
             S[(size_t)r0 * w + c0];
    };
    const auto& vs = batch_variants();
    j.tiles_of.assign(vs.size(), {});
    j.tiles_x_of.assign(vs.size(), -1);
    for (size_t vi = 0; vi < vs.size(); ++vi) {
      const BatchVariant& v = vs[vi];
      const int tiles_x = (m + v.tile_w - 1) / v.tile_w;
      const int tiles_y = (n + v.tile_h - 1) / v.tile_h;
      std::vector<int2>& out = j.tiles_of[vi];
      for (int ty = 0; ty < tiles_y; ++ty)
        for (int tx = 0; tx < tiles_x; ++tx) {
          const int r0 = ty * v.tile_h, c0 = tx * v.tile_w;
          if (count(r0, r0 + v.tile_h, c0, c0 + v.tile_w) == 0) continue;
          const int R0 = r0 - v.depth, R1 = r0 + v.tile_h + v.depth;
          const int C0 = c0 - v.depth, C1 = c0 + v.tile_w + v.depth;
          const bool inside = R0 >= 0 && C0 >= 0 && R1 <= n && C1 <= m;
          const bool all = inside && count(R0, R1, C0, C1) == (long long)(R1 - R0) * (C1 - C0);
          out.push_back(make_int2(ty * tiles_x + tx, all ? 2 : 1));
        }
      j.tiles_x_of[vi] = tiles_x;
    }
  }

  // Kernels whose dynamic shared-memory limit was raised (per variant and
  // precision).
  bool prepared[8][3] = {};

  // Runs `sweeps[id]` more sweeps of the listed jobs in one persistent launch
  // of variant v; returns the device milliseconds (measured with events).
  float launch(const std::vector<int>& ids, const std::vector<int>& sw, int vi, bool time_it,
               bool async = false) {
    const BatchVariant& v = batch_variants()[vi];
    std::vector<BJobDev> dj;
    std::vector<int2> tiles;
    std::vector<int> levels;
    for (size_t k = 0; k < ids.size(); ++k) {
      BatchJob& j = jobs[ids[k]];
      if (j.tiles_of.size() != batch_variants().size()) tile_lists(j);
      const std::vector<int2>& tl = j.tiles_of[vi];
      const int tx = j.tiles_x_of[vi];
      BJobDev d;
      d.G = j.G;
      d.mask = j.mask;
      d.g = j.g;
      d.x[0] = j.x[0];
      d.x[1] = j.x[1];
      d.e[0] = j.e[0];
      d.e[1] = j.e[1];
      d.r = j.r;
      d.tiles_x = tx;
      d.ntiles = (int)tl.size();
      d.tile_off = (int)tiles.size();
      d.sweeps = sw[k];
      d.parity = j.cur;
      tiles.insert(tiles.end(), tl.begin(), tl.end());
      dj.push_back(d);
      const int lv = precision == FPIE_FP32 ? (sw[k] + v.depth - 1) / v.depth
                                            : (sw[k] > 0 ? mixed_levels(sw[k], v.depth) : 0);
      levels.push_back(d.ntiles > 0 ? lv : 0);
    }
    const int nj = (int)dj.size();
    std::vector<int> order(nj);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return levels[a] > levels[b]; });
    const int nlevels = nj ? levels[order[0]] : 0;
    std::vector<long long> ct(nj + 1, 0), lo(nlevels + 1, 0);
    std::vector<int> act(std::max(nlevels, 1), 0);
    for (int k = 0; k < nj; ++k) ct[k + 1] = ct[k] + 3LL * dj[order[k]].ntiles;
    for (int z = 0; z < nlevels; ++z) {
      int a = 0;
      while (a < nj && levels[order[a]] > z) ++a;
      act[z] = a;
      lo[z + 1] = lo[z] + ct[a];
    }
    float ms = 0.f;
    if (nlevels > 0 && lo[nlevels] > 0) {
      // One device block for the queue tables (freed after the launch).
      const size_t b_jobs = sizeof(BJobDev) * nj, b_order = sizeof(int) * nj,
                   b_ct = sizeof(long long) * (nj + 1), b_lo = sizeof(long long) * (nlevels + 1),
                   b_act = sizeof(int) * nlevels, b_tiles = sizeof(int2) * std::max<size_t>(tiles.size(), 1),
                   b_done = sizeof(int) * nj;
      auto al = [](size_t x) { return (x + 255) / 256 * 256; };
      const size_t bytes = al(b_jobs) + al(b_order) + al(b_ct) + al(b_lo) + al(b_act) +
                           al(b_tiles) + al(b_done) + 256;
      std::vector<char> host(bytes, 0);
      AsyncScratch tables(bytes, stream);
      char* dev = tables.bytes();
      size_t off = 0;
      auto put = [&](const void* src, size_t n) {
        if (n) std::memcpy(host.data() + off, src, n);
        const size_t o = off;
        off += al(n);
        return dev + o;
      };
      BQueue q;
      q.jobs = reinterpret_cast<const BJobDev*>(put(dj.data(), b_jobs));
      q.order = reinterpret_cast<const int*>(put(order.data(), b_order));
      q.ct = reinterpret_cast<const long long*>(put(ct.data(), b_ct));
      q.lo = reinterpret_cast<const long long*>(put(lo.data(), b_lo));
      q.act = reinterpret_cast<const int*>(put(act.data(), b_act));
      q.tiles = reinterpret_cast<const int2*>(put(tiles.data(), sizeof(int2) * tiles.size()));
      if (tiles.empty()) off += al(sizeof(int2));
      q.done = reinterpret_cast<int*>(dev + off);
      off += al(b_done);
      q.next = reinterpret_cast<unsigned long long*>(dev + off);
      q.error = reinterpret_cast<int*>(dev + off + 8);
      q.nlevels = nlevels;
      q.njobs = nj;
      q.ntiles = (int)tiles.size();
      const size_t dyn = batch_smem_bytes(nj, (int)tiles.size());
      q.smem_tables = dyn > 0 ? 1 : 0;
      q.spin_limit = spin_limit;
      FPIE_CUDA(cudaMemcpyAsync(dev, host.data(), bytes, cudaMemcpyHostToDevice, stream));
      FPIE_REQUIRE(vi >= 0 && vi < 8 && precision >= 0 && precision < 3, FPIE_ERR_STATE,
                   "batch kernel variant out of range");
      if (!prepared[vi][precision]) {
        v.prepare[precision]();
        prepared[vi][precision] = true;
      }
      int occ = 0;
      FPIE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, v.kernel[precision],
                                                              v.warps * 32, dyn));
      const int grid = std::max(1, occ) * sms;
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      if (time_it) {
        FPIE_CUDA(cudaEventCreate(&e0));
        FPIE_CUDA(cudaEventCreate(&e1));
        FPIE_CUDA(cudaEventRecord(e0, stream));
      }
      v.launch[precision](grid, q, stream);
      FPIE_CUDA(cudaGetLastError());
      ++launches;
      if (time_it) FPIE_CUDA(cudaEventRecord(e1, stream));
      if (async && !time_it) {
        // The flag is read by wait(); the queue tables are freed after the
        // copy in stream order.  The jobs' bookkeeping below still applies.
        if (!h_errs) FPIE_CUDA(cudaMallocHost(&h_errs, kMaxPending * sizeof(int)));
        if (n_pending == kMaxPending) wait();
        h_errs[n_pending] = 0;
        FPIE_CUDA(cudaMemcpyAsync(&h_errs[n_pending], q.error, sizeof(int),
                                  cudaMemcpyDeviceToHost, stream));
        ++n_pending;
      } else {
        int herr = 0;
        FPIE_CUDA(cudaMemcpyAsync(&herr, q.error, sizeof(int), cudaMemcpyDeviceToHost, stream));
        FPIE_CUDA(cudaStreamSynchronize(stream));
        if (time_it) {
          FPIE_CUDA(cudaEventElapsedTime(&ms, e0, e1));
          cudaEventDestroy(e0);
          cudaEventDestroy(e1);
        }
        FPIE_REQUIRE(herr == 0, FPIE_ERR_TIMEOUT,
                     "batch kernel: a dependency wait exceeded its spin limit");
      }
    }
    for (size_t k = 0; k < ids.size(); ++k) {
      BatchJob& j = jobs[ids[k]];
      if (levels[k] > 0) {
        // FP32: one buffer flip per level; mixed: one per fold level.
        const int flips = precision == FPIE_FP32 ? levels[k] : (sw[k] + 63) / 64;
        if (flips & 1) j.cur ^= 1;
      }
      j.sweeps_done += sw[k];
    }
    return ms;
  }

  std::vector<int> live_ids() const {
    std::vector<int> ids;
    for (size_t k = 0; k < jobs.size(); ++k)
      if (jobs[k].live) ids.push_back((int)k);
    return ids;
  }

  // Advances every live job by min(limit, its remaining sweeps); limit < 0
  // means "to completion".  Tunes the kernel on the first call with enough
  // work (each candidate runs 64 real sweeps of every job).
  void run(int limit, bool async = false) {
    std::vector<int> ids = live_ids();
    auto remaining = [&](int id) {
      const int rem = jobs[id].sweeps_total - jobs[id].sweeps_done;
      return limit < 0 ? rem : std::min(rem, limit);
    };
    int budget_sweeps = limit;
    if (!tuned && !pinned) {
      const int ncand = (int)batch_variants().size();
      int minrem = 1 << 30;
      for (int id : ids) minrem = std::min(minrem, remaining(id));
      if (!ids.empty() && minrem >= 64 * (ncand + 1)) {
        int best = 0;
        float best_ms = 1e30f;
        for (int v = 0; v < ncand; ++v) {
          std::vector<int> sw(ids.size(), 64);
          const float ms = launch(ids, sw, v, true);
          if (ms < best_ms) { best_ms = ms; best = v; }
        }
        variant = best;
        tuned = true;
        if (budget_sweeps >= 0) budget_sweeps -= 64 * ncand;
      }
    }
    std::vector<int> sw;
    std::vector<int> run_ids;
    for (int id : ids) {
      int rem = jobs[id].sweeps_total - jobs[id].sweeps_done;
      if (budget_sweeps >= 0) rem = std::min(rem, std::max(0, budget_sweeps));
      if (rem > 0) { run_ids.push_back(id); sw.push_back(rem); }
    }
    if (!run_ids.empty()) launch(run_ids, sw, variant, false, async);
  }

  // Waits for everything queued on the batch's stream and checks the error
  // flags of the asynchronous runs.
  void wait() {
    FPIE_CUDA(cudaStreamSynchronize(stream));
    bool timed_out = false;
    for (int k = 0; k < n_pending; ++k) timed_out = timed_out || h_errs[k] != 0;
    n_pending = 0;
    FPIE_REQUIRE(!timed_out, FPIE_ERR_TIMEOUT,
                 "batch kernel: a dependency wait exceeded its spin limit");
  }

  // Queues the FP64 residual norms of the listed jobs' current states (one
  // refine launch + one reduction per job) and one copy of all of them into
  // a pinned array; norms_wait() waits for that copy only.
  void norms_async(const int* ids, int count) {
    FPIE_REQUIRE((ids || count == 0) && count >= 0, FPIE_ERR_ARG, "bad arguments");
    if (count > h_norms_cap) {
      if (h_norms) {
        if (norms_done) FPIE_CUDA(cudaEventSynchronize(norms_done));
        cudaFreeHost(h_norms);
        h_norms = nullptr;
      }
      FPIE_CUDA(cudaMallocHost(&h_norms, 6 * sizeof(double) * (size_t)count));
      h_norms_cap = count;
    }
    if (!norms_done) FPIE_CUDA(cudaEventCreateWithFlags(&norms_done, cudaEventDisableTiming));
    if (count > 0) {
      AsyncScratch dn(6 * sizeof(double) * (size_t)count, stream);
      double* d = reinterpret_cast<double*>(dn.bytes());
      for (int k = 0; k < count; ++k) {
        BatchJob& j = job(ids[k]);
        launch_refine(FPIE_FP32, j.L.sweep_grid, j.L.sweep_block, j.G, j.mask, j.g, j.x[j.cur],
                      nullptr, nullptr, nullptr, j.parts, stream);
        launch_norms_finalize(j.parts, j.L.nparts, d + 6 * (size_t)k, stream);
        FPIE_CUDA(cudaGetLastError());
        launches += 2;
      }
      FPIE_CUDA(cudaMemcpyAsync(h_norms, d, 6 * sizeof(double) * (size_t)count,
                                cudaMemcpyDeviceToHost, stream));
    }
    FPIE_CUDA(cudaEventRecord(norms_done, stream));
    norms_count = count;
  }

  void norms_wait(double* out) {
    FPIE_REQUIRE(norms_count >= 0, FPIE_ERR_STATE, "no norms queued");
    FPIE_REQUIRE(out != nullptr || norms_count == 0, FPIE_ERR_ARG, "null output array");
    FPIE_CUDA(cudaEventSynchronize(norms_done));
    if (norms_count > 0) std::memcpy(out, h_norms, 6 * sizeof(double) * (size_t)norms_count);
    norms_count = -1;
  }

  // FP64 residual norms of the listed jobs' current states (one refine
  // launch + one reduction per job), copied to out[6 * k ...].
  void norms(const int* ids, int count, double* out) {
    FPIE_REQUIRE(ids && out && count >= 0, FPIE_ERR_ARG, "bad arguments");
    wait();
    std::vector<double> h(6 * (size_t)std::max(count, 1));
    for (int k = 0; k < count; ++k) {
      BatchJob& j = job(ids[k]);
      launch_refine(FPIE_FP32, j.L.sweep_grid, j.L.sweep_block, j.G, j.mask, j.g, j.x[j.cur],
                    nullptr, nullptr, nullptr, j.parts, stream);
      launch_norms_finalize(j.parts, j.L.nparts, j.norm, stream);
      FPIE_CUDA(cudaGetLastError());
      launches += 2;
      FPIE_CUDA(cudaMemcpyAsync(h.data() + 6 * (size_t)k, j.norm, 6 * sizeof(double),
                                cudaMemcpyDeviceToHost, stream));
    }
    FPIE_CUDA(cudaStreamSynchronize(stream));
    std::memcpy(out, h.data(), 6 * sizeof(double) * (size_t)count);
  }

  void finish(int id) {
    BatchJob& j = job(id);
    launch_grid_finish(j.L, j.G, j.mask, j.g, j.x[j.cur], j.img, j.parts, stream);
    launch_finalize(j.parts, j.L.nparts, j.err, stream);
    FPIE_CUDA(cudaGetLastError());
    launches += 2;
  }

  void result(int id, uint8_t* img, float* err) {
    FPIE_REQUIRE(img && err, FPIE_ERR_ARG, "null output array");
    if (n_pending) wait();
    BatchJob& j = job(id);
    finish(id);
    FPIE_CUDA(cudaMemcpyAsync(img, j.img, (size_t)j.n * j.m * 3, cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaMemcpyAsync(err, j.err, 3 * sizeof(float), cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
  }

  void state(int id, float* out) {
    FPIE_REQUIRE(out, FPIE_ERR_ARG, "null output array");
    if (n_pending) wait();
    BatchJob& j = job(id);
    const size_t plane_bytes = (size_t)j.G.plane * sizeof(float);
    std::vector<float> h(3 * (size_t)j.G.plane);
    FPIE_CUDA(cudaMemcpyAsync(h.data(), j.x[j.cur], 3 * plane_bytes, cudaMemcpyDeviceToHost, stream));
    FPIE_CUDA(cudaStreamSynchronize(stream));
    for (int i = 0; i < j.n; ++i)
      for (int k = 0; k < j.m; ++k)
        for (int c = 0; c < 3; ++c)
          out[((size_t)i * j.m + k) * 3 + c] = h[(size_t)c * j.G.plane + j.G.at(i, k)];
  }
};

}  // namespace fpie

using namespace fpie;

struct fpie_batch;

extern "C" {

int fpie_batch_create(double budget_bytes, fpie_batch** out) {
  return guarded([&] {
    FPIE_REQUIRE(out != nullptr, FPIE_ERR_ARG, "null output pointer");
    FPIE_REQUIRE(budget_bytes > 0, FPIE_ERR_ARG, "budget must be positive");
    *out = reinterpret_cast<fpie_batch*>(new Batch((size_t)budget_bytes));
  });
}

int fpie_batch_destroy(fpie_batch* b) {
  return guarded([&] {
    if (b) delete reinterpret_cast<Batch*>(b);
  });
}

static Batch* batch_of(fpie_batch* b) {
  FPIE_REQUIRE(b != nullptr, FPIE_ERR_ARG, "null batch handle");
  Batch* h = reinterpret_cast<Batch*>(b);
  FPIE_CUDA(cudaSetDevice(h->device));
  return h;
}

int fpie_batch_add(fpie_batch* b, int n, int m, const int32_t* mask, const float* tgt,
                   const float* grad, int iterations, int* job_id) {
  return guarded([&] {
    const int id = batch_of(b)->add(n, m, mask, tgt, grad, iterations);
    if (job_id) *job_id = id;
  });
}

int fpie_batch_job_bytes(int n, int m, double* bytes) {
  return guarded([&] {
    FPIE_REQUIRE(bytes && n >= 1 && m >= 1, FPIE_ERR_ARG, "bad arguments");
    *bytes = (double)Batch::job_bytes(n, m);
  });
}

int fpie_batch_set_precision(fpie_batch* b, int precision) {
  return guarded([&] {
    Batch* h = batch_of(b);
    FPIE_REQUIRE(precision == FPIE_FP32 || precision == FPIE_MIXED_FP16 ||
                     precision == FPIE_MIXED_BF16, FPIE_ERR_ARG, "unknown precision");
    FPIE_REQUIRE(h->live_ids().empty(), FPIE_ERR_STATE,
                 "set the precision before adding jobs");
    h->precision = precision;
  });
}

int fpie_batch_job_bytes_for(fpie_batch* b, int n, int m, double* bytes) {
  return guarded([&] {
    FPIE_REQUIRE(bytes && n >= 1 && m >= 1, FPIE_ERR_ARG, "bad arguments");
    *bytes = (double)Batch::job_bytes(n, m, batch_of(b)->precision);
  });
}

int fpie_batch_run(fpie_batch* b, int max_sweeps) {
  return guarded([&] { batch_of(b)->run(max_sweeps); });
}

int fpie_batch_run_async(fpie_batch* b, int max_sweeps) {
  return guarded([&] { batch_of(b)->run(max_sweeps, true); });
}

int fpie_batch_wait(fpie_batch* b) {
  return guarded([&] { batch_of(b)->wait(); });
}

int fpie_batch_norms_async(fpie_batch* b, const int* jobs, int count) {
  return guarded([&] { batch_of(b)->norms_async(jobs, count); });
}

int fpie_batch_norms_wait(fpie_batch* b, double* out) {
  return guarded([&] { batch_of(b)->norms_wait(out); });
}

int fpie_batch_add_images(fpie_batch* b, const uint8_t* src, int src_h, int src_w,
                          const uint8_t* mask, int mask_h, int mask_w, int mask_channels,
                          const uint8_t* tgt, int tgt_h, int tgt_w, int src_row, int src_col,
                          int tgt_row, int tgt_col, int gradient, int iterations, int* job_id,
                          int* box) {
  return guarded([&] {
    const int id = batch_of(b)->add_images(src, src_h, src_w, mask, mask_h, mask_w,
                                           mask_channels, tgt, tgt_h, tgt_w, src_row, src_col,
                                           tgt_row, tgt_col, gradient, iterations, box);
    if (job_id) *job_id = id;
  });
}

int fpie_batch_progress(fpie_batch* b, int job, int* done, int* total) {
  return guarded([&] {
    BatchJob& j = batch_of(b)->job(job);
    if (done) *done = j.sweeps_done;
    if (total) *total = j.sweeps_total;
  });
}

int fpie_batch_result(fpie_batch* b, int job, uint8_t* img, float* err) {
  return guarded([&] { batch_of(b)->result(job, img, err); });
}

int fpie_batch_state(fpie_batch* b, int job, float* out) {
  return guarded([&] { batch_of(b)->state(job, out); });
}

int fpie_batch_norms(fpie_batch* b, const int* jobs, int count, double* out) {
  return guarded([&] { batch_of(b)->norms(jobs, count, out); });
}

int fpie_batch_remove(fpie_batch* b, int job) {
  return guarded([&] {
    Batch* h = batch_of(b);
    BatchJob& j = h->job(job);
    h->free_job(j);  // stream-ordered: after any work queued for the job
  });
}

int fpie_batch_memory(fpie_batch* b, double* used, double* budget) {
  return guarded([&] {
    Batch* h = batch_of(b);
    if (used) *used = (double)h->used;
    if (budget) *budget = (double)h->budget;
  });
}

int fpie_batch_set_kernel(fpie_batch* b, const char* name) {
  return guarded([&] {
    Batch* h = batch_of(b);
    FPIE_REQUIRE(name != nullptr, FPIE_ERR_ARG, "null kernel name");
    if (std::string(name) == "auto") {
      h->pinned = false;
      h->tuned = false;
      return;
    }
    for (size_t k = 0; k < batch_variants().size(); ++k)
      if (std::string(name) == batch_variants()[k].name) {
        h->variant = (int)k;
        h->pinned = true;
        return;
      }
    throw Error{FPIE_ERR_ARG, std::string("unknown batch kernel '") + name + "'"};
  });
}

int fpie_batch_kernel(fpie_batch* b, char* buf, int len) {
  return guarded([&] {
    FPIE_REQUIRE(buf && len > 0, FPIE_ERR_ARG, "null or empty buffer");
    std::snprintf(buf, (size_t)len, "%s", batch_variants()[batch_of(b)->variant].name);
  });
}

int fpie_batch_set_spin_limit(fpie_batch* b, long long spins) {
  return guarded([&] {
    FPIE_REQUIRE(spins > 0, FPIE_ERR_ARG, "spin limit must be positive");
    batch_of(b)->spin_limit = spins;
  });
}

int fpie_batch_launch_count(fpie_batch* b, long long* count) {
  return guarded([&] {
    FPIE_REQUIRE(count, FPIE_ERR_ARG, "null pointer");
    *count = batch_of(b)->launches;
  });
}

}  // extern "C"
