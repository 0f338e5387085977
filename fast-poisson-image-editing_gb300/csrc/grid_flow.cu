// Dependency-flow grid sweep ("p16w8k16d", "p16w8k12d"): a whole step in
// one launch.
//
// The sweeps are cut into levels of up to K = 16 (the packed variant
// p16w8k16's temporal depth: 96x96 tiles in 128x128 register-resident
// regions, same arithmetic, bit-identical results) or K = 12 (104x104
// tiles in the same regions).  A work item is one
// (level, active tile, channel); items are numbered level-major and CTA b
// of a cooperative launch takes items b, b + gridDim.x, ...  Item
// (z, tile, c) reads buffer (p + z) & 1 over its region and writes the tile
// interior to buffer (p + z + 1) & 1.  It may start once every active tile
// of its 3x3 neighbourhood (same channel, itself included) has finished
// level z - 1, which covers both hazards on the ping-pong buffers:
//   - read after write: the region (tile + K-pixel apron) lies inside the
//     neighbourhood, whose level z - 1 outputs are then complete;
//   - write after read: the buffer being written was read at level z - 1
//     only by items of the neighbourhood, which are then finished.
// Inactive tiles (no masked pixel) never change and hold the same values
// in both buffers, so nobody waits for them.
//
// A CTA never waits for a later-numbered item, and all CTAs of a
// cooperative launch are co-resident, so the waits always end; they are
// bounded anyway (the solver's spin limit): past it the CTA records an
// error, every CTA stops at its next wait, and the host reports
// FPIE_ERR_TIMEOUT.
//
// What this buys over one launch per 16 sweeps: no launch gaps, and no
// wave tail -- when a level has, say, 243 items on 152 SMs, CTAs that are
// done with their level-z items go on to level z + 1 items whose
// neighbourhoods are ready instead of idling until the whole level ends.
//
// The same launch runs the mixed forms (TS = __half / __nv_bfloat16: the
// refinement cycles' level schedule) and, for the EquSolver's red-black
// order on its grid placement ("rb16w8k8d"), levels of 8 red-black sweeps on
// the same tiles and apron (16 half-steps, each shrinking the valid region
// by one cell).
#include <algorithm>
#include <atomic>
#include <type_traits>

#include "common.cuh"

#include "grid_flow.cuh"
#include "grid_tbp.cuh"
#include "mixed_levels.cuh"

namespace fpie {

namespace {

constexpr int kR = 16, kW = 8;
// Temporal depth K (sweeps per level, and the apron): tiles of
// (8 * 16 - 2K) x (128 - 2K) in 128 x 128 regions.  K = 16 (96 x 96 tiles)
// runs every form; K = 12 (104 x 104 tiles, FP32 Jacobi only) covers some
// grids with fewer tiles -- an 802-pixel side takes 8 of them instead of 9,
// which cuts the region work per sweep by a fifth.
constexpr int kK = 16;
template <int K>
struct FlowTile {
  static_assert(K % 4 == 0 && K <= kPad, "the apron must keep float4 columns aligned");
  static constexpr int H = kW * kR - 2 * K;
  static constexpr int W = 128 - 2 * K;
};

// Per active tile: {tile, flag, nb[0..8]} with nb = 3 x (active-list index)
// of each tile of the 3x3 neighbourhood (row-major, itself at 4), -1 where
// there is no active tile; padded to 12 ints (three int4 loads).  flag: 2 =
// region fully masked (no selects); else the region's pinned-boundary
// sweep body for FP32 Jacobi sweeps (kBody*; the mixed and red-black forms
// take their select path for any flag but 2).
struct FlowRec {
  int tile, flag, nb[9], pad;
};
static_assert(sizeof(FlowRec) == 48, "three int4");

// Sweep bodies of regions holding unmasked pixels (FlowRec.flag), chosen
// once per mask by flow_body_kernel from where the region's pinned pixels
// lie: every one in the same column group of the lanes (a vertical edge),
// in at most two pair rows of every warp (horizontal edges), or anywhere
// (kBodyAll: the select on every unmasked pixel, which measured faster
// than selecting the pinned ones in every group and storing around the
// free ones).
constexpr int kBodyAll = 3, kBodyRows = 4, kBodyCol0 = 5;  // kBodyCol0 + j: column group j

struct FlowArgs {
  GridGeom G;
  const uint8_t* mask;
  const uint8_t* code;   // FP32 Jacobi: per pixel bit 0 = masked, bit 1 = pinned
  const float* g;
  float* x[2];
  void* e[2];            // mixed forms: the correction planes (FP16 / BF16)
  float* r;              // mixed forms: the FP32 residual planes
  const int* list;       // active tiles in tile order; list[-1] = their count
  const FlowRec* rec;    // per active tile
  int* done;             // per (active tile, channel): levels finished
  int* error;
  int tiles_x, sweeps, parity;
  long long spin_limit;
  int red_black;         // red-black sweeps: kK / 2 per level, same tiles and apron
  int smem_recs;         // the records are copied to shared memory first
};

// Records of at most this many active tiles (30 KB; with the 16 KB of edge
// rows the kernel stays under the default 48 KB of shared memory, so L1
// keeps its size) are copied to shared memory at the start of a launch.
// Thread 0 reads the next item's record after the current item and only
// then can load its neighbourhood counters: from L2 that is two round trips
// before the release barrier, which holds back this item's release.
constexpr int kFlowRecsSmem = 640;

__device__ __forceinline__ FlowRec load_rec(const FlowRec* r) {
  const int4* q = reinterpret_cast<const int4*>(r);
  const int4 a = q[0], b = q[1], d = q[2];
  return FlowRec{a.x, a.y, {a.z, a.w, b.x, b.y, b.z, b.w, d.x, d.y, d.z}, d.w};
}

// The nine neighbourhood counters of channel c (INT_MAX where none).
__device__ __forceinline__ void load_counters(const FlowArgs& A, const FlowRec& R, int c,
                                              int (&v)[9]) {
#pragma unroll
  for (int k = 0; k < 9; ++k)
    v[k] = R.nb[k] >= 0 ? *(const volatile int*)(A.done + R.nb[k] + c) : 0x7fffffff;
}

// Publishes a finished item: a release reduction on its counter.
__device__ __forceinline__ void release_add(int* counter) {
  asm volatile("red.release.gpu.global.add.s32 [%0], 1;" : : "l"(counter) : "memory");
}

__device__ __forceinline__ bool counters_reach(const int (&v)[9], int level) {
  bool ok = true;
#pragma unroll
  for (int k = 0; k < 9; ++k) ok = ok && v[k] >= level;
  return ok;
}

// Thread 0: waits until the counters in v (loaded earlier, possibly stale --
// counters only grow) all reach `level`, reloading them together each round.
// A round is one L2 round trip: the error flag is loaded with the counters,
// not before them, and the first rounds poll again at once (a neighbour
// about to finish is the common case); later rounds back off 64 ns.
// False if the wait gave up or another CTA did.
__device__ __forceinline__ bool wait_counters(const FlowArgs& A, const FlowRec& R, int c,
                                              int level, int (&v)[9]) {
  for (long long spins = 0; !counters_reach(v, level); ++spins) {
    if (spins >= A.spin_limit) {
      atomicExch(A.error, 1);
      return false;
    }
    if (spins >= 8) __nanosleep(64);
    const int err = *(volatile int*)A.error;
    load_counters(A, R, c, v);
    if (err) return false;
  }
  return true;
}

// One FP32 Jacobi item of a fully masked region (FULL: no selects) or of a
// region whose unmasked pixels all keep their values by a select (!FULL).
// Items are out of line: inlined into the item loop, the compiler's
// register assignment needs several times the register moves per sweep of
// the same code in the launch-per-tile kernel (measured by instruction
// counters).
template <int K, bool FULL>
__device__ __noinline__ void flow_item(const FlowArgs& A, int tile, int c, int z,
                                       float4 (&edge)[2][2][kW][32], int lane, int w) {
  const GridGeom& G = A.G;
  const int ty = tile / A.tiles_x, tx = tile - ty * A.tiles_x;
  const long long base = G.at(ty * FlowTile<K>::H - K + w * kR, tx * FlowTile<K>::W - K + 4 * lane);
  const long long co = c * G.plane;
  const int pin = (A.parity + z) & 1;
  const int ks = min(K, A.sweeps - z * K);
  // CG: the state is read through L2, since other CTAs wrote it during
  // this launch.
  tbp_body<kR, kW, K, FULL, float, false, true>(G, A.mask, A.g + co, A.x[pin] + co,
                                                A.x[pin ^ 1] + co, base, ks, lane, w, edge);
}

// One FP32 Jacobi item of a region whose pinned pixels lie in one column
// group or in few pair rows, by its body (FlowRec.flag): the pinned-boundary
// sweeps (code plane, free pixels not stored).  The five bodies share one
// function (out-of-line bodies of their own measured slower); the select on
// every unmasked pixel keeps its own (flow_item), which measured faster than
// a sixth case here.
template <int K>
__device__ __noinline__ void flow_pin_item(const FlowArgs& A, int flag, int tile, int c, int z,
                                           float4 (&edge)[2][2][kW][32], int lane, int w) {
  const GridGeom& G = A.G;
  const int ty = tile / A.tiles_x, tx = tile - ty * A.tiles_x;
  const long long base = G.at(ty * FlowTile<K>::H - K + w * kR, tx * FlowTile<K>::W - K + 4 * lane);
  const long long co = c * G.plane;
  const int pin = (A.parity + z) & 1;
  const int ks = min(K, A.sweeps - z * K);
  const float* gc = A.g + co;
  const float* xi = A.x[pin] + co;
  float* xo = A.x[pin ^ 1] + co;
  switch (flag) {
    case kBodyRows:
      tbp_body<kR, kW, K, false, float, false, true, false, false, kRowSel>(G, A.code, gc, xi, xo,
                                                                         base, ks, lane, w, edge);
      break;
    case kBodyCol0:
      tbp_body<kR, kW, K, false, float, false, true, false, false, 1>(G, A.code, gc, xi, xo, base,
                                                                   ks, lane, w, edge);
      break;
    case kBodyCol0 + 1:
      tbp_body<kR, kW, K, false, float, false, true, false, false, 2>(G, A.code, gc, xi, xo, base,
                                                                   ks, lane, w, edge);
      break;
    case kBodyCol0 + 2:
      tbp_body<kR, kW, K, false, float, false, true, false, false, 4>(G, A.code, gc, xi, xo, base,
                                                                   ks, lane, w, edge);
      break;
    default:
      tbp_body<kR, kW, K, false, float, false, true, false, false, 8>(G, A.code, gc, xi, xo, base,
                                                                   ks, lane, w, edge);
      break;
  }
}

// The FP32 Jacobi item of a region with body `flag` (FlowRec).  PINB: the
// pinned-boundary bodies where the flag names one; else (and in kernels
// built without them, whose smaller code runs curved masks ~6% faster) the
// select on every unmasked pixel.
template <int K, bool PINB>
__device__ __forceinline__ void flow_jacobi_item(const FlowArgs& A, int flag, int tile, int c,
                                                 int z, float4 (&edge)[2][2][kW][32], int lane,
                                                 int w) {
  if (flag == 2)
    flow_item<K, true>(A, tile, c, z, edge, lane, w);
  else if (!PINB || flag == kBodyAll)
    flow_item<K, false>(A, tile, c, z, edge, lane, w);
  else if constexpr (PINB)
    flow_pin_item<K>(A, flag, tile, c, z, edge, lane, w);
}

// One item of the red-black order (the EquSolver's grid placement): kK / 2
// red-black sweeps on the same region, apron kK.  Out of line like flow_item.
template <bool FULL>
__device__ __noinline__ void flow_rb_item(const FlowArgs& A, int tile, int c, int z,
                                          float4 (&edge)[2][2][kW][32], int lane, int w) {
  const GridGeom& G = A.G;
  const int ty = tile / A.tiles_x, tx = tile - ty * A.tiles_x;
  const long long base = G.at(ty * FlowTile<kK>::H - kK + w * kR, tx * FlowTile<kK>::W - kK + 4 * lane);
  const long long co = c * G.plane;
  const int pin = (A.parity + z) & 1;
  const int ks = min(kK / 2, A.sweeps - z * (kK / 2));
  tbp_body<kR, kW, kK, FULL, float, false, true, false, true>(
      G, A.mask, A.g + co, A.x[pin] + co, A.x[pin ^ 1] + co, base, ks, lane, w, edge);
}

// The mixed forms' items at level z (the batched kernel's level schedule,
// mixed_level: fold + first inner sweeps, inner sweeps on the correction,
// final fold), one out-of-line function per level type so that each gets
// the register assignment of its own body (one function holding all three
// needed 255 registers and spilled).
template <bool FULL, typename TS>
__device__ __noinline__ void flow_fold_item(const FlowArgs& A, int tile, int c, int cycle, int k,
                                            float4 (&edge)[2][2][kW][32], int lane, int w) {
  const GridGeom& G = A.G;
  const int ty = tile / A.tiles_x, tx = tile - ty * A.tiles_x;
  const long long base = G.at(ty * FlowTile<kK>::H - kK + w * kR, tx * FlowTile<kK>::W - kK + 4 * lane);
  const long long co = c * G.plane;
  const float* gc = A.g + co;
  TS* e0 = static_cast<TS*>(A.e[0]);
  TS* e1 = static_cast<TS*>(A.e[1]);
  // x parity before this cycle's fold: one flip per earlier fold.
  const int xp = (A.parity + (cycle > 0 ? cycle - 1 : 0)) & 1;
  if (cycle > 0)  // full previous cycles end in e[1]
    tbp_fold_body<kR, kW, kK, FULL, TS, true, true>(G, A.mask, gc, A.x[xp] + co, e1 + co,
                                                    A.x[xp ^ 1] + co, A.r + co, e0 + co, base, k,
                                                    lane, w, edge);
  else
    tbp_fold_body<kR, kW, kK, FULL, TS, false, true>(G, A.mask, gc, A.x[xp] + co, nullptr,
                                                     nullptr, A.r + co, e0 + co, base, k, lane,
                                                     w, edge);
}

template <bool FULL, typename TS>
__device__ __noinline__ void flow_inner_item(const FlowArgs& A, int tile, int c, int pos, int k,
                                             float4 (&edge)[2][2][kW][32], int lane, int w) {
  const GridGeom& G = A.G;
  const int ty = tile / A.tiles_x, tx = tile - ty * A.tiles_x;
  const long long base = G.at(ty * FlowTile<kK>::H - kK + w * kR, tx * FlowTile<kK>::W - kK + 4 * lane);
  const long long co = c * G.plane;
  TS* e0 = static_cast<TS*>(A.e[0]);
  TS* e1 = static_cast<TS*>(A.e[1]);
  const TS* ein = ((pos - 1) & 1) ? e1 : e0;
  TS* eout = (pos & 1) ? e1 : e0;
  tbp_body<kR, kW, kK, FULL, TS, false, true>(G, A.mask, A.r + co, ein + co, eout + co, base, k,
                                              lane, w, edge);
}

template <typename TS>
__device__ __noinline__ void flow_flush_item(const FlowArgs& A, int tile, int c, int cycle,
                                             int nlast) {
  const GridGeom& G = A.G;
  const int ty = tile / A.tiles_x, tx = tile - ty * A.tiles_x;
  const long long co = c * G.plane;
  TS* e0 = static_cast<TS*>(A.e[0]);
  TS* e1 = static_cast<TS*>(A.e[1]);
  const int xp = (A.parity + cycle - 1) & 1;
  const TS* elast = (((nlast - 1) & 1) ? e1 : e0) + co;
  refine_tile<TS>(G, A.mask, A.g + co, A.x[xp] + co, elast, A.x[xp ^ 1] + co, nullptr, ty * FlowTile<kK>::H,
                  tx * FlowTile<kK>::W, FlowTile<kK>::H, FlowTile<kK>::W);
}

// Thread 0 keeps the next item's record and counters, loaded right after
// the current item's sweeps so that their latency overlaps the release
// fence and barrier; the other threads get tile and flag through shared
// memory.
// TS = float: the FP32 sweeps; __half / __nv_bfloat16: the mixed forms.
// K: the temporal depth (the mixed and red-black forms run at kK only).
template <typename TS, int K, bool PINB = false>
__global__ void __launch_bounds__(kW * 32, 1) grid_flow_kernel(FlowArgs A) {
  constexpr bool MIXED = !std::is_same<TS, float>::value;
  static_assert(K == kK || !MIXED, "the mixed forms' cycles are 64 sweeps of kK-sweep levels");
  __shared__ float4 edge[2][2][kW][32];
  __shared__ int s_stop, s_tile, s_flag;
  extern __shared__ __align__(16) unsigned char flow_dyn[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int per = 3 * A.list[-1];
  const FlowRec* recs = A.rec;
  if (A.smem_recs) {  // uniform per launch
    int4* dst = reinterpret_cast<int4*>(flow_dyn);
    const int4* src = reinterpret_cast<const int4*>(A.rec);
    for (int k = threadIdx.x; k < per; k += blockDim.x) dst[k] = src[k];  // 3 int4 per record
    __syncthreads();
    recs = reinterpret_cast<const FlowRec*>(flow_dyn);
  }
  const int per_level = A.red_black ? K / 2 : K;
  const int levels = MIXED ? mixed_levels(A.sweeps, K) : (A.sweeps + per_level - 1) / per_level;
  const long long total = (long long)levels * per;
  FlowRec R{};
  int v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (threadIdx.x == 0 && blockIdx.x < total) {
    const int r = (int)blockIdx.x % per;
    R = load_rec(recs + r / 3);
    load_counters(A, R, r % 3, v);
  }
  for (long long idx = blockIdx.x; idx < total; idx += gridDim.x) {
    const int z = (int)(idx / per), r = (int)(idx - (long long)z * per);
    const int a = r / 3, c = r - 3 * a;
    if (threadIdx.x == 0) {
      const bool ok = z == 0 || wait_counters(A, R, c, z, v);
      // Acquire: the counters read above (relaxed) order the neighbours'
      // published writes before every read that follows the barrier below.
      asm volatile("fence.acq_rel.gpu;" ::: "memory");
      s_stop = !ok;
      s_tile = R.tile;
      s_flag = R.flag;
    }
    __syncthreads();
    if (s_stop) break;
    const int tile = s_tile;
    if constexpr (MIXED) {
      const MixedLevel L = mixed_level(z, A.sweeps, K);
      if (L.type == 0) {
        if (s_flag == 2)
          flow_fold_item<true, TS>(A, tile, c, L.cycle, L.k, edge, lane, w);
        else
          flow_fold_item<false, TS>(A, tile, c, L.cycle, L.k, edge, lane, w);
      } else if (L.type == 1) {
        if (s_flag == 2)
          flow_inner_item<true, TS>(A, tile, c, L.pos, L.k, edge, lane, w);
        else
          flow_inner_item<false, TS>(A, tile, c, L.pos, L.k, edge, lane, w);
      } else {
        flow_flush_item<TS>(A, tile, c, L.cycle, L.nlast);
      }
    } else if constexpr (K == kK) {
      if (A.red_black) {
        if (s_flag == 2)
          flow_rb_item<true>(A, tile, c, z, edge, lane, w);
        else
          flow_rb_item<false>(A, tile, c, z, edge, lane, w);
      } else {
        flow_jacobi_item<K, PINB>(A, s_flag, tile, c, z, edge, lane, w);
      }
    } else {
      flow_jacobi_item<K, PINB>(A, s_flag, tile, c, z, edge, lane, w);
    }
    const long long next = idx + gridDim.x;
    if (threadIdx.x == 0 && next < total) {
      const int rn = (int)(next % per);
      R = load_rec(recs + rn / 3);
      load_counters(A, R, rn % 3, v);
    }
    // Release: the CTA barrier orders every thread's writes before the
    // release reduction, which makes them visible before the count.  Thread
    // 32 issues it, not thread 0: thread 0's acquire fence at the next item
    // would otherwise wait for this reduction to be performed at L2.
    __syncthreads();
    if (threadIdx.x == 32) release_add(A.done + 3 * a + c);
  }
}

// inv[t] = index of tile t in the active list, -1 for inactive tiles.
__global__ void grid_code_kernel(GridGeom G, const uint8_t* __restrict__ mask,
                                 uint8_t* __restrict__ code) {
  const long long n = G.plane;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const int row = (int)(p / G.pitch), col = (int)(p - (long long)row * G.pitch);
    uint8_t c = 1;
    if (!mask[p]) {
      const bool nb = (row > 0 && mask[p - G.pitch]) || (row < G.rows - 1 && mask[p + G.pitch]) ||
                      (col > 0 && mask[p - 1]) || (col < G.pitch - 1 && mask[p + 1]);
      c = nb ? 2 : 0;
    }
    code[p] = c;
  }
}

// One block per active tile (blocks past the active count return): the
// sweep body of its region (kBody*) from the code plane, for regions with
// unmasked pixels (tile flag 1).  Warps whose strip holds no masked pixel
// idle in the sweeps and do not count.
__global__ void flow_body_kernel(GridGeom G, const uint8_t* __restrict__ code,
                                 const int* __restrict__ list, int tiles_x, int th, int tw, int k,
                                 FlowRec* __restrict__ rec) {
  __shared__ unsigned s_masked[kW], s_col[kW], s_rows[kW];
  const int a = blockIdx.x;
  if (a >= list[-1] || rec[a].flag == 2) return;  // uniform per block
  if (threadIdx.x < kW) s_masked[threadIdx.x] = s_col[threadIdx.x] = s_rows[threadIdx.x] = 0;
  __syncthreads();
  const int tile = list[a], ty = tile / tiles_x, tx = tile - ty * tiles_x;
  const int r0 = ty * th - k, c0 = tx * tw - k;
  for (int q = threadIdx.x; q < kW * kR * 128; q += blockDim.x) {
    const int i = q >> 7, j = q & 127;  // region row, column
    const uint8_t cv = code[G.at(r0 + i, c0 + j)];
    const int w = i / kR, pr = (i % kR) % (kR / 2);
    if (cv & 1) s_masked[w] = 1;
    if (cv & 2) {
      atomicOr(&s_col[w], 1u << (j & 3));
      atomicOr(&s_rows[w], 1u << pr);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned col = 0;
    bool wide = false;
    for (int w = 0; w < kW; ++w)
      if (s_masked[w]) {
        col |= s_col[w];
        wide = wide || __popc(s_rows[w]) > 2;
      }
    int body = kBodyAll;
    if (col == 0 || col == 1) body = kBodyCol0;
    else if (col == 2) body = kBodyCol0 + 1;
    else if (col == 4) body = kBodyCol0 + 2;
    else if (col == 8) body = kBodyCol0 + 3;
    else if (!wide) body = kBodyRows;
    rec[a].flag = body;
  }
}

__global__ void flow_inv_kernel(const int* __restrict__ list, int tiles, int* __restrict__ inv) {
  const int n = list[-1];
  for (int t = threadIdx.x; t < tiles; t += blockDim.x) inv[t] = -1;
  __syncthreads();  // one block: the -1 fill precedes the scatter
  for (int a = threadIdx.x; a < n; a += blockDim.x) inv[list[a]] = a;
}

__global__ void flow_rec_kernel(const int* __restrict__ list, const int* __restrict__ inv,
                                const uint8_t* __restrict__ flags, int tiles_x, int tiles_y,
                                FlowRec* __restrict__ rec) {
  const int n = list[-1];
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
    const int tile = list[a], ty = tile / tiles_x, tx = tile - ty * tiles_x;
    FlowRec R;
    R.tile = tile;
    R.flag = flags[tile];
    R.pad = 0;
    for (int k = 0; k < 9; ++k) {
      const int y = ty + k / 3 - 1, x = tx + k % 3 - 1;
      const int b = (y >= 0 && y < tiles_y && x >= 0 && x < tiles_x) ? inv[y * tiles_x + x] : -1;
      R.nb[k] = b >= 0 ? 3 * b : -1;
    }
    rec[a] = R;
  }
}

}  // namespace

bool flow_depth_ok(int depth) { return depth == 16 || depth == 12; }
int flow_tile_h(int depth) { return depth == 12 ? FlowTile<12>::H : FlowTile<kK>::H; }
int flow_tile_w(int depth) { return depth == 12 ? FlowTile<12>::W : FlowTile<kK>::W; }
int flow_depth() { return kK; }
int flow_rb_depth() { return kK / 2; }

// Dynamic shared memory of a launch over `tiles` tiles (at most that many
// active): every record when they fit, else none.
static size_t flow_rec_smem(int tiles) {
  return tiles <= kFlowRecsSmem ? sizeof(FlowRec) * (size_t)tiles : 0;
}

int flow_ctas() {
  // Occupancy queries cost tens of microseconds; the answer is fixed per
  // device, and every reset rebuilds the flow tables.
  static std::atomic<int> cached[64];
  int dev = 0, sms = 0, per_sm = 0;
  FPIE_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && cached[dev].load(std::memory_order_relaxed) > 0)
    return cached[dev].load(std::memory_order_relaxed);
  FPIE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  int m = 1 << 30;
  const void* ks[6] = {(const void*)grid_flow_kernel<float, kK>,
                       (const void*)grid_flow_kernel<float, 12>,
                       (const void*)grid_flow_kernel<float, kK, true>,
                       (const void*)grid_flow_kernel<float, 12, true>,
                       (const void*)grid_flow_kernel<__half, kK>,
                       (const void*)grid_flow_kernel<__nv_bfloat16, kK>};
  for (const void* k : ks) {
    FPIE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kW * 32,
                                                            sizeof(FlowRec) * kFlowRecsSmem));
    m = std::min(m, per_sm);
  }
  FPIE_REQUIRE(m >= 1, FPIE_ERR_CUDA, "the flow sweep kernel does not fit on an SM");
  if (dev >= 0 && dev < 64) cached[dev].store(sms * m, std::memory_order_relaxed);
  return sms * m;
}

void launch_flow_tables(const GridGeom& G, const uint8_t* code, int depth, const int* list,
                        const uint8_t* flags, int tiles_x, int tiles, int* inv, void* rec,
                        cudaStream_t st) {
  flow_inv_kernel<<<1, 1024, 0, st>>>(list + 1, tiles, inv);
  flow_rec_kernel<<<(tiles + 255) / 256, 256, 0, st>>>(list + 1, inv, flags, tiles_x,
                                                       tiles / tiles_x,
                                                       static_cast<FlowRec*>(rec));
  flow_body_kernel<<<tiles, 256, 0, st>>>(G, code, list + 1, tiles_x, flow_tile_h(depth),
                                          flow_tile_w(depth), depth, static_cast<FlowRec*>(rec));
}

size_t flow_rec_bytes() { return sizeof(FlowRec); }

void launch_grid_code(const GridGeom& G, const uint8_t* mask, uint8_t* code, cudaStream_t st) {
  grid_code_kernel<<<stride_blocks(G.plane, 256, 4), 256, 0, st>>>(G, mask, code);
}

void launch_flow(const GridGeom& G, const uint8_t* mask, const uint8_t* code, const float* g,
                 float* x0, float* x1, int parity, const int* list, const void* rec, int* done,
                 int tiles_x, int tiles, int sweeps, int* error, long long spin_limit, int ctas,
                 cudaStream_t st, bool red_black, int depth, bool pin_bodies) {
  FPIE_REQUIRE(sweeps >= 1, FPIE_ERR_ARG, "flow sweep kernel: at least one sweep");
  FPIE_REQUIRE(depth == kK || (depth == 12 && !red_black), FPIE_ERR_ARG,
               "flow sweep kernel: depth 16, or 12 for Jacobi sweeps");
  FPIE_REQUIRE(!pin_bodies || code, FPIE_ERR_STATE, "flow sweep kernel: no code plane");
  FPIE_REQUIRE(tiles_x >= 1 && tiles % tiles_x == 0 && ctas >= 1, FPIE_ERR_STATE,
               "flow sweep kernel: bad tiling");
  FlowArgs a{G, mask, code, g, {x0, x1}, {nullptr, nullptr}, nullptr, list + 1,
             static_cast<const FlowRec*>(rec), done, error, tiles_x, sweeps, parity & 1,
             spin_limit, red_black ? 1 : 0, flow_rec_smem(tiles) > 0 ? 1 : 0};
  void* args[] = {&a};
  FPIE_REQUIRE(!pin_bodies || !red_black, FPIE_ERR_ARG,
               "flow sweep kernel: pinned-boundary bodies are for Jacobi sweeps");
  const void* k = depth == 12 ? (pin_bodies ? (const void*)grid_flow_kernel<float, 12, true>
                                            : (const void*)grid_flow_kernel<float, 12>)
                              : (pin_bodies ? (const void*)grid_flow_kernel<float, kK, true>
                                            : (const void*)grid_flow_kernel<float, kK>);
  FPIE_CUDA(cudaLaunchCooperativeKernel(k, dim3(ctas), dim3(kW * 32), args, flow_rec_smem(tiles),
                                        st));
}

void launch_flow_mixed(const GridGeom& G, const uint8_t* mask, const float* g, float* x0, float* x1,
                       int parity, bool bf16, void* e0, void* e1, float* r, const int* list,
                       const void* rec, int* done, int tiles_x, int tiles, int sweeps, int* error,
                       long long spin_limit, int ctas, cudaStream_t st) {
  FPIE_REQUIRE(sweeps >= 1, FPIE_ERR_ARG, "flow sweep kernel: at least one sweep");
  FPIE_REQUIRE(tiles_x >= 1 && tiles % tiles_x == 0 && ctas >= 1, FPIE_ERR_STATE,
               "flow sweep kernel: bad tiling");
  FlowArgs a{G, mask, nullptr, g, {x0, x1}, {e0, e1}, r, list + 1, static_cast<const FlowRec*>(rec), done,
             error, tiles_x, sweeps, parity & 1, spin_limit, 0, flow_rec_smem(tiles) > 0 ? 1 : 0};
  void* args[] = {&a};
  const void* k = bf16 ? (const void*)grid_flow_kernel<__nv_bfloat16, kK>
                       : (const void*)grid_flow_kernel<__half, kK>;
  FPIE_CUDA(cudaLaunchCooperativeKernel(k, dim3(ctas), dim3(kW * 32), args, flow_rec_smem(tiles),
                                        st));
}

int flow_mixed_flips(int sweeps) { return (sweeps + 63) / 64; }

}  // namespace fpie
