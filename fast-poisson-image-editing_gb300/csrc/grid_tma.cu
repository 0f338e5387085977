// Persistent temporally blocked sweep with TMA prefetch ("p16w8k16t").
//
// Same tiling and arithmetic as the packed variant p16w8k16 (grid_tbp.cuh:
// 96x96 tiles, 128x128 regions, up to 16 sweeps per launch, bit-identical
// results), but each CTA is persistent: it takes (active tile, channel)
// items round-robin and, while it sweeps one item from registers, the
// Tensor Memory Accelerator copies the next item's region -- x (64 KB),
// grad (64 KB) and mask (16 KB) -- into shared memory (cp.async.bulk.tensor,
// completion counted on an mbarrier).  The region load that every CTA of a
// launch-per-tile kernel waits for is hidden behind the previous item's
// sweeps.
//
// Items: a list of the active tiles (tma_list_kernel, in tile order, built
// once per mask) x 3 channels; item i is tile list[i / 3], channel i % 3,
// and CTA b takes items b, b + gridDim.x, ...  Each CTA copies its share of
// the list into shared memory at the start, so issuing the next copy never
// waits on a global load (a stalled issuing thread would hold every warp at
// the next barrier).
//
// Threads wait on the mbarrier with mbarrier.try_wait (suspended in
// hardware, not spinning on shared memory, which would slow the very copies
// being waited for).  A wait is bounded by a number of checks (the solver's
// spin limit, default 2^26) and by about a second of SM clock: past either
// the CTA records an error, waits again (bounded) for its copies in flight
// to land, and stops taking items; the host reports FPIE_ERR_TIMEOUT.
//
// TMA rules, checked here or on the host before any launch: every box
// starts at a column that is a multiple of 16 bytes (region column
// 96*tx + 16 from a 128-byte-aligned row, for floats and mask bytes
// alike), global strides are multiples of 16 bytes, the shared
// destinations are 1024-byte aligned, and every box lies inside the
// allocation (the grid keeps kPad + slack rows/columns of padding), so no
// out-of-bounds fill is relied on.
#include <cuda.h>

#include <algorithm>
#include <string>

#include "common.cuh"
#include "grid_tbp.cuh"
#include "grid_tma.cuh"

namespace fpie {

namespace {

constexpr int kR = 16, kW = 8, kK = 16, kH = kR / 2;
constexpr int kTH = kW * kR - 2 * kK;  // 96
constexpr int kTW = 128 - 2 * kK;      // 96
constexpr int kRegion = 128;
constexpr unsigned kXBytes = kRegion * kRegion * 4;
constexpr unsigned kMBytes = kRegion * kRegion;
constexpr unsigned kTxBytes = 2 * kXBytes + kMBytes;
constexpr unsigned kDynBytes = kTxBytes + 1024;  // + room to align the base to 1024
constexpr long long kDrainChecks = 1LL << 26;  // wait for copies in flight after a time-out
constexpr long long kWaitCycles = 2000000000LL;  // ~1 s at the maximum SM clock
constexpr unsigned kSuspendNs = 4000;            // hardware suspend hint per check
// Items one CTA may take (its schedule lives in shared memory); the host
// checks 3 x tiles <= kMaxItemsPerCta x CTAs before a launch.
constexpr int kMaxItemsPerCta = 2048;

static_assert(kTH == kTW && kTH == 96, "tile extents");
// Column coordinate of a region: 96*tx - kK + kPad elements from a row start
// that is 128-byte aligned; it must be a multiple of 16 bytes for floats
// and for mask bytes.
static_assert((kTW % 16) == 0 && ((kPad - kK) % 16) == 0, "TMA column alignment");

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tm, int c0, int c1,
                                            int c2, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];"
      :
      : "r"(smem_addr(dst)), "l"(reinterpret_cast<uint64_t>(tm)), "r"(c0), "r"(c1), "r"(c2),
        "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, int c0, int c1,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];"
      :
      : "r"(smem_addr(dst)), "l"(reinterpret_cast<uint64_t>(tm)), "r"(c0), "r"(c1),
        "r"(smem_addr(bar))
      : "memory");
}

// Non-blocking test of phase `parity` of the mbarrier.
__device__ __forceinline__ bool mbar_test(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Checks phase `parity`, letting the hardware suspend the thread (up to
// about kSuspendNs) until it completes.
__device__ __forceinline__ bool mbar_try(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity), "r"(kSuspendNs)
      : "memory");
  return ok != 0;
}

// Waits for the phase; false after `limit` unsuccessful checks (0: only
// the immediate test) or kWaitCycles SM cycles.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity,
                                                  long long limit) {
  if (mbar_test(bar, parity)) return true;
  const long long t0 = clock64();
  for (long long n = 0; n < limit; ++n) {
    if (mbar_try(bar, parity)) return true;
    if (clock64() - t0 > kWaitCycles) return false;
  }
  return false;
}

struct TmaArgs {
  GridGeom G;
  float* xout;
  const uint8_t* flags;  // per tile: 0 inactive, 1 mixed, 2 fully masked
  const int* list;       // active tiles in tile order; list[-1] = their count
  int tiles_x, ksweeps;
  int* error;
  long long wait_limit;
};

__device__ __forceinline__ void issue_item(const TmaArgs& A, const CUtensorMap* tx,
                                           const CUtensorMap* tg, const CUtensorMap* tm, int tile,
                                           int c, float* xs, float* gs, uint8_t* ms, uint64_t* bar) {
  const int ty = tile / A.tiles_x, txi = tile - ty * A.tiles_x;
  const int row0 = ty * kTH - kK + kPad, col0 = txi * kTW - kK + kPad;
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
               :
               : "r"(smem_addr(bar)), "r"(kTxBytes)
               : "memory");
  tma_load_3d(xs, tx, col0, row0, c, bar);
  tma_load_3d(gs, tg, col0, row0, c, bar);
  tma_load_2d(ms, tm, col0, row0, bar);
}

// One item k of this CTA (tile `tile`, channel c): region from shared
// memory into registers; then, once every thread has its copy, thread 0
// starts the copy of item k+1 (its tile read from the CTA's schedule in
// shared memory, so nothing here waits on global memory); then the sweeps
// and the store of the tile interior.
//
// Kept out of line: inlined into the persistent loop, the compiler's
// register assignment needed about five times the register moves per sweep
// (measured by instruction counters) of the same code in the
// launch-per-tile kernel; as a separate function it matches that kernel.
template <bool FULL>
__device__ __noinline__ void tma_item(const TmaArgs& A, const CUtensorMap& tm_x,
                                      const CUtensorMap& tm_g, const CUtensorMap& tm_m, int tile,
                                      int c, int next_tile, int next_c, float* xs, float* gs,
                                      uint8_t* ms, uint64_t* bar, float4 (&edge)[2][2][kW][32],
                                      int lane, int w) {
  const GridGeom& G = A.G;
  float2 P[kH][4], Gp[kH][4];
  uint32_t mk[kR];
#pragma unroll
  for (int i = 0; i < kH; ++i) {
    const int ra = w * kR + i, rb = ra + kH;
    const float4 a = *reinterpret_cast<const float4*>(xs + ra * kRegion + 4 * lane);
    const float4 b = *reinterpret_cast<const float4*>(xs + rb * kRegion + 4 * lane);
    const float4 ga = *reinterpret_cast<const float4*>(gs + ra * kRegion + 4 * lane);
    const float4 gb = *reinterpret_cast<const float4*>(gs + rb * kRegion + 4 * lane);
    P[i][0] = make_float2(a.x, b.x);
    P[i][1] = make_float2(a.y, b.y);
    P[i][2] = make_float2(a.z, b.z);
    P[i][3] = make_float2(a.w, b.w);
    Gp[i][0] = make_float2(ga.x, gb.x);
    Gp[i][1] = make_float2(ga.y, gb.y);
    Gp[i][2] = make_float2(ga.z, gb.z);
    Gp[i][3] = make_float2(ga.w, gb.w);
    if (!FULL) {
      mk[i] = *reinterpret_cast<const uint32_t*>(ms + ra * kRegion + 4 * lane);
      mk[i + kH] = *reinterpret_cast<const uint32_t*>(ms + rb * kRegion + 4 * lane);
    }
  }
  __syncthreads();  // every thread has its region: the staging buffers are free
  if (threadIdx.x == 0 && next_tile >= 0) {
    // Order the generic-proxy reads above before the async-proxy writes.
    asm volatile("fence.proxy.async.shared::cta;" : : : "memory");
    issue_item(A, &tm_x, &tm_g, &tm_m, next_tile, next_c, xs, gs, ms, bar);
  }
  tbp_sweeps<kR, kW, FULL, false>(P, Gp, mk, A.ksweeps, lane, w, edge, nullptr);
  const int ty = tile / A.tiles_x, txi = tile - ty * A.tiles_x;
  const long long base = G.at(ty * kTH - kK + w * kR, txi * kTW - kK + 4 * lane);
  float* oc = A.xout + c * G.plane;
  if (lane >= kK / 4 && lane < 32 - kK / 4) {
#pragma unroll
    for (int i = 0; i < kH; ++i) {
      const int ra = w * kR + i, rb = ra + kH;
      if (ra >= kK && ra < kW * kR - kK)
        *reinterpret_cast<float4*>(oc + base + (long long)i * G.pitch) =
            make_float4(P[i][0].x, P[i][1].x, P[i][2].x, P[i][3].x);
      if (rb >= kK && rb < kW * kR - kK)
        *reinterpret_cast<float4*>(oc + base + (long long)(i + kH) * G.pitch) =
            make_float4(P[i][0].y, P[i][1].y, P[i][2].y, P[i][3].y);
    }
  }
}

// Items of CTA b: i = b, b + gridDim.x, ... < 3 x (active tiles); item i is
// tile list[i / 3], channel i % 3.  The CTA copies its tiles into s_tiles
// once, at the start.
__global__ void __launch_bounds__(kW * 32, 1)
grid_tma_kernel(const __grid_constant__ CUtensorMap tm_x, const __grid_constant__ CUtensorMap tm_g,
                const __grid_constant__ CUtensorMap tm_m, TmaArgs A) {
  extern __shared__ unsigned char tma_dyn[];
  __shared__ float4 edge[2][2][kW][32];
  __shared__ __align__(8) uint64_t bar;
  __shared__ int s_fail;
  __shared__ int s_tiles[kMaxItemsPerCta];
  unsigned char* smem = tma_dyn + ((1024u - (smem_addr(tma_dyn) & 1023u)) & 1023u);
  float* xs = reinterpret_cast<float*>(smem);
  float* gs = reinterpret_cast<float*>(smem + kXBytes);
  uint8_t* ms = smem + 2 * kXBytes;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int b = blockIdx.x, nctas = gridDim.x;
  const int items = 3 * A.list[-1];
  const int nk = b < items ? min(kMaxItemsPerCta, (items - b + nctas - 1) / nctas) : 0;
  for (int k = threadIdx.x; k < nk; k += blockDim.x) s_tiles[k] = A.list[(b + k * nctas) / 3];
  if (threadIdx.x == 0) {
    s_fail = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" : : "r"(smem_addr(&bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" : : : "memory");
    if (nk > 0) issue_item(A, &tm_x, &tm_g, &tm_m, A.list[b / 3], b % 3, xs, gs, ms, &bar);
  }
  __syncthreads();
  unsigned parity = 0;
  for (int k = 0; k < nk; ++k) {
    if (!mbar_wait_bounded(&bar, parity, A.wait_limit)) s_fail = 1;
    __syncthreads();
    if (s_fail) {
      if (threadIdx.x == 0) {
        atomicExch(A.error, 1);
        mbar_wait_bounded(&bar, parity, kDrainChecks);  // let the copies in flight land
      }
      break;
    }
    parity ^= 1u;
    const int i = b + k * nctas, tile = s_tiles[k];
    const int next_tile = k + 1 < nk ? s_tiles[k + 1] : -1, next_c = (i + nctas) % 3;
    if (A.flags[tile] == 2)
      tma_item<true>(A, tm_x, tm_g, tm_m, tile, i % 3, next_tile, next_c, xs, gs, ms, &bar, edge,
                     lane, w);
    else
      tma_item<false>(A, tm_x, tm_g, tm_m, tile, i % 3, next_tile, next_c, xs, gs, ms, &bar, edge,
                      lane, w);
    // The next item's first sweep writes the edge buffers: no warp may
    // still be reading this item's last sweep's edges.
    __syncthreads();
  }
}

// Active-tile list: list[-1] = number of tiles with a nonzero flag, then
// their indices in increasing order.  One CTA of 1024 threads; each thread
// takes a contiguous run of tiles, and a block-wide scan of the per-thread
// counts gives each run's output offset.
__global__ void __launch_bounds__(1024) tma_list_kernel(const uint8_t* __restrict__ flags,
                                                        int tiles, int* __restrict__ list) {
  __shared__ int part[1024];
  const int t = threadIdx.x, per = (tiles + 1023) / 1024;
  const int lo = min(tiles, t * per), hi = min(tiles, lo + per);
  int cnt = 0;
  for (int i = lo; i < hi; ++i) cnt += flags[i] != 0;
  part[t] = cnt;
  __syncthreads();
  for (int d = 1; d < 1024; d <<= 1) {  // inclusive scan (Hillis-Steele)
    const int v = t >= d ? part[t - d] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int o = part[t] - cnt;
  for (int i = lo; i < hi; ++i)
    if (flags[i]) list[o++] = i;
  if (t == 1023) list[-1] = part[1023];
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                 const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                 const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
  static EncodeTiled fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    // The CUDA 12.0 ABI of the entry point, which the typedef above follows.
    FPIE_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                               cudaEnableDefault, &q));
    FPIE_REQUIRE(p != nullptr && q == cudaDriverEntryPointSuccess, FPIE_ERR_CUDA,
                 "cuTensorMapEncodeTiled is not available from the driver");
    fn = reinterpret_cast<EncodeTiled>(p);
  }
  return fn;
}

void encode(CUtensorMap* tm, CUtensorMapDataType type, int rank, const void* base,
            const cuuint64_t* dims, const cuuint64_t* strides, const cuuint32_t* box) {
  FPIE_REQUIRE((reinterpret_cast<uintptr_t>(base) & 15) == 0, FPIE_ERR_STATE,
               "TMA base not 16-byte aligned");
  for (int k = 0; k < rank - 1; ++k)
    FPIE_REQUIRE(strides[k] % 16 == 0, FPIE_ERR_STATE, "TMA stride not a multiple of 16 bytes");
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = encoder()(tm, type, rank, const_cast<void*>(base), dims, strides, box, estr,
                               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                               CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  FPIE_REQUIRE(r == CUDA_SUCCESS, FPIE_ERR_CUDA,
               "cuTensorMapEncodeTiled failed with CUresult " + std::to_string((int)r));
}

}  // namespace

int tma_tile_h() { return kTH; }
int tma_tile_w() { return kTW; }
int tma_depth() { return kK; }

// Per device (the attribute is), so it runs on every call.
void prepare_tma() {
  FPIE_CUDA(cudaFuncSetAttribute(grid_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kDynBytes));
}

void launch_tma_list(const uint8_t* flags, int tiles, int* list, cudaStream_t st) {
  tma_list_kernel<<<1, 1024, 0, st>>>(flags, tiles, list + 1);
}

int tma_ctas(int items) {
  prepare_tma();
  int dev = 0, sms = 0, per_sm = 0;
  FPIE_CUDA(cudaGetDevice(&dev));
  FPIE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  FPIE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grid_tma_kernel, kW * 32,
                                                          kDynBytes));
  FPIE_REQUIRE(per_sm >= 1, FPIE_ERR_CUDA, "the TMA sweep kernel does not fit on an SM");
  return std::max(1, std::min(items, sms * per_sm));
}

void launch_tma(const GridGeom& G, const uint8_t* mask, const float* g, const float* xin,
                float* xout, const uint8_t* flags, const int* list, int tiles_x, int tiles,
                int ksweeps, int* error, long long wait_limit, int ctas, cudaStream_t st) {
  FPIE_REQUIRE(ksweeps >= 1 && ksweeps <= kK, FPIE_ERR_ARG, "TMA sweep kernel: 1..16 sweeps");
  FPIE_REQUIRE(G.pitch % 32 == 0, FPIE_ERR_STATE, "grid pitch must be a multiple of 32");
  FPIE_REQUIRE(tiles_x >= 1 && tiles % tiles_x == 0 && ctas >= 1, FPIE_ERR_STATE,
               "TMA sweep kernel: bad tiling");
  FPIE_REQUIRE(3LL * tiles <= (long long)kMaxItemsPerCta * ctas, FPIE_ERR_ARG,
               "TMA sweep kernel: grid too large for the per-CTA schedule");
  // The last region of each axis must lie inside the allocation.
  const int tiles_y = tiles / tiles_x;
  FPIE_REQUIRE((tiles_x - 1) * kTW - kK + kPad + kRegion <= G.pitch &&
                   (tiles_y - 1) * kTH - kK + kPad + kRegion <= G.rows,
               FPIE_ERR_STATE, "TMA region outside the grid allocation");
  CUtensorMap mx, mg, mm;
  const cuuint64_t fdims[3] = {(cuuint64_t)G.pitch, (cuuint64_t)G.rows, 3};
  const cuuint64_t fstr[2] = {(cuuint64_t)G.pitch * 4, (cuuint64_t)G.plane * 4};
  const cuuint32_t fbox[3] = {kRegion, kRegion, 1};
  encode(&mx, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, xin, fdims, fstr, fbox);
  encode(&mg, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, g, fdims, fstr, fbox);
  const cuuint64_t mdims[2] = {(cuuint64_t)G.pitch, (cuuint64_t)G.rows};
  const cuuint64_t mstr[1] = {(cuuint64_t)G.pitch};
  const cuuint32_t mbox[2] = {kRegion, kRegion};
  encode(&mm, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, mask, mdims, mstr, mbox);
  TmaArgs a{G, xout, flags, list + 1, tiles_x, ksweeps, error, wait_limit};
  grid_tma_kernel<<<ctas, kW * 32, kDynBytes, st>>>(mx, mg, mm, a);
}

}  // namespace fpie
