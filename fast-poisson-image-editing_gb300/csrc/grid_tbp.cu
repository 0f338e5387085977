// Temporally blocked grid sweep with packed FP32 pairs ("p" variants).
//
// Same tiling as grid_tb.cu (a CTA = one channel of one tile; lane l of warp w
// owns columns 4l..4l+3 and R rows of a 128-column region), but each thread
// keeps its strip as R/2 row pairs: pair i holds rows i and i + R/2 of the
// strip.  Then, for every pair except the first and the last, the up, down,
// left and right neighbours are themselves pairs the thread already holds,
// so a pixel update of two rows at once is four __fadd2_rn and one
// __fmul2_rn (Blackwell's packed FP32 adds: two IEEE round-to-nearest adds
// per instruction).  Only pair 0's "up" and pair R/2-1's "down" mix a row
// from another warp (shared memory) with one of the thread's own.
//
// Each lane of a packed add is an ordinary float32 add, and the addition
// order is the numpy backend's ((((g + up) + down) + left) + right) * 0.25,
// so results are bit-identical to every other sweep kernel.
//
// The select that keeps unmasked pixels is compiled only into the path for
// regions holding unmasked pixels (tile flag 1); fully masked regions (flag
// 2) take a path without it.  The choice is made once per CTA.
#include "common.cuh"
#include "grid_tb.cuh"
#include "grid_tbp.cuh"

namespace fpie {

// RB: red-black sweeps (the EquSolver's red-black order on its grid
// placement); K is then the apron, ksweeps <= K / 2.
template <int R, int W, int K, typename TS, bool ZS, bool GS = false, bool RB = false>
__global__ void __launch_bounds__(W * 32)
grid_tbp_kernel(GridGeom G, const uint8_t* __restrict__ mask,
                const float* __restrict__ g, const TS* __restrict__ xin,
                TS* __restrict__ xout, const uint8_t* __restrict__ active,
                int tiles_x, int ksweeps) {
  extern __shared__ float4 tbp_dyn[];
  constexpr int TH = W * R - 2 * K;
  constexpr int TW = 128 - 2 * K;
  static_assert(R % 2 == 0 && R >= 4, "rows per thread must be even");
  static_assert(K % 4 == 0 && K > 0 && K <= kPad, "apron must be a multiple of 4, at most kPad");
  static_assert(TH > 0, "tile must have rows");
  __shared__ float4 edge[2][2][W][32];
  const int tile = blockIdx.x;
  const uint8_t flag = active[tile];
  if (!flag) return;
  const int c = blockIdx.y;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int ty = tile / tiles_x, tx = tile - ty * tiles_x;
  const long long base = G.at(ty * TH - K + w * R, tx * TW - K + 4 * lane);
  const TS* xc = xin + c * G.plane;
  const float* gc = g + c * G.plane;
  TS* oc = xout + c * G.plane;
  float2* sg = reinterpret_cast<float2*>(tbp_dyn) + (size_t)w * (R / 2) * 32 * 4;
  if (flag == 2)
    tbp_body<R, W, K, true, TS, ZS, false, GS, RB>(G, mask, gc, xc, oc, base, ksweeps, lane, w, edge, sg);
  else
    tbp_body<R, W, K, false, TS, ZS, false, GS, RB>(G, mask, gc, xc, oc, base, ksweeps, lane, w, edge, sg);
}

// Fused first launch of a refinement cycle (tbp_fold_body): all channels'
// tiles, like grid_tbp_kernel.
template <int R, int W, int K, typename TS, bool HASE>
__global__ void __launch_bounds__(W * 32)
grid_tbp_fold_kernel(GridGeom G, const uint8_t* __restrict__ mask, const float* __restrict__ g,
                     const float* __restrict__ xin, const TS* __restrict__ elast,
                     float* __restrict__ xout, float* __restrict__ rout, TS* __restrict__ eout,
                     const uint8_t* __restrict__ active, int tiles_x, int ksweeps) {
  constexpr int TH = W * R - 2 * K;
  constexpr int TW = 128 - 2 * K;
  __shared__ float4 edge[2][2][W][32];
  const int tile = blockIdx.x;
  const uint8_t flag = active[tile];
  if (!flag) return;
  const int c = blockIdx.y;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int ty = tile / tiles_x, tx = tile - ty * tiles_x;
  const long long base = G.at(ty * TH - K + w * R, tx * TW - K + 4 * lane);
  const long long co = c * G.plane;
  if (flag == 2)
    tbp_fold_body<R, W, K, true, TS, HASE>(G, mask, g + co, xin + co, HASE ? elast + co : nullptr,
                                           xout + co, rout + co, eout + co, base, ksweeps, lane, w, edge);
  else
    tbp_fold_body<R, W, K, false, TS, HASE>(G, mask, g + co, xin + co, HASE ? elast + co : nullptr,
                                            xout + co, rout + co, eout + co, base, ksweeps, lane, w, edge);
}

namespace {

void no_prepare() {}

template <int R, int W, bool GS>
constexpr size_t tbp_smem() {
  return GS ? (size_t)W * R * 32 * 4 * sizeof(float2) / 2 : 0;
}

template <int R, int W, int K, bool GS>
void prepare_tbp() {
  if (tbp_smem<R, W, GS>() > 48 * 1024)
    FPIE_CUDA(cudaFuncSetAttribute(grid_tbp_kernel<R, W, K, float, false, GS>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)tbp_smem<R, W, GS>()));
}

template <int R, int W, int K, bool GS = false, bool RB = false>
void launch_tbp(const GridGeom& G, const uint8_t* mask, const float* g,
                const float* xin, float* xout, const uint8_t* active,
                int tiles_x, int tiles, int ksweeps, cudaStream_t st) {
  grid_tbp_kernel<R, W, K, float, false, GS, RB><<<dim3(tiles, 3), W * 32, tbp_smem<R, W, GS>(), st>>>(
      G, mask, g, xin, xout, active, tiles_x, ksweeps);
}

template <int R, int W, int K, bool GS = false>
TbVariant make_packed(const char* name) {
  TbVariant v;
  v.name = name;
  v.rows_per_thread = R;
  v.warps = W;
  v.depth = K;
  v.apron = K;
  v.tile_h = W * R - 2 * K;
  v.tile_w = 128 - 2 * K;
  v.launch = &launch_tbp<R, W, K, GS>;
  v.prepare = GS ? &prepare_tbp<R, W, K, GS> : &no_prepare;
  return v;
}

// Red-black variant: KS red-black sweeps per launch on tiles with an apron
// of 2 * KS.
template <int R, int W, int KS>
TbVariant make_packed_rb(const char* name) {
  TbVariant v;
  v.name = name;
  v.rows_per_thread = R;
  v.warps = W;
  v.depth = KS;
  v.apron = 2 * KS;
  v.tile_h = W * R - 4 * KS;
  v.tile_w = 128 - 4 * KS;
  v.red_black = true;
  v.launch = &launch_tbp<R, W, 2 * KS, false, true>;
  v.prepare = &no_prepare;
  return v;
}

template <int R, int W, int K, typename TS>
void launch_tbp_lp(const GridGeom& G, const uint8_t* mask, const float* r, const void* ein,
                   void* eout, const uint8_t* active, int tiles_x, int tiles, int ksweeps,
                   int zero_start, cudaStream_t st) {
  if (zero_start)
    grid_tbp_kernel<R, W, K, TS, true><<<dim3(tiles, 3), W * 32, 0, st>>>(
        G, mask, r, nullptr, static_cast<TS*>(eout), active, tiles_x, ksweeps);
  else
    grid_tbp_kernel<R, W, K, TS, false><<<dim3(tiles, 3), W * 32, 0, st>>>(
        G, mask, r, static_cast<const TS*>(ein), static_cast<TS*>(eout), active, tiles_x,
        ksweeps);
}

template <int R, int W, int K, typename TS>
void launch_fold(const GridGeom& G, const uint8_t* mask, const float* g, const float* xin,
                 const void* elast, float* xout, float* rout, void* eout, const uint8_t* active,
                 int tiles_x, int tiles, int ksweeps, cudaStream_t st) {
  if (elast)
    grid_tbp_fold_kernel<R, W, K, TS, true><<<dim3(tiles, 3), W * 32, 0, st>>>(
        G, mask, g, xin, static_cast<const TS*>(elast), xout, rout, static_cast<TS*>(eout),
        active, tiles_x, ksweeps);
  else
    grid_tbp_fold_kernel<R, W, K, TS, false><<<dim3(tiles, 3), W * 32, 0, st>>>(
        G, mask, g, xin, nullptr, xout, rout, static_cast<TS*>(eout), active, tiles_x, ksweeps);
}

template <int R, int W, int K>
MixedVariant make_mixed(const char* name) {
  MixedVariant v;
  v.name = name;
  v.depth = K;
  v.tile_h = W * R - 2 * K;
  v.tile_w = 128 - 2 * K;
  v.launch_fp16 = &launch_tbp_lp<R, W, K, __half>;
  v.launch_bf16 = &launch_tbp_lp<R, W, K, __nv_bfloat16>;
  v.fold_fp16 = &launch_fold<R, W, K, __half>;
  v.fold_bf16 = &launch_fold<R, W, K, __nv_bfloat16>;
  return v;
}

}  // namespace

const std::vector<MixedVariant>& mixed_variants() {
  static const std::vector<MixedVariant> v = {
      make_mixed<16, 8, 16>("p16w8k16"),
      make_mixed<8, 16, 16>("p8w16k16"),
      make_mixed<16, 8, 8>("p16w8k8"),
  };
  return v;
}

void append_packed_variants(std::vector<TbVariant>& v) {
  v.push_back(make_packed<16, 8, 8>("p16w8k8"));
  v.push_back(make_packed<16, 8, 16>("p16w8k16"));
  // Short regions (64 rows) for small grids: twice the tiles of the 128-row
  // variants, so a small paste keeps more SMs busy.
  v.push_back(make_packed<8, 8, 8>("p8w8k8"));
  v.push_back(make_packed<8, 16, 16>("p8w16k16"));
  v.push_back(make_packed_rb<16, 8, 8>("rb16w8k8"));
}

}  // namespace fpie
