// Temporally blocked grid sweep: up to K Jacobi sweeps per launch.
//
// A CTA handles one channel plane of one tile.  It loads a 128-column x
// (W*R)-row region (the tile plus a K-pixel apron on every side) into
// registers: lane l of warp w owns columns 4l..4l+3 and rows w*R..w*R+R-1 of
// the region, with their grad values and mask bits.  Each sweep then needs
//   * left/right neighbours: the group's inner pixels from its own registers,
//     the group's edge pixels from the adjacent lanes (warp shuffles);
//   * up/down neighbours: the strip's inner rows from its own registers, the
//     strip's first/last row from the warps above/below (shared memory,
//     double-buffered by sweep parity so one barrier per sweep suffices).
// Values near the region border go stale sweep by sweep (their neighbours
// outside the region are not updated), but after k <= K sweeps every pixel
// at least K away from the border is exact, so the tile interior is written
// back and the apron discarded.  Arithmetic per pixel is exactly the
// one-sweep kernel's (numpy order), so results are bit-identical for any K.
//
// HBM traffic per launch: x, grad and mask of the region once in, the tile's
// x once out -- about 37/k bytes per pixel-sweep instead of 37.
#include "common.cuh"
#include "grid_tb.cuh"

namespace fpie {

// One sweep over the strip in registers.  FULL: the whole region is masked,
// so the per-pixel mask select is skipped (same arithmetic for set pixels).
template <int R, int W, bool FULL, bool GS>
__device__ __forceinline__ void tb_sweep(float4 (&x)[R], const float4 (&gg)[R],
                                         const uint32_t (&mk)[R],
                                         const float4* __restrict__ sg,
                                         float4 prev, float4 below, int lane) {
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const float4 cur = x[r];
    const float4 dn = r < R - 1 ? x[r + 1] : below;
    const float lf = __shfl_up_sync(0xffffffffu, cur.w, 1);
    const float rt = __shfl_down_sync(0xffffffffu, cur.x, 1);
    const float4 g = GS ? sg[r * 32 + lane] : gg[r];
    float4 o;
    o.x = jacobi5(g.x, prev.x, dn.x, lf, cur.y);
    o.y = jacobi5(g.y, prev.y, dn.y, cur.x, cur.z);
    o.z = jacobi5(g.z, prev.z, dn.z, cur.y, cur.w);
    o.w = jacobi5(g.w, prev.w, dn.w, cur.z, rt);
    if (!FULL) {
      const uint32_t m = mk[r];
      o.x = (m & 0x000000ffu) ? o.x : cur.x;
      o.y = (m & 0x0000ff00u) ? o.y : cur.y;
      o.z = (m & 0x00ff0000u) ? o.z : cur.z;
      o.w = (m & 0xff000000u) ? o.w : cur.w;
    }
    prev = cur;
    x[r] = o;
  }
}

// GS: the grad values live in shared memory (dynamic, W*R*32 float4)
// instead of registers, which frees 4R registers per thread for taller
// regions at the same occupancy.
template <int R, int W, int K, bool GS>
__global__ void __launch_bounds__(W * 32)
grid_tb_kernel(GridGeom G, const uint8_t* __restrict__ mask,
               const float* __restrict__ g, const float* __restrict__ xin,
               float* __restrict__ xout, const uint8_t* __restrict__ active,
               int tiles_x, int ksweeps) {
  constexpr int TH = W * R - 2 * K;
  constexpr int TW = 128 - 2 * K;
  static_assert(K % 4 == 0 && K > 0 && K <= kPad, "apron must be a multiple of 4, at most kPad");
  static_assert(TH > 0, "tile must have rows");
  __shared__ float4 edge[2][2][W][32];  // [parity][0 = first row, 1 = last row][warp][lane]
  extern __shared__ float4 sgrad[];     // GS only: [W*R rows][32 lanes]

  const int tile = blockIdx.x;
  const uint8_t flag = active[tile];
  if (!flag) return;
  const int c = blockIdx.y;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int ty = tile / tiles_x, tx = tile - ty * tiles_x;
  const int row0 = ty * TH - K + w * R;    // crop row of this strip's first row
  const int col0 = tx * TW - K + 4 * lane;  // crop column of this lane's first column
  const long long base = G.at(row0, col0);
  const float* xc = xin + c * G.plane;
  const float* gc = g + c * G.plane;
  float4* sg = sgrad + w * R * 32;

  float4 x[R], gg[R];
  uint32_t mk[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const long long p = base + (long long)r * G.pitch;
    x[r] = ld4(xc + p);
    if (GS)
      sg[r * 32 + lane] = ld4(gc + p);
    else
      gg[r] = ld4(gc + p);
    mk[r] = __ldg(reinterpret_cast<const unsigned int*>(mask + p));
  }

  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int s = 0; s < ksweeps; ++s) {
    const int par = s & 1;
    edge[par][0][w][lane] = x[0];
    edge[par][1][w][lane] = x[R - 1];
    __syncthreads();  // also orders the grad stores before the first sweep
    const float4 prev = w > 0 ? edge[par][1][w - 1][lane] : zero;
    const float4 below = w < W - 1 ? edge[par][0][w + 1][lane] : zero;
    if (flag == 2)
      tb_sweep<R, W, true, GS>(x, gg, mk, sg, prev, below, lane);
    else
      tb_sweep<R, W, false, GS>(x, gg, mk, sg, prev, below, lane);
  }

  if (lane >= K / 4 && lane < 32 - K / 4) {
    float* oc = xout + c * G.plane;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int rr = w * R + r;  // region row
      if (rr >= K && rr < W * R - K)
        *reinterpret_cast<float4*>(oc + base + (long long)r * G.pitch) = x[r];
    }
  }
}

// flags[t] = 0: tile t's interior (clipped to the crop) has no masked pixel;
// 2: every pixel of its region (interior plus a k-pixel apron, padding
// included) is masked; 1: otherwise.
__global__ void grid_tile_flags_kernel(GridGeom G, const uint8_t* __restrict__ mask,
                                       int th, int tw, int k, int tiles_x,
                                       uint8_t* __restrict__ flags) {
  const int t = blockIdx.x;
  const int ty = t / tiles_x, tx = t - ty * tiles_x;
  const int r0 = ty * th, c0 = tx * tw;
  const int r1 = min(r0 + th, G.n), c1 = min(c0 + tw, G.m);
  int any = 0;
  for (int q = threadIdx.x; q < (r1 - r0) * (c1 - c0); q += blockDim.x) {
    const int i = r0 + q / (c1 - c0), j = c0 + q % (c1 - c0);
    any |= mask[G.at(i, j)];
  }
  // Region rows/cols may reach past the crop into the zero padding.
  const int R0 = r0 - k, C0 = c0 - k, RH = th + 2 * k, RW = tw + 2 * k;
  int all = 1;
  for (int q = threadIdx.x; q < RH * RW; q += blockDim.x) {
    const int i = R0 + q / RW, j = C0 + q % RW;
    all &= (i >= 0 && i < G.n && j >= 0 && j < G.m) ? (int)mask[G.at(i, j)] : 0;
  }
  any = __syncthreads_or(any);
  all = __syncthreads_and(all);
  if (threadIdx.x == 0) flags[t] = any ? (all ? 2 : 1) : 0;
}

namespace {

template <int R, int W, int K, bool GS>
constexpr size_t tb_dyn_smem() {
  return GS ? (size_t)W * R * 32 * sizeof(float4) : 0;
}

template <int R, int W, int K, bool GS>
void prepare_tb() {
  if (tb_dyn_smem<R, W, K, GS>() > 48 * 1024)
    FPIE_CUDA(cudaFuncSetAttribute(grid_tb_kernel<R, W, K, GS>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)tb_dyn_smem<R, W, K, GS>()));
}

template <int R, int W, int K, bool GS>
void launch_tb(const GridGeom& G, const uint8_t* mask, const float* g,
               const float* xin, float* xout, const uint8_t* active,
               int tiles_x, int tiles, int ksweeps, cudaStream_t st) {
  grid_tb_kernel<R, W, K, GS><<<dim3(tiles, 3), W * 32, tb_dyn_smem<R, W, K, GS>(), st>>>(
      G, mask, g, xin, xout, active, tiles_x, ksweeps);
}

template <int R, int W, int K, bool GS>
TbVariant make_variant(const char* name) {
  TbVariant v;
  v.name = name;
  v.rows_per_thread = R;
  v.warps = W;
  v.depth = K;
  v.apron = K;
  v.tile_h = W * R - 2 * K;
  v.tile_w = 128 - 2 * K;
  v.launch = &launch_tb<R, W, K, GS>;
  v.prepare = &prepare_tb<R, W, K, GS>;
  return v;
}

}  // namespace

void append_packed_variants(std::vector<TbVariant>& v);  // grid_tbp.cu

const std::vector<TbVariant>& tb_variants() {
  static const std::vector<TbVariant> v = [] {
    std::vector<TbVariant> t = {
        make_variant<8, 8, 8, false>("r8w8k8"),
        make_variant<16, 8, 8, false>("r16w8k8"),
        make_variant<8, 16, 8, false>("r8w16k8"),
        make_variant<16, 8, 16, false>("r16w8k16"),
        make_variant<8, 16, 16, false>("r8w16k16"),
        make_variant<16, 10, 8, true>("r16w10k8s"),
        make_variant<16, 12, 8, true>("r16w12k8s"),
        make_variant<12, 16, 16, true>("r12w16k16s"),
    };
    append_packed_variants(t);
    return t;
  }();
  return v;
}

void launch_tile_flags(const GridGeom& G, const uint8_t* mask, int th, int tw, int k,
                       int tiles_x, int tiles, uint8_t* flags, cudaStream_t st) {
  grid_tile_flags_kernel<<<tiles, 256, 0, st>>>(G, mask, th, tw, k, tiles_x, flags);
}

}  // namespace fpie
