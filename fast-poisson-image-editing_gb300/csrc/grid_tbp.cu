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

namespace fpie {

__device__ __forceinline__ float2 pick2(uint32_t ma, uint32_t mb, uint32_t bit,
                                        float2 upd, float2 old) {
  return make_float2((ma & bit) ? upd.x : old.x, (mb & bit) ? upd.y : old.y);
}

template <int R, int W, int K, bool FULL>
__device__ __forceinline__ void tbp_body(const GridGeom& G, const uint8_t* __restrict__ mask,
                                         const float* __restrict__ gc,
                                         const float* __restrict__ xc, float* __restrict__ oc,
                                         long long base, int ksweeps, int lane, int w,
                                         float4 (&edge)[2][2][W][32]) {
  constexpr int H = R / 2;
  float2 P[H][4], Gp[H][4];
  uint32_t mk[R];
#pragma unroll
  for (int i = 0; i < H; ++i) {
    const long long pa = base + (long long)i * G.pitch;
    const long long pb = base + (long long)(i + H) * G.pitch;
    const float4 a = ld4(xc + pa), b = ld4(xc + pb);
    const float4 ga = ld4(gc + pa), gb = ld4(gc + pb);
    P[i][0] = make_float2(a.x, b.x);
    P[i][1] = make_float2(a.y, b.y);
    P[i][2] = make_float2(a.z, b.z);
    P[i][3] = make_float2(a.w, b.w);
    Gp[i][0] = make_float2(ga.x, gb.x);
    Gp[i][1] = make_float2(ga.y, gb.y);
    Gp[i][2] = make_float2(ga.z, gb.z);
    Gp[i][3] = make_float2(ga.w, gb.w);
    if (!FULL) {
      mk[i] = __ldg(reinterpret_cast<const unsigned int*>(mask + pa));
      mk[i + H] = __ldg(reinterpret_cast<const unsigned int*>(mask + pb));
    }
  }
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  const float2 q = make_float2(0.25f, 0.25f);
  for (int s = 0; s < ksweeps; ++s) {
    const int par = s & 1;
    edge[par][0][w][lane] = make_float4(P[0][0].x, P[0][1].x, P[0][2].x, P[0][3].x);
    edge[par][1][w][lane] = make_float4(P[H - 1][0].y, P[H - 1][1].y, P[H - 1][2].y, P[H - 1][3].y);
    __syncthreads();
    const float4 above = w > 0 ? edge[par][1][w - 1][lane] : zero;
    const float4 below = w < W - 1 ? edge[par][0][w + 1][lane] : zero;
    // Pair 0's up: (row -1 from the warp above, row H-1 own).
    float2 up[4] = {make_float2(above.x, P[H - 1][0].x), make_float2(above.y, P[H - 1][1].x),
                    make_float2(above.z, P[H - 1][2].x), make_float2(above.w, P[H - 1][3].x)};
    // Pair H-1's down: (row H own, row R from the warp below).
    const float2 dlast[4] = {make_float2(P[0][0].y, below.x), make_float2(P[0][1].y, below.y),
                             make_float2(P[0][2].y, below.z), make_float2(P[0][3].y, below.w)};
#pragma unroll
    for (int i = 0; i < H; ++i) {
      float2 cur[4] = {P[i][0], P[i][1], P[i][2], P[i][3]};
      float2 dn[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) dn[j] = i < H - 1 ? P[i + 1][j] : dlast[j];
      const float2 lf = make_float2(__shfl_up_sync(0xffffffffu, cur[3].x, 1),
                                    __shfl_up_sync(0xffffffffu, cur[3].y, 1));
      const float2 rt = make_float2(__shfl_down_sync(0xffffffffu, cur[0].x, 1),
                                    __shfl_down_sync(0xffffffffu, cur[0].y, 1));
      float2 o[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float2 l = j > 0 ? cur[j - 1] : lf;
        const float2 r = j < 3 ? cur[j + 1] : rt;
        float2 t = __fadd2_rn(Gp[i][j], up[j]);
        t = __fadd2_rn(t, dn[j]);
        t = __fadd2_rn(t, l);
        t = __fadd2_rn(t, r);
        o[j] = __fmul2_rn(t, q);
      }
      if (!FULL) {
        o[0] = pick2(mk[i], mk[i + H], 0x000000ffu, o[0], cur[0]);
        o[1] = pick2(mk[i], mk[i + H], 0x0000ff00u, o[1], cur[1]);
        o[2] = pick2(mk[i], mk[i + H], 0x00ff0000u, o[2], cur[2]);
        o[3] = pick2(mk[i], mk[i + H], 0xff000000u, o[3], cur[3]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        up[j] = cur[j];
        P[i][j] = o[j];
      }
    }
  }
  if (lane >= K / 4 && lane < 32 - K / 4) {
#pragma unroll
    for (int i = 0; i < H; ++i) {
      const int ra = w * R + i, rb = w * R + i + H;  // region rows
      if (ra >= K && ra < W * R - K)
        *reinterpret_cast<float4*>(oc + base + (long long)i * G.pitch) =
            make_float4(P[i][0].x, P[i][1].x, P[i][2].x, P[i][3].x);
      if (rb >= K && rb < W * R - K)
        *reinterpret_cast<float4*>(oc + base + (long long)(i + H) * G.pitch) =
            make_float4(P[i][0].y, P[i][1].y, P[i][2].y, P[i][3].y);
    }
  }
}

template <int R, int W, int K>
__global__ void __launch_bounds__(W * 32)
grid_tbp_kernel(GridGeom G, const uint8_t* __restrict__ mask,
                const float* __restrict__ g, const float* __restrict__ xin,
                float* __restrict__ xout, const uint8_t* __restrict__ active,
                int tiles_x, int ksweeps) {
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
  const float* xc = xin + c * G.plane;
  const float* gc = g + c * G.plane;
  float* oc = xout + c * G.plane;
  if (flag == 2)
    tbp_body<R, W, K, true>(G, mask, gc, xc, oc, base, ksweeps, lane, w, edge);
  else
    tbp_body<R, W, K, false>(G, mask, gc, xc, oc, base, ksweeps, lane, w, edge);
}

namespace {

void no_prepare() {}

template <int R, int W, int K>
void launch_tbp(const GridGeom& G, const uint8_t* mask, const float* g,
                const float* xin, float* xout, const uint8_t* active,
                int tiles_x, int tiles, int ksweeps, cudaStream_t st) {
  grid_tbp_kernel<R, W, K><<<dim3(tiles, 3), W * 32, 0, st>>>(G, mask, g, xin, xout, active,
                                                             tiles_x, ksweeps);
}

template <int R, int W, int K>
TbVariant make_packed(const char* name) {
  TbVariant v;
  v.name = name;
  v.rows_per_thread = R;
  v.warps = W;
  v.depth = K;
  v.tile_h = W * R - 2 * K;
  v.tile_w = 128 - 2 * K;
  v.launch = &launch_tbp<R, W, K>;
  v.prepare = &no_prepare;
  return v;
}

}  // namespace

void append_packed_variants(std::vector<TbVariant>& v) {
  v.push_back(make_packed<16, 8, 8>("p16w8k8"));
  v.push_back(make_packed<16, 8, 16>("p16w8k16"));
  v.push_back(make_packed<8, 16, 16>("p8w16k16"));
  v.push_back(make_packed<12, 10, 16>("p12w10k16"));
  v.push_back(make_packed<8, 12, 8>("p8w12k8"));
}

}  // namespace fpie
