// Resident grid sweep: the whole step in one cooperative launch.
//
// For grids small enough that every (tile, channel) region fits one CTA per
// SM -- square800 is 7 x 7 tiles x 3 channels = 147 CTAs on 152 SMs -- each
// CTA loads its 128x128 region (120x120 tile plus a K = 4 apron) once and
// keeps it in registers for all sweeps of the step, in the packed row-pair
// layout of grid_tbp.cuh.  Every K sweeps it
//   1. writes its tile interior to the period's buffer (two buffers used
//      alternately: period p writes buffer (p+1) & 1),
//   2. publishes its period count (flag, after a fence),
//   3. waits until each of its active neighbour tiles (same channel, up to
//      8) has published the same period -- a bounded spin; past the limit
//      it records an error and the whole grid returns,
//   4. reloads only its apron (rows/columns within K of the region border)
//      from that buffer, through L2.
// Neighbour-to-neighbour waits replace a grid-wide barrier.  Two buffers
// suffice: a CTA cannot start period p+2 (which overwrites buffer p & 1)
// before its neighbours published p+1, i.e. before they finished reading
// their period-p aprons.  Inactive tiles (no masked pixel) never change, so
// their pixels are identical in both buffers and nobody waits for them.
// The launch is cooperative, so all CTAs are co-resident and every wait
// ends unless a CTA faults; the spin limit bounds even that case.
//
// Arithmetic per pixel is the other sweep kernels' (numpy order): results
// are bit-identical.
#include "common.cuh"
#include "grid_resident.cuh"

namespace fpie {

namespace {

constexpr int kR = 16, kW = 8, kK = 4, kH = kR / 2;
constexpr int kTH = kW * kR - 2 * kK;  // 120
constexpr int kTW = 128 - 2 * kK;      // 120

struct ResidentArgs {
  GridGeom G;
  const uint8_t* mask;
  const float* g;
  float* buf[2];            // buf[0] holds the step's initial state
  const int2* ctas;         // per CTA: (tile index, flag 1/2)
  const int* nbrs;          // per CTA: 8 neighbour CTA indices (-1 = none)
  int tiles_x;
  int sweeps;
  int* period;              // per CTA: periods published
  int* error;
  long long spin_limit;
};

__device__ __forceinline__ float4 ldcg4(const float* p) {
  return __ldcg(reinterpret_cast<const float4*>(p));
}

template <bool FULL>
__device__ __forceinline__ void resident_body(const ResidentArgs& A, int cta, int c,
                                              long long base, int lane, int w,
                                              float4 (&edge)[2][2][kW][32], int* s_stop) {
  const GridGeom& G = A.G;
  const float* gc = A.g + c * G.plane;
  float2 P[kH][4], Gp[kH][4];
  uint32_t mk[kR];
#pragma unroll
  for (int i = 0; i < kH; ++i) {
    const long long pa = base + (long long)i * G.pitch, pb = base + (long long)(i + kH) * G.pitch;
    const float4 a = ldcg4(A.buf[0] + c * G.plane + pa), b = ldcg4(A.buf[0] + c * G.plane + pb);
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
      mk[i] = __ldg(reinterpret_cast<const unsigned int*>(A.mask + pa));
      mk[i + kH] = __ldg(reinterpret_cast<const unsigned int*>(A.mask + pb));
    }
  }
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  const float2 q = make_float2(0.25f, 0.25f);
  const int periods = (A.sweeps + kK - 1) / kK;
  const bool lane_apron = lane < kK / 4 || lane >= 32 - kK / 4;
  int s_total = 0;
  for (int per = 0; per < periods; ++per) {
    const int ks = min(kK, A.sweeps - per * kK);
    for (int s = 0; s < ks; ++s, ++s_total) {
      const int par = s_total & 1;
      edge[par][0][w][lane] = make_float4(P[0][0].x, P[0][1].x, P[0][2].x, P[0][3].x);
      edge[par][1][w][lane] = make_float4(P[kH - 1][0].y, P[kH - 1][1].y, P[kH - 1][2].y, P[kH - 1][3].y);
      __syncthreads();
      const float4 above = w > 0 ? edge[par][1][w - 1][lane] : zero;
      const float4 below = w < kW - 1 ? edge[par][0][w + 1][lane] : zero;
      float2 up[4] = {make_float2(above.x, P[kH - 1][0].x), make_float2(above.y, P[kH - 1][1].x),
                      make_float2(above.z, P[kH - 1][2].x), make_float2(above.w, P[kH - 1][3].x)};
      const float2 dlast[4] = {make_float2(P[0][0].y, below.x), make_float2(P[0][1].y, below.y),
                               make_float2(P[0][2].y, below.z), make_float2(P[0][3].y, below.w)};
#pragma unroll
      for (int i = 0; i < kH; ++i) {
        float2 cur[4] = {P[i][0], P[i][1], P[i][2], P[i][3]};
        float2 dn[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) dn[j] = i < kH - 1 ? P[i + 1][j] : dlast[j];
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
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const uint32_t bit = 0xffu << (8 * j);
            o[j] = make_float2((mk[i] & bit) ? o[j].x : cur[j].x, (mk[i + kH] & bit) ? o[j].y : cur[j].y);
          }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          up[j] = cur[j];
          P[i][j] = o[j];
        }
      }
    }
    // Publish the tile interior of this period.
    float* out = A.buf[(per + 1) & 1] + c * G.plane;
    if (!lane_apron) {
#pragma unroll
      for (int i = 0; i < kH; ++i) {
        const int ra = w * kR + i, rb = ra + kH;
        if (ra >= kK && ra < kW * kR - kK)
          *reinterpret_cast<float4*>(out + base + (long long)i * G.pitch) =
              make_float4(P[i][0].x, P[i][1].x, P[i][2].x, P[i][3].x);
        if (rb >= kK && rb < kW * kR - kK)
          *reinterpret_cast<float4*>(out + base + (long long)(i + kH) * G.pitch) =
              make_float4(P[i][0].y, P[i][1].y, P[i][2].y, P[i][3].y);
      }
    }
    if (per == periods - 1) break;  // the last period needs no apron
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicExch(A.period + cta, per + 1);
    // Wait for the active neighbours' interiors of this period.
    if (threadIdx.x < 8) {
      const int nb = A.nbrs[cta * 8 + threadIdx.x];
      if (nb >= 0) {
        long long spins = 0;
        while (*(volatile int*)(A.period + nb) < per + 1) {
          if (*(volatile int*)A.error) break;
          if (++spins > A.spin_limit) {
            atomicExch(A.error, 1);
            break;
          }
          __nanosleep(64);
        }
      }
      __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) *s_stop = *(volatile int*)A.error;
    __syncthreads();
    if (*s_stop) return;
    // Reload the apron (rows or columns within K of the region border).
#pragma unroll
    for (int i = 0; i < kH; ++i) {
      const int ra = w * kR + i, rb = ra + kH;
      const bool apa = lane_apron || ra < kK || ra >= kW * kR - kK;
      const bool apb = lane_apron || rb < kK || rb >= kW * kR - kK;
      if (apa) {
        const float4 v = ldcg4(out + base + (long long)i * G.pitch);
        P[i][0].x = v.x;
        P[i][1].x = v.y;
        P[i][2].x = v.z;
        P[i][3].x = v.w;
      }
      if (apb) {
        const float4 v = ldcg4(out + base + (long long)(i + kH) * G.pitch);
        P[i][0].y = v.x;
        P[i][1].y = v.y;
        P[i][2].y = v.z;
        P[i][3].y = v.w;
      }
    }
  }
}

__global__ void __launch_bounds__(kW * 32)
grid_resident_kernel(ResidentArgs A) {
  __shared__ float4 edge[2][2][kW][32];
  __shared__ int s_stop;
  const int cta = blockIdx.x;
  const int2 tf = A.ctas[cta];
  const int tile = tf.x / 3, c = tf.x - 3 * tile;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int ty = tile / A.tiles_x, tx = tile - ty * A.tiles_x;
  const long long base = A.G.at(ty * kTH - kK + w * kR, tx * kTW - kK + 4 * lane);
  if (tf.y == 2)
    resident_body<true>(A, cta, c, base, lane, w, edge, &s_stop);
  else
    resident_body<false>(A, cta, c, base, lane, w, edge, &s_stop);
}

}  // namespace

int resident_tile_h() { return kTH; }
int resident_tile_w() { return kTW; }
int resident_depth() { return kK; }

int resident_max_ctas() {
  int dev = 0, sms = 0, occ = 0;
  FPIE_CUDA(cudaGetDevice(&dev));
  FPIE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  FPIE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, grid_resident_kernel, kW * 32, 0));
  return sms * occ;
}

void launch_resident(const GridGeom& G, const uint8_t* mask, const float* g, float* buf0,
                     float* buf1, const int2* ctas, const int* nbrs, int nctas, int tiles_x,
                     int sweeps, int* period, int* error, long long spin_limit, cudaStream_t st) {
  ResidentArgs a{G, mask, g, {buf0, buf1}, ctas, nbrs, tiles_x, sweeps, period, error, spin_limit};
  void* args[] = {&a};
  FPIE_CUDA(cudaLaunchCooperativeKernel((const void*)grid_resident_kernel, dim3(nctas),
                                        dim3(kW * 32), args, 0, st));
}

}  // namespace fpie
