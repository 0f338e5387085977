// Packed temporally blocked tile body shared by the launch-per-block
// kernels (grid_tbp.cu) and the persistent batch kernel (batch.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <type_traits>

#include "common.cuh"

namespace fpie {

// Loads/stores of 4 consecutive state values in the storage type TS, as
// float4 (the arithmetic is always FP32).  FP16/BF16 values are 8 bytes per
// group of 4, so the same 4-aligned indexing keeps every access aligned.
// CG = true reads through L2 only (ld.global.cg): required when other CTAs
// of the same launch wrote the data (the persistent batch kernel).
template <typename TS, bool CG = false>
struct Lanes4;

template <bool CG>
struct Lanes4<float, CG> {
  static __device__ __forceinline__ float4 load(const float* p) {
    return CG ? __ldcg(reinterpret_cast<const float4*>(p)) : ld4(p);
  }
  static __device__ __forceinline__ void store(float* p, float4 v) {
    *reinterpret_cast<float4*>(p) = v;
  }
};

template <bool CG>
struct Lanes4<__half, CG> {
  static __device__ __forceinline__ float4 load(const __half* p) {
    const uint2 u = CG ? __ldcg(reinterpret_cast<const uint2*>(p))
                       : __ldg(reinterpret_cast<const uint2*>(p));
    __half2 a, b;
    memcpy(&a, &u.x, 4);
    memcpy(&b, &u.y, 4);
    const float2 fa = __half22float2(a), fb = __half22float2(b);
    return make_float4(fa.x, fa.y, fb.x, fb.y);
  }
  static __device__ __forceinline__ void store(__half* p, float4 v) {
    const __half2 a = __floats2half2_rn(v.x, v.y), b = __floats2half2_rn(v.z, v.w);
    uint2 u;
    memcpy(&u.x, &a, 4);
    memcpy(&u.y, &b, 4);
    *reinterpret_cast<uint2*>(p) = u;
  }
};

template <bool CG>
struct Lanes4<__nv_bfloat16, CG> {
  static __device__ __forceinline__ float4 load(const __nv_bfloat16* p) {
    const uint2 u = CG ? __ldcg(reinterpret_cast<const uint2*>(p))
                       : __ldg(reinterpret_cast<const uint2*>(p));
    __nv_bfloat162 a, b;
    memcpy(&a, &u.x, 4);
    memcpy(&b, &u.y, 4);
    const float2 fa = __bfloat1622float2(a), fb = __bfloat1622float2(b);
    return make_float4(fa.x, fa.y, fb.x, fb.y);
  }
  static __device__ __forceinline__ void store(__nv_bfloat16* p, float4 v) {
    const __nv_bfloat162 a = __floats2bfloat162_rn(v.x, v.y), b = __floats2bfloat162_rn(v.z, v.w);
    uint2 u;
    memcpy(&u.x, &a, 4);
    memcpy(&u.y, &b, 4);
    *reinterpret_cast<uint2*>(p) = u;
  }
};

__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

__device__ __forceinline__ float2 pick2(uint32_t ma, uint32_t mb, uint32_t bit,
                                        float2 upd, float2 old) {
  return make_float2((ma & bit) ? upd.x : old.x, (mb & bit) ? upd.y : old.y);
}

// Grad pair row i (registers, or this warp's shared-memory copy when GS).
template <int R, bool GS>
__device__ __forceinline__ void tbp_grad(const float2 (&Gp)[GS ? 1 : R / 2][4],
                                         const float2* __restrict__ sg, int i, int lane,
                                         float2 (&gv)[4]) {
  if (GS) {
    const float4* q = reinterpret_cast<const float4*>(sg + ((size_t)i * 32 + lane) * 4);
    const float4 a = q[0], b = q[1];
    gv[0] = make_float2(a.x, a.y);
    gv[1] = make_float2(a.z, a.w);
    gv[2] = make_float2(b.x, b.y);
    gv[3] = make_float2(b.z, b.w);
  } else {
#pragma unroll
    for (int j = 0; j < 4; ++j) gv[j] = Gp[GS ? 0 : i][j];
  }
}

// New values of pair row i from its old value `cur` and the old pairs above
// and below: ((((g + up) + down) + left) + right) * 0.25 per lane, the numpy
// order, with unmasked pixels keeping `cur`.
template <int R, bool FULL>
__device__ __forceinline__ void tbp_update(const float2 (&cur)[4], const float2 (&up)[4],
                                           const float2 (&dn)[4], const float2 (&gv)[4],
                                           const uint32_t (&mk)[R], int i, float2 (&o)[4]) {
  constexpr int H = R / 2;
  const float2 q = make_float2(0.25f, 0.25f);
  const float2 lf = make_float2(__shfl_up_sync(0xffffffffu, cur[3].x, 1),
                                __shfl_up_sync(0xffffffffu, cur[3].y, 1));
  const float2 rt = make_float2(__shfl_down_sync(0xffffffffu, cur[0].x, 1),
                                __shfl_down_sync(0xffffffffu, cur[0].y, 1));
  // The four column groups' chains advance together, one addition step at
  // a time, so that independent packed adds sit next to each other.
  float2 t[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) t[j] = __fadd2_rn(gv[j], up[j]);
#pragma unroll
  for (int j = 0; j < 4; ++j) t[j] = __fadd2_rn(t[j], dn[j]);
#pragma unroll
  for (int j = 0; j < 4; ++j) t[j] = __fadd2_rn(t[j], j > 0 ? cur[j - 1] : lf);
#pragma unroll
  for (int j = 0; j < 4; ++j) t[j] = __fadd2_rn(t[j], j < 3 ? cur[j + 1] : rt);
#pragma unroll
  for (int j = 0; j < 4; ++j) o[j] = __fmul2_rn(t[j], q);
  if (!FULL) {
    o[0] = pick2(mk[i], mk[i + H], 0x000000ffu, o[0], cur[0]);
    o[1] = pick2(mk[i], mk[i + H], 0x0000ff00u, o[1], cur[1]);
    o[2] = pick2(mk[i], mk[i + H], 0x00ff0000u, o[2], cur[2]);
    o[3] = pick2(mk[i], mk[i + H], 0xff000000u, o[3], cur[3]);
  }
}

// One sweep of the strip held in P (pairs of rows i, i+R/2), using edge
// buffer `par`.  FWD visits pair rows 0..H-1 keeping a copy of each old row
// as the next row's "up"; !FWD visits H-1..0 keeping the old row as the
// next row's "down".  In registers a forward sweep leaves each new row where
// the old row above it was, and a backward sweep moves it back, so a
// forward + backward pair needs no register copies at the loop's back edge.
// Either order computes the same values (Jacobi: every update reads old
// values only).
template <int R, int W, bool FULL, bool GS, bool FWD>
__device__ __forceinline__ void tbp_sweep(float2 (&P)[R / 2][4], const float2 (&Gp)[GS ? 1 : R / 2][4],
                                          const uint32_t (&mk)[R], int par, int lane, int w,
                                          float4 (&edge)[2][2][W][32], const float2* __restrict__ sg) {
  constexpr int H = R / 2;
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  edge[par][0][w][lane] = make_float4(P[0][0].x, P[0][1].x, P[0][2].x, P[0][3].x);
  edge[par][1][w][lane] = make_float4(P[H - 1][0].y, P[H - 1][1].y, P[H - 1][2].y, P[H - 1][3].y);
  __syncthreads();
  const float4 above = w > 0 ? edge[par][1][w - 1][lane] : zero;
  const float4 below = w < W - 1 ? edge[par][0][w + 1][lane] : zero;
  // Pair 0's up: (row -1 from the warp above, row H-1 own).
  const float2 ufirst[4] = {make_float2(above.x, P[H - 1][0].x), make_float2(above.y, P[H - 1][1].x),
                            make_float2(above.z, P[H - 1][2].x), make_float2(above.w, P[H - 1][3].x)};
  // Pair H-1's down: (row H own, row R from the warp below).
  const float2 dlast[4] = {make_float2(P[0][0].y, below.x), make_float2(P[0][1].y, below.y),
                           make_float2(P[0][2].y, below.z), make_float2(P[0][3].y, below.w)};
  if (FWD) {
    float2 up[4] = {ufirst[0], ufirst[1], ufirst[2], ufirst[3]};
#pragma unroll
    for (int i = 0; i < H; ++i) {
      const float2 cur[4] = {P[i][0], P[i][1], P[i][2], P[i][3]};
      float2 dn[4], gv[4], o[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) dn[j] = i < H - 1 ? P[i + 1][j] : dlast[j];
      tbp_grad<R, GS>(Gp, sg, i, lane, gv);
      tbp_update<R, FULL>(cur, up, dn, gv, mk, i, o);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        up[j] = cur[j];
        P[i][j] = o[j];
      }
    }
  } else {
    float2 dn[4] = {dlast[0], dlast[1], dlast[2], dlast[3]};
#pragma unroll
    for (int i = H - 1; i >= 0; --i) {
      const float2 cur[4] = {P[i][0], P[i][1], P[i][2], P[i][3]};
      float2 up[4], gv[4], o[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) up[j] = i > 0 ? P[i - 1][j] : ufirst[j];
      tbp_grad<R, GS>(Gp, sg, i, lane, gv);
      tbp_update<R, FULL>(cur, up, dn, gv, mk, i, o);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        dn[j] = cur[j];
        P[i][j] = o[j];
      }
    }
  }
}

// ksweeps packed sweeps of the strip held in P (pairs of rows i, i+R/2),
// grad pairs in Gp (or shared memory sg when GS), mask words in mk:
// forward/backward sweep pairs, then a last forward sweep if ksweeps is odd.
// Sweep s uses edge buffer s & 1, so one barrier per sweep suffices.
template <int R, int W, bool FULL, bool GS>
__device__ __forceinline__ void tbp_sweeps(float2 (&P)[R / 2][4], const float2 (&Gp)[GS ? 1 : R / 2][4],
                                           const uint32_t (&mk)[R], int ksweeps, int lane, int w,
                                           float4 (&edge)[2][2][W][32], const float2* __restrict__ sg) {
  constexpr int H = R / 2;
  // A warp whose strip holds no masked pixel (small paste jobs leave most
  // of a region's strips so) keeps publishing its edge rows and taking part
  // in the barriers, but skips the updates: its values never change.
  if (!FULL) {
    uint32_t any = 0;
#pragma unroll
    for (int i = 0; i < R; ++i) any |= mk[i];
    if (__all_sync(0xffffffffu, any == 0u)) {
      const float4 top = make_float4(P[0][0].x, P[0][1].x, P[0][2].x, P[0][3].x);
      const float4 bot = make_float4(P[H - 1][0].y, P[H - 1][1].y, P[H - 1][2].y, P[H - 1][3].y);
      for (int s = 0; s < ksweeps; ++s) {
        edge[s & 1][0][w][lane] = top;
        edge[s & 1][1][w][lane] = bot;
        __syncthreads();
      }
      return;
    }
  }
  int s = 0;
  for (; s + 2 <= ksweeps; s += 2) {
    tbp_sweep<R, W, FULL, GS, true>(P, Gp, mk, 0, lane, w, edge, sg);
    tbp_sweep<R, W, FULL, GS, false>(P, Gp, mk, 1, lane, w, edge, sg);
  }
  if (s < ksweeps) tbp_sweep<R, W, FULL, GS, true>(P, Gp, mk, 0, lane, w, edge, sg);
}

// ---- pinned-boundary sweeps (FP32 Jacobi on regions holding unmasked pixels)
// The words in mk are code bytes: bit 0 = masked, bit 1 = pinned, i.e.
// unmasked with a masked 4-neighbour.  Only pinned pixels must keep their
// values: every 4-neighbour of a masked pixel is masked or pinned, so what
// the other unmasked ("free") pixels compute never reaches a masked pixel,
// and they are not stored (store_kept).  Selects are then needed only where
// pinned pixels lie.  These are copies of tbp_update / tbp_sweep with
// those selects (the select path above keeps its own code unchanged).

// SEL: select in the column groups j of bit j, or (kRowSel) in every group
// of the pair rows i of the warp-uniform mask rsel (bit i).
constexpr int kRowSel = 16;

template <int R, int SEL>
__device__ __forceinline__ void tbp_update_pin(const float2 (&cur)[4], const float2 (&up)[4],
                                               const float2 (&dn)[4], const float2 (&gv)[4],
                                               const uint32_t (&mk)[R], int i, float2 (&o)[4],
                                               uint32_t rsel) {
  constexpr int H = R / 2;
  const float2 q = make_float2(0.25f, 0.25f);
  const float2 lf = make_float2(__shfl_up_sync(0xffffffffu, cur[3].x, 1),
                                __shfl_up_sync(0xffffffffu, cur[3].y, 1));
  const float2 rt = make_float2(__shfl_down_sync(0xffffffffu, cur[0].x, 1),
                                __shfl_down_sync(0xffffffffu, cur[0].y, 1));
  float2 t[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) t[j] = __fadd2_rn(gv[j], up[j]);
#pragma unroll
  for (int j = 0; j < 4; ++j) t[j] = __fadd2_rn(t[j], dn[j]);
#pragma unroll
  for (int j = 0; j < 4; ++j) t[j] = __fadd2_rn(t[j], j > 0 ? cur[j - 1] : lf);
#pragma unroll
  for (int j = 0; j < 4; ++j) t[j] = __fadd2_rn(t[j], j < 3 ? cur[j + 1] : rt);
#pragma unroll
  for (int j = 0; j < 4; ++j) o[j] = __fmul2_rn(t[j], q);
  if (SEL == kRowSel) {
    if ((rsel >> i) & 1u) {
#pragma unroll
      for (int j = 0; j < 4; ++j) o[j] = pick2(mk[i], mk[i + H], 0x02u << (8 * j), cur[j], o[j]);
    }
  } else {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (SEL & (1 << j)) o[j] = pick2(mk[i], mk[i + H], 0x02u << (8 * j), cur[j], o[j]);
  }
}

template <int R, int W, int SEL, bool FWD>
__device__ __forceinline__ void tbp_sweep_pin(float2 (&P)[R / 2][4], const float2 (&Gp)[R / 2][4],
                                              const uint32_t (&mk)[R], int par, int lane, int w,
                                              float4 (&edge)[2][2][W][32], uint32_t rsel) {
  constexpr int H = R / 2;
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  edge[par][0][w][lane] = make_float4(P[0][0].x, P[0][1].x, P[0][2].x, P[0][3].x);
  edge[par][1][w][lane] = make_float4(P[H - 1][0].y, P[H - 1][1].y, P[H - 1][2].y, P[H - 1][3].y);
  __syncthreads();
  const float4 above = w > 0 ? edge[par][1][w - 1][lane] : zero;
  const float4 below = w < W - 1 ? edge[par][0][w + 1][lane] : zero;
  const float2 ufirst[4] = {make_float2(above.x, P[H - 1][0].x), make_float2(above.y, P[H - 1][1].x),
                            make_float2(above.z, P[H - 1][2].x), make_float2(above.w, P[H - 1][3].x)};
  const float2 dlast[4] = {make_float2(P[0][0].y, below.x), make_float2(P[0][1].y, below.y),
                           make_float2(P[0][2].y, below.z), make_float2(P[0][3].y, below.w)};
  if (FWD) {
    float2 up[4] = {ufirst[0], ufirst[1], ufirst[2], ufirst[3]};
#pragma unroll
    for (int i = 0; i < H; ++i) {
      const float2 cur[4] = {P[i][0], P[i][1], P[i][2], P[i][3]};
      float2 dn[4], o[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) dn[j] = i < H - 1 ? P[i + 1][j] : dlast[j];
      tbp_update_pin<R, SEL>(cur, up, dn, Gp[i], mk, i, o, rsel);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        up[j] = cur[j];
        P[i][j] = o[j];
      }
    }
  } else {
    float2 dn[4] = {dlast[0], dlast[1], dlast[2], dlast[3]};
#pragma unroll
    for (int i = H - 1; i >= 0; --i) {
      const float2 cur[4] = {P[i][0], P[i][1], P[i][2], P[i][3]};
      float2 up[4], o[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) up[j] = i > 0 ? P[i - 1][j] : ufirst[j];
      tbp_update_pin<R, SEL>(cur, up, dn, Gp[i], mk, i, o, rsel);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        dn[j] = cur[j];
        P[i][j] = o[j];
      }
    }
  }
}

// ksweeps pinned-boundary sweeps of the strip in P (forward/backward pairs,
// one barrier per sweep, like tbp_sweeps).  The caller picks SEL per region,
// so that every warp of the CTA runs the same sweep code.  A warp whose
// strip holds no masked pixel only publishes its edges and takes part in
// the barriers; false then (nothing of it needs storing).
template <int R, int W, int SEL>
__device__ __forceinline__ bool tbp_sweeps_pin(float2 (&P)[R / 2][4], const float2 (&Gp)[R / 2][4],
                                               const uint32_t (&mk)[R], int ksweeps, int lane, int w,
                                               float4 (&edge)[2][2][W][32]) {
  constexpr int H = R / 2;
  uint32_t acc = 0;
#pragma unroll
  for (int i = 0; i < R; ++i) acc |= mk[i];
  if (__all_sync(0xffffffffu, (acc & 0x01010101u) == 0u)) {
    const float4 top = make_float4(P[0][0].x, P[0][1].x, P[0][2].x, P[0][3].x);
    const float4 bot = make_float4(P[H - 1][0].y, P[H - 1][1].y, P[H - 1][2].y, P[H - 1][3].y);
    for (int s = 0; s < ksweeps; ++s) {
      edge[s & 1][0][w][lane] = top;
      edge[s & 1][1][w][lane] = bot;
      __syncthreads();
    }
    return false;
  }
  uint32_t rsel = 0;
  if (SEL == kRowSel) {
#pragma unroll
    for (int i = 0; i < H; ++i)
      if ((mk[i] | mk[i + H]) & 0x02020202u) rsel |= 1u << i;
    rsel = __reduce_or_sync(0xffffffffu, rsel);
  }
  int s = 0;
  for (; s + 2 <= ksweeps; s += 2) {
    tbp_sweep_pin<R, W, SEL, true>(P, Gp, mk, 0, lane, w, edge, rsel);
    tbp_sweep_pin<R, W, SEL, false>(P, Gp, mk, 1, lane, w, edge, rsel);
  }
  if (s < ksweeps) tbp_sweep_pin<R, W, SEL, true>(P, Gp, mk, 0, lane, w, edge, rsel);
  return true;
}

// Stores the 4 FP32 state values at p whose pixels are not free (code
// bytes in `word`: masked, or pinned -- a pinned value never changed, so
// storing it is harmless): one vector store when all four are, else
// predicated scalar stores, without branches (a divergent branch per row
// costs more than the stores).
__device__ __forceinline__ void store_kept(float* p, float4 v, uint32_t word) {
  const uint32_t m = (word | (word >> 1)) & 0x01010101u;
  asm volatile(
      "{\n\t"
      ".reg .pred pv, p0, p1, p2, p3;\n\t"
      ".reg .b32 t;\n\t"
      "setp.eq.u32 pv, %5, 16843009;\n\t"
      "@pv st.global.v4.f32 [%0], {%1, %2, %3, %4};\n\t"
      "and.b32 t, %5, 1;\n\t"
      "setp.ne.and.u32 p0, t, 0, !pv;\n\t"
      "and.b32 t, %5, 256;\n\t"
      "setp.ne.and.u32 p1, t, 0, !pv;\n\t"
      "and.b32 t, %5, 65536;\n\t"
      "setp.ne.and.u32 p2, t, 0, !pv;\n\t"
      "and.b32 t, %5, 16777216;\n\t"
      "setp.ne.and.u32 p3, t, 0, !pv;\n\t"
      "@p0 st.global.f32 [%0], %1;\n\t"
      "@p1 st.global.f32 [%0+4], %2;\n\t"
      "@p2 st.global.f32 [%0+8], %3;\n\t"
      "@p3 st.global.f32 [%0+12], %4;\n\t"
      "}"
      :
      : "l"(p), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w), "r"(m)
      : "memory");
}

// ---- red-black order (the reference's OpenMP EquSolver, placed on a grid) --
// A cell's colour is the parity of row + col on the grid; a sweep updates the
// odd cells (the first half of the equation numbering), then the even ones.
// Region origins and every warp's first row are even, and a pair row i holds
// rows i and i + R/2 (same parity), so the cells of column group j in pair
// row i have parity (i + j) % 2: which registers a half-step updates is
// fixed at compile time.  An updated cell reads only cells of the other
// colour, which the half-step leaves alone, so the update is in place and
// its order is free; each update is ((((g + up) + down) + left) + right) *
// 0.25 as in every other kernel.  The valid part of a region shrinks by one
// cell per half-step, so K red-black sweeps need an apron of 2K.
template <int R, int W, bool FULL, bool ODD>
__device__ __forceinline__ void tbp_rb_half(float2 (&P)[R / 2][4], const float2 (&Gp)[R / 2][4],
                                            const uint32_t (&mk)[R], int par, int lane, int w,
                                            float4 (&edge)[2][2][W][32]) {
  constexpr int H = R / 2;
  static_assert(H % 2 == 0, "the two rows of a pair must have the same parity");
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  edge[par][0][w][lane] = make_float4(P[0][0].x, P[0][1].x, P[0][2].x, P[0][3].x);
  edge[par][1][w][lane] = make_float4(P[H - 1][0].y, P[H - 1][1].y, P[H - 1][2].y, P[H - 1][3].y);
  __syncthreads();
  const float4 above = w > 0 ? edge[par][1][w - 1][lane] : zero;
  const float4 below = w < W - 1 ? edge[par][0][w + 1][lane] : zero;
  const float av[4] = {above.x, above.y, above.z, above.w};
  const float bv[4] = {below.x, below.y, below.z, below.w};
  const float2 q = make_float2(0.25f, 0.25f);
#pragma unroll
  for (int i = 0; i < H; ++i) {
    const int j0 = (i + (ODD ? 1 : 0)) & 1;  // column groups j0 and j0 + 2 have this colour
    // The neighbour across the lane boundary: lane-1's group 3 (for j0 = 0)
    // or lane+1's group 0 (for j0 = 1); all lanes take part in the shuffle.
    const float2 src = j0 == 0 ? P[i][3] : P[i][0];
    const float2 nb = j0 == 0 ? make_float2(__shfl_up_sync(0xffffffffu, src.x, 1),
                                            __shfl_up_sync(0xffffffffu, src.y, 1))
                              : make_float2(__shfl_down_sync(0xffffffffu, src.x, 1),
                                            __shfl_down_sync(0xffffffffu, src.y, 1));
    float2 up[2], dn[2], l[2], r[2], t[2];
#pragma unroll
    for (int jj = 0; jj < 2; ++jj) {
      const int j = j0 + 2 * jj;
      up[jj] = i > 0 ? P[i - 1][j] : make_float2(av[j], P[H - 1][j].x);
      dn[jj] = i < H - 1 ? P[i + 1][j] : make_float2(P[0][j].y, bv[j]);
      l[jj] = j > 0 ? P[i][j - 1] : nb;
      r[jj] = j < 3 ? P[i][j + 1] : nb;
    }
    // The two column groups' chains advance together, one step at a time.
#pragma unroll
    for (int jj = 0; jj < 2; ++jj) t[jj] = __fadd2_rn(Gp[i][j0 + 2 * jj], up[jj]);
#pragma unroll
    for (int jj = 0; jj < 2; ++jj) t[jj] = __fadd2_rn(t[jj], dn[jj]);
#pragma unroll
    for (int jj = 0; jj < 2; ++jj) t[jj] = __fadd2_rn(t[jj], l[jj]);
#pragma unroll
    for (int jj = 0; jj < 2; ++jj) t[jj] = __fadd2_rn(t[jj], r[jj]);
#pragma unroll
    for (int jj = 0; jj < 2; ++jj) {
      const int j = j0 + 2 * jj;
      const float2 o = __fmul2_rn(t[jj], q);
      P[i][j] = FULL ? o : pick2(mk[i], mk[i + H], 0xffu << (8 * j), o, P[i][j]);
    }
  }
}

// ksweeps red-black sweeps (odd half, even half) of the strip in P.
template <int R, int W, bool FULL>
__device__ __forceinline__ void tbp_rb_sweeps(float2 (&P)[R / 2][4], const float2 (&Gp)[R / 2][4],
                                              const uint32_t (&mk)[R], int ksweeps, int lane, int w,
                                              float4 (&edge)[2][2][W][32]) {
  constexpr int H = R / 2;
  if (!FULL) {
    uint32_t any = 0;
#pragma unroll
    for (int i = 0; i < R; ++i) any |= mk[i];
    if (__all_sync(0xffffffffu, any == 0u)) {  // nothing to update: edges and barriers only
      const float4 top = make_float4(P[0][0].x, P[0][1].x, P[0][2].x, P[0][3].x);
      const float4 bot = make_float4(P[H - 1][0].y, P[H - 1][1].y, P[H - 1][2].y, P[H - 1][3].y);
      for (int h = 0; h < 2 * ksweeps; ++h) {
        edge[h & 1][0][w][lane] = top;
        edge[h & 1][1][w][lane] = bot;
        __syncthreads();
      }
      return;
    }
  }
  for (int s = 0; s < ksweeps; ++s) {
    tbp_rb_half<R, W, FULL, true>(P, Gp, mk, 0, lane, w, edge);
    tbp_rb_half<R, W, FULL, false>(P, Gp, mk, 1, lane, w, edge);
  }
}

// TS: storage type of the swept state (float for the plain solver; __half
// or __nv_bfloat16 for the correction of the mixed form).  zero_start: the
// state starts at 0 instead of being loaded (first inner launch of a
// refinement cycle).
// GS: the grad pairs live in shared memory (sg: this warp's H x 32 x 4
// float2, i.e. W*R*32*16 bytes per CTA, dynamic) instead of registers,
// freeing 4R registers per thread for taller regions.
// RB: red-black sweeps (K is then the apron, 2 x the sweeps per launch).
// PSEL >= 0 (with !FULL, FP32 Jacobi sweeps): `mask` is the code plane,
// the sweeps are tbp_sweeps_pin<..., PSEL> and free pixels are not stored;
// both state buffers must hold the same values at unmasked pixels, which
// then never change.
template <int R, int W, int K, bool FULL, typename TS, bool ZS, bool CG = false, bool GS = false,
          bool RB = false, int PSEL = -1>
__device__ __forceinline__ void tbp_body(const GridGeom& G, const uint8_t* __restrict__ mask,
                                         const float* __restrict__ gc,
                                         const TS* __restrict__ xc, TS* __restrict__ oc,
                                         long long base, int ksweeps,
                                         int lane, int w, float4 (&edge)[2][2][W][32],
                                         float2* __restrict__ sg = nullptr) {
  constexpr int H = R / 2;
  float2 P[H][4], Gp[GS ? 1 : H][4];
  uint32_t mk[R];
#pragma unroll
  for (int i = 0; i < H; ++i) {
    const long long pa = base + (long long)i * G.pitch;
    const long long pb = base + (long long)(i + H) * G.pitch;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 a = ZS ? z4 : Lanes4<TS, CG>::load(xc + pa);
    const float4 b = ZS ? z4 : Lanes4<TS, CG>::load(xc + pb);
    // In the persistent batch kernel (CG) "g" may be the residual another CTA
    // wrote during this launch, so it is read through L2 as well.
    const float4 ga = Lanes4<float, CG>::load(gc + pa), gb = Lanes4<float, CG>::load(gc + pb);
    P[i][0] = make_float2(a.x, b.x);
    P[i][1] = make_float2(a.y, b.y);
    P[i][2] = make_float2(a.z, b.z);
    P[i][3] = make_float2(a.w, b.w);
    if (GS) {
      float2* q = sg + ((size_t)i * 32 + lane) * 4;
      *reinterpret_cast<float4*>(q) = make_float4(ga.x, gb.x, ga.y, gb.y);
      *reinterpret_cast<float4*>(q + 2) = make_float4(ga.z, gb.z, ga.w, gb.w);
    } else {
      Gp[GS ? 0 : i][0] = make_float2(ga.x, gb.x);
      Gp[GS ? 0 : i][1] = make_float2(ga.y, gb.y);
      Gp[GS ? 0 : i][2] = make_float2(ga.z, gb.z);
      Gp[GS ? 0 : i][3] = make_float2(ga.w, gb.w);
    }
    if (!FULL) {
      mk[i] = __ldg(reinterpret_cast<const unsigned int*>(mask + pa));
      mk[i + H] = __ldg(reinterpret_cast<const unsigned int*>(mask + pb));
    }
  }
  if constexpr (PSEL >= 0 && !FULL) {
    static_assert(!RB && !GS && std::is_same<TS, float>::value,
                  "pinned-boundary sweeps: FP32 Jacobi, grad in registers");
    if (!tbp_sweeps_pin<R, W, PSEL>(P, Gp, mk, ksweeps, lane, w, edge)) return;
    if (lane >= K / 4 && lane < 32 - K / 4) {
#pragma unroll
      for (int i = 0; i < H; ++i) {
        const int ra = w * R + i, rb = w * R + i + H;  // region rows
        if (ra >= K && ra < W * R - K)
          store_kept(oc + base + (long long)i * G.pitch,
                     make_float4(P[i][0].x, P[i][1].x, P[i][2].x, P[i][3].x), mk[i]);
        if (rb >= K && rb < W * R - K)
          store_kept(oc + base + (long long)(i + H) * G.pitch,
                     make_float4(P[i][0].y, P[i][1].y, P[i][2].y, P[i][3].y), mk[i + H]);
      }
    }
    return;
  } else if constexpr (RB) {
    static_assert(!GS, "red-black sweeps keep grad in registers");
    tbp_rb_sweeps<R, W, FULL>(P, Gp, mk, ksweeps, lane, w, edge);
  } else {
    tbp_sweeps<R, W, FULL, GS>(P, Gp, mk, ksweeps, lane, w, edge, sg);
  }
  if (lane >= K / 4 && lane < 32 - K / 4) {
#pragma unroll
    for (int i = 0; i < H; ++i) {
      const int ra = w * R + i, rb = w * R + i + H;  // region rows
      if (ra >= K && ra < W * R - K)
        Lanes4<TS>::store(oc + base + (long long)i * G.pitch,
                          make_float4(P[i][0].x, P[i][1].x, P[i][2].x, P[i][3].x));
      if (rb >= K && rb < W * R - K)
        Lanes4<TS>::store(oc + base + (long long)(i + H) * G.pitch,
                          make_float4(P[i][0].y, P[i][1].y, P[i][2].y, P[i][3].y));
    }
  }
}

// First inner launch of a refinement cycle with the refine step fused in:
// loads x (FP32) and, when HASE, the previous cycle's correction e, forms
// xn = x + e and the FP32 residual r = -(4xn - g - up - down - left - right)
// (the refine kernel's formula, so values are identical) on the whole
// region in registers -- the outermost ring, whose neighbours lie outside,
// gets a wrong r, which like every region-border error cannot reach the
// tile in K sweeps -- writes xn (if HASE) and r for the tile interior, then
// runs ksweeps correction sweeps from e = 0 and writes e for the tile.
template <int R, int W, int K, bool FULL, typename TS, bool HASE, bool CG = false>
__device__ __forceinline__ void tbp_fold_body(const GridGeom& G, const uint8_t* __restrict__ mask,
                                              const float* __restrict__ gc,
                                              const float* __restrict__ xin,
                                              const TS* __restrict__ elast,
                                              float* __restrict__ xout, float* __restrict__ rout,
                                              TS* __restrict__ eout, long long base, int ksweeps,
                                              int lane, int w, float4 (&edge)[2][2][W][32]) {
  constexpr int H = R / 2;
  float2 P[H][4], Gp[H][4];
  uint32_t mk[R];
#pragma unroll
  for (int i = 0; i < H; ++i) {
    const long long pa = base + (long long)i * G.pitch;
    const long long pb = base + (long long)(i + H) * G.pitch;
    float4 a = Lanes4<float, CG>::load(xin + pa), b = Lanes4<float, CG>::load(xin + pb);
    if (HASE) {
      const float4 ea = Lanes4<TS, CG>::load(elast + pa), eb = Lanes4<TS, CG>::load(elast + pb);
      a = make_float4(__fadd_rn(a.x, ea.x), __fadd_rn(a.y, ea.y), __fadd_rn(a.z, ea.z), __fadd_rn(a.w, ea.w));
      b = make_float4(__fadd_rn(b.x, eb.x), __fadd_rn(b.y, eb.y), __fadd_rn(b.z, eb.z), __fadd_rn(b.w, eb.w));
    }
    const float4 ga = ld4(gc + pa), gb = ld4(gc + pb);
    P[i][0] = make_float2(a.x, b.x);
    P[i][1] = make_float2(a.y, b.y);
    P[i][2] = make_float2(a.z, b.z);
    P[i][3] = make_float2(a.w, b.w);
    Gp[i][0] = make_float2(ga.x, gb.x);
    Gp[i][1] = make_float2(ga.y, gb.y);
    Gp[i][2] = make_float2(ga.z, gb.z);
    Gp[i][3] = make_float2(ga.w, gb.w);
    mk[i] = __ldg(reinterpret_cast<const unsigned int*>(mask + pa));
    mk[i + H] = __ldg(reinterpret_cast<const unsigned int*>(mask + pb));
  }
  // Residual of xn (edge slot 1; the sweeps below start with slot 0).
  {
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    edge[1][0][w][lane] = make_float4(P[0][0].x, P[0][1].x, P[0][2].x, P[0][3].x);
    edge[1][1][w][lane] = make_float4(P[H - 1][0].y, P[H - 1][1].y, P[H - 1][2].y, P[H - 1][3].y);
    __syncthreads();
    const float4 above = w > 0 ? edge[1][1][w - 1][lane] : zero;
    const float4 below = w < W - 1 ? edge[1][0][w + 1][lane] : zero;
    float2 up[4] = {make_float2(above.x, P[H - 1][0].x), make_float2(above.y, P[H - 1][1].x),
                    make_float2(above.z, P[H - 1][2].x), make_float2(above.w, P[H - 1][3].x)};
    const float2 dlast[4] = {make_float2(P[0][0].y, below.x), make_float2(P[0][1].y, below.y),
                             make_float2(P[0][2].y, below.z), make_float2(P[0][3].y, below.w)};
#pragma unroll
    for (int i = 0; i < H; ++i) {
      const float2 cur[4] = {P[i][0], P[i][1], P[i][2], P[i][3]};
      float2 dn[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) dn[j] = i < H - 1 ? P[i + 1][j] : dlast[j];
      const float2 lf = make_float2(__shfl_up_sync(0xffffffffu, cur[3].x, 1),
                                    __shfl_up_sync(0xffffffffu, cur[3].y, 1));
      const float2 rt = make_float2(__shfl_down_sync(0xffffffffu, cur[0].x, 1),
                                    __shfl_down_sync(0xffffffffu, cur[0].y, 1));
      // grid_res in packed form, the same IEEE operations in the same order:
      // 4x - g as one fused multiply-add (4x is exact, so the single rounding
      // equals grid_res's rounding of the subtraction), then four additions
      // of the negated neighbours (a - b is a + (-b)).
      const float2 four = make_float2(4.0f, 4.0f);
      float2 t[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) t[j] = __ffma2_rn(cur[j], four, neg2(Gp[i][j]));
#pragma unroll
      for (int j = 0; j < 4; ++j) t[j] = __fadd2_rn(t[j], neg2(up[j]));
#pragma unroll
      for (int j = 0; j < 4; ++j) t[j] = __fadd2_rn(t[j], neg2(dn[j]));
#pragma unroll
      for (int j = 0; j < 4; ++j) t[j] = __fadd2_rn(t[j], neg2(j > 0 ? cur[j - 1] : lf));
#pragma unroll
      for (int j = 0; j < 4; ++j) t[j] = __fadd2_rn(t[j], neg2(j < 3 ? cur[j + 1] : rt));
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const uint32_t bit = 0xffu << (8 * j);
        up[j] = cur[j];
        // the residual becomes the sweeps' right-hand side
        Gp[i][j] = make_float2((mk[i] & bit) ? -t[j].x : 0.0f, (mk[i + H] & bit) ? -t[j].y : 0.0f);
      }
    }
  }
  if (lane >= K / 4 && lane < 32 - K / 4) {
#pragma unroll
    for (int i = 0; i < H; ++i) {
      const int ra = w * R + i, rb = ra + H;
      const long long pa = base + (long long)i * G.pitch, pb = base + (long long)(i + H) * G.pitch;
      if (ra >= K && ra < W * R - K) {
        if (HASE && mk[i])
          *reinterpret_cast<float4*>(xout + pa) = make_float4(P[i][0].x, P[i][1].x, P[i][2].x, P[i][3].x);
        *reinterpret_cast<float4*>(rout + pa) =
            make_float4(Gp[i][0].x, Gp[i][1].x, Gp[i][2].x, Gp[i][3].x);
      }
      if (rb >= K && rb < W * R - K) {
        if (HASE && mk[i + H])
          *reinterpret_cast<float4*>(xout + pb) = make_float4(P[i][0].y, P[i][1].y, P[i][2].y, P[i][3].y);
        *reinterpret_cast<float4*>(rout + pb) =
            make_float4(Gp[i][0].y, Gp[i][1].y, Gp[i][2].y, Gp[i][3].y);
      }
    }
  }
#pragma unroll
  for (int i = 0; i < H; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) P[i][j] = make_float2(0.f, 0.f);
  tbp_sweeps<R, W, FULL, false>(P, Gp, mk, ksweeps, lane, w, edge, nullptr);
  if (lane >= K / 4 && lane < 32 - K / 4) {
#pragma unroll
    for (int i = 0; i < H; ++i) {
      const int ra = w * R + i, rb = ra + H;
      if (ra >= K && ra < W * R - K)
        Lanes4<TS>::store(eout + base + (long long)i * G.pitch,
                          make_float4(P[i][0].x, P[i][1].x, P[i][2].x, P[i][3].x));
      if (rb >= K && rb < W * R - K)
        Lanes4<TS>::store(eout + base + (long long)(i + H) * G.pitch,
                          make_float4(P[i][0].y, P[i][1].y, P[i][2].y, P[i][3].y));
    }
  }
}

}  // namespace fpie
