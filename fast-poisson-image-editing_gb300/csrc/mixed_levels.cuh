// Level schedule of the mixed forms and the per-tile refine step, shared by
// the batched kernel (batch.cu) and the dependency-flow kernel
// (grid_flow.cu).
#pragma once

#include "common.cuh"
#include "grid_tbp.cuh"

namespace fpie {

// Level schedule of the mixed forms for a launch of S sweeps with depth K
// (P = 64 / K launches per full cycle): every cycle of up to 64 sweeps is
// ceil(len / K) inner levels, the first of which folds the previous
// cycle's correction into x and recomputes the residual (tbp_fold_body);
// one flush level at the end folds the last correction.  The x buffer
// flips once per fold: C = ceil(S / 64) times per launch.
struct MixedLevel {
  int type;   // 0 = fold + first inner, 1 = inner, 2 = flush
  int k;      // sweeps of an inner level
  int pos;    // index within the cycle
  int cycle;
  int nlast;  // levels of the last cycle
};

__host__ __device__ inline int mixed_levels(int S, int K) {
  const int P = 64 / K, C = (S + 63) / 64;
  const int nlast = (S - 64 * (C - 1) + K - 1) / K;
  return (C - 1) * P + nlast + 1;
}

__host__ __device__ inline MixedLevel mixed_level(int z, int S, int K) {
  const int P = 64 / K, C = (S + 63) / 64, nfull = C - 1;
  const int nlast = (S - 64 * nfull + K - 1) / K;
  MixedLevel L{0, 0, 0, 0, nlast};
  if (z == nfull * P + nlast) {
    L.type = 2;
    L.cycle = C;
    return L;
  }
  int len = 64;
  if (z < nfull * P) {
    L.cycle = z / P;
    L.pos = z % P;
  } else {
    L.cycle = nfull;
    L.pos = z - nfull * P;
    len = S - 64 * nfull;
  }
  L.k = len - L.pos * K < K ? len - L.pos * K : K;
  L.type = L.pos == 0 ? 0 : 1;
  return L;
}

template <typename TS>
__device__ __forceinline__ float4 ld4cg_any(const TS* p) {
  return Lanes4<TS, true>::load(p);
}

// One channel of one tile interior: optional fold x_out = x_in + e, then
// the FP32 residual r = g + sum(neighbours) - 4x of the (folded) state.
// Reads go through L2 (other CTAs wrote x and e in this launch).
template <typename TS>
__device__ void refine_tile(const GridGeom& G, const uint8_t* __restrict__ mask,
                            const float* __restrict__ gc, const float* xin, const TS* e,
                            float* xout, float* r, int r0, int c0, int th, int tw) {
  const int gpr = tw / 4;
  for (int q = threadIdx.x; q < th * gpr; q += blockDim.x) {
    const int i = r0 + q / gpr, j = c0 + 4 * (q % gpr);
    if (i >= G.n || j >= G.m) continue;
    const long long p = G.at(i, j);
    const uint32_t mk = *reinterpret_cast<const uint32_t*>(mask + p);
    float4 ce = __ldcg(reinterpret_cast<const float4*>(xin + p));
    float4 up = __ldcg(reinterpret_cast<const float4*>(xin + p - G.pitch));
    float4 dn = __ldcg(reinterpret_cast<const float4*>(xin + p + G.pitch));
    float lf = __ldcg(xin + p - 1), rt = __ldcg(xin + p + 4);
    if (e) {
      const float4 ec = ld4cg_any(e + p), eu = ld4cg_any(e + p - G.pitch), ed = ld4cg_any(e + p + G.pitch);
      const float4 el = ld4cg_any(e + p - 4), er = ld4cg_any(e + p + 4);
      ce = make_float4(__fadd_rn(ce.x, ec.x), __fadd_rn(ce.y, ec.y), __fadd_rn(ce.z, ec.z), __fadd_rn(ce.w, ec.w));
      up = make_float4(__fadd_rn(up.x, eu.x), __fadd_rn(up.y, eu.y), __fadd_rn(up.z, eu.z), __fadd_rn(up.w, eu.w));
      dn = make_float4(__fadd_rn(dn.x, ed.x), __fadd_rn(dn.y, ed.y), __fadd_rn(dn.z, ed.z), __fadd_rn(dn.w, ed.w));
      lf = __fadd_rn(lf, el.w);
      rt = __fadd_rn(rt, er.x);
      if (mk) *reinterpret_cast<float4*>(xout + p) = ce;
    }
    const float4 gv = __ldg(reinterpret_cast<const float4*>(gc + p));
    const float xv[6] = {lf, ce.x, ce.y, ce.z, ce.w, rt};
    const float g4[4] = {gv.x, gv.y, gv.z, gv.w}, u4[4] = {up.x, up.y, up.z, up.w},
                d4[4] = {dn.x, dn.y, dn.z, dn.w};
    float rr[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const bool on = (mk >> (8 * k)) & 0xffu;
      rr[k] = on ? -grid_res(xv[k + 1], g4[k], u4[k], d4[k], xv[k], xv[k + 2]) : 0.0f;
    }
    if (r) *reinterpret_cast<float4*>(r + p) = make_float4(rr[0], rr[1], rr[2], rr[3]);
  }
}

}  // namespace fpie
