// correction.cuh — the matrix-free correction r = b(x) − Ã·x of one vertex in FP32, with the
// reference's residual of x from the same incidence sums; positions as FP32 hi/lo pairs.
//
// With the projections d_e = ℓ_e·(x_a − x_b)/‖x_a − x_b‖ at x (DistanceTerm.cpp:94-102), for a
// free vertex v
//   t_v = m_v/h²·(x_v − x̂_v) + Σ_e κ_e·((x_v − x_o) − d_e) + Σ_s (−k_s w_v)·(w_sᵀx)
// is the reference's residual force (Integrator.cpp:230-263: r_v = ‖t_v‖ / m_v), and
//   r_v = −(m_v/h²·(x_v − x̂_v) + Σ_e κ_e·((x_v − x_o) − d_e)) + Σ_s (−k_s w_v)·(w_sᵀx)
// is b − Ã·x for the reference's b and Ã (Assembler.cpp:94-332), provided pinned vertices enter
// the matrix terms at their pin positions q (pin elimination moves them into b; the bend part of
// that is the constant bending RHS). The projection is odd in x_a − x_b, so each edge is seen
// from v as (x_v − x_o).
#pragma once

#include "device.cuh"

namespace pdg {

// FP64 value as an FP32 pair with hi + lo = v to ~2⁻⁴⁸ relative.
__device__ __forceinline__ void split(double v, float& hi, float& lo) {
  hi = static_cast<float>(v);
  lo = static_cast<float>(v - static_cast<double>(hi));
}

// Difference of two positions held as hi/lo pairs, to FP32 rounding of the result.
__device__ __forceinline__ float3 diffHL(float4 ah, float4 al, float4 bh, float4 bl) {
  return make_float3((ah.x - bh.x) + (al.x - bl.x), (ah.y - bh.y) + (al.y - bl.y), (ah.z - bh.z) + (al.z - bl.z));
}

// Pin position q_u as the hi/lo pair the host split it into.
__device__ __forceinline__ void pinHL(const InstanceDev& I, int u, float4& h, float4& l) {
  h = __ldg(I.qhl + 2 * u);
  l = __ldg(I.qhl + 2 * u + 1);
}

// (hi, lo) + d as a renormalised pair: Knuth's two-sum of hi and d, then a fast two-sum.
__device__ __forceinline__ void addHL(float& hi, float& lo, float d) {
  const float s = hi + d;
  const float bb = s - hi;
  const float e = (hi - (s - bb)) + (d - bb);
  const float l = lo + e;
  hi = s + l;
  lo = l - (hi - s);
}

// Incidence sums of one vertex, accumulated by the lanes of a group and then reduced.
struct CorrectionSums {
  float a[3] = {0.f, 0.f, 0.f};  // mass + edge terms of t
  float f[3] = {0.f, 0.f, 0.f};  // bend terms of t
  float p[3] = {0.f, 0.f, 0.f};  // what the matrix adds to f − a by seeing pinned vertices at q

  // Edge incidences [e0, e1) of E (other vertex | pinned << 31, ℓ, κ as FP32 bits) and bend
  // incidences [s0, s1) of S (a, b, c | pinned << 31, (−k)·w_v bits); lane gl of G takes every
  // G-th. X holds positions as (hi, lo) float4 pairs per vertex; with CG they are read from L2
  // (other CTAs write them).
  template <bool CG = false>
  __device__ __forceinline__ void accumulate(const InstanceDev& I, const int4* E, int e0, int e1, const int4* S,
                                             int s0, int s1, const float4* X, float4 vh, float4 vl, int gl, int G) {
    auto X_ = [&](int i) { return CG ? __ldcg(X + i) : X[i]; };
    for (int q = e0 + gl; q < e1; q += G) {
      const int4 e = E[q];
      const int o = e.x & 0x7fffffff;
      const float rest = __int_as_float(e.y), kap = __int_as_float(e.z);
      const float3 rel = diffHL(vh, vl, X_(2 * o), X_(2 * o + 1));  // x_v − x_o
      const float len = sqrtf(rel.x * rel.x + rel.y * rel.y + rel.z * rel.z);
      float dx = 0.f, dy = 0.f, dz = 0.f;
      if (!(len <= 1e-12f)) {
        const float sc = rest / len;
        dx = rel.x * sc;
        dy = rel.y * sc;
        dz = rel.z * sc;
      }
      a[0] = fmaf(kap, rel.x - dx, a[0]);
      a[1] = fmaf(kap, rel.y - dy, a[1]);
      a[2] = fmaf(kap, rel.z - dz, a[2]);
      if (e.x < 0) {  // pinned neighbour: the matrix sees it at q
        float4 qh, ql;
        pinHL(I, o, qh, ql);
        const float3 relq = diffHL(vh, vl, qh, ql);
        p[0] = fmaf(kap, relq.x - rel.x, p[0]);
        p[1] = fmaf(kap, relq.y - rel.y, p[1]);
        p[2] = fmaf(kap, relq.z - rel.z, p[2]);
      }
    }
    for (int q = s0 + gl; q < s1; q += G) {
      const int4 st = S[q];
      const int ia = st.x & 0x7fffffff, ib = st.y & 0x7fffffff, ic = st.z & 0x7fffffff;
      const float fac = __int_as_float(st.w);
      float4 ah = X_(2 * ia), al = X_(2 * ia + 1), bh = X_(2 * ib), bl = X_(2 * ib + 1), ch = X_(2 * ic),
             cl = X_(2 * ic + 1);
      const float3 u = diffHL(ah, al, bh, bl), w = diffHL(ch, cl, bh, bl);
      f[0] = fmaf(fac, u.x + w.x, f[0]);
      f[1] = fmaf(fac, u.y + w.y, f[1]);
      f[2] = fmaf(fac, u.z + w.z, f[2]);
      if ((st.x | st.y | st.z) < 0) {  // pinned members: the matrix part sees them at q
        if (st.x < 0) pinHL(I, ia, ah, al);
        if (st.y < 0) pinHL(I, ib, bh, bl);
        if (st.z < 0) pinHL(I, ic, ch, cl);
        const float3 uq = diffHL(ah, al, bh, bl), wq = diffHL(ch, cl, bh, bl);
        p[0] = fmaf(fac, (u.x + w.x) - (uq.x + wq.x), p[0]);
        p[1] = fmaf(fac, (u.y + w.y) - (uq.y + wq.y), p[1]);
        p[2] = fmaf(fac, (u.z + w.z) - (uq.z + wq.z), p[2]);
      }
    }
  }
  // mass term (x − x̂)·m/h², added by one lane
  __device__ __forceinline__ void addMass(float4 vh, float4 vl, float4 xhh, float4 xhl, float mh2) {
    const float3 d = diffHL(vh, vl, xhh, xhl);
    a[0] = fmaf(d.x, mh2, a[0]);
    a[1] = fmaf(d.y, mh2, a[1]);
    a[2] = fmaf(d.z, mh2, a[2]);
  }
  template <int G>
  __device__ __forceinline__ void reduce() {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) {
        a[c] += __shfl_xor_sync(0xffffffffu, a[c], o);
        f[c] += __shfl_xor_sync(0xffffffffu, f[c], o);
        p[c] += __shfl_xor_sync(0xffffffffu, p[c], o);
      }
    }
  }
  // ‖t‖ / m
  __device__ __forceinline__ float residual(float invM) const {
    const float t0 = a[0] + f[0], t1 = a[1] + f[1], t2 = a[2] + f[2];
    return sqrtf(t0 * t0 + t1 * t1 + t2 * t2) * invM;
  }
  // r = −(mass + edge terms) + bend terms, pinned neighbours at q
  __device__ __forceinline__ float3 correction() const {
    return make_float3((f[0] - a[0]) - p[0], (f[1] - a[1]) - p[1], (f[2] - a[2]) - p[2]);
  }
};

}  // namespace pdg
