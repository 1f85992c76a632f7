// team_solve32.cuh — the FP32 supernodal solve of solve32.cuh with its rows strided over a team:
// one CTA, a thread-block cluster, or a cooperative grid of CTAs (Team<true> with grid slots).
#pragma once

#include "solve32.cuh"
#include "substep_team.cuh"

namespace pdg {

// Y holds the right-hand side on entry and the solution on exit (elimination order); T is a
// temporary of the same size. Every phase ends with a team barrier.
template <bool CLUSTER>
struct TeamSolve32 {
  template <int G, class Body>
  static __device__ __forceinline__ void rows(const Team<CLUSTER>& tm, int cnt, Body&& body) {
    const int lane = threadIdx.x & (G - 1);
    const int groups = static_cast<int>(blockDim.x) / G;
    const int gid = tm.rank * groups + static_cast<int>(threadIdx.x) / G;
    const int stride = tm.size * groups;
    for (int base = 0; base < cnt; base += stride) {  // uniform trip count keeps shuffles converged
      const int idx = base + gid;
      float a0 = 0.f, a1 = 0.f, a2 = 0.f;
      body.accumulate(idx, lane, G, a0, a1, a2);
      if (G > 1) {
        a0 = groupSumF<G>(a0);
        a1 = groupSumF<G>(a1);
        a2 = groupSumF<G>(a2);
      }
      if (lane == 0) body.finish(idx, a0, a1, a2);
    }
  }
  template <class Body>
  static __device__ __forceinline__ void dispatch(const Team<CLUSTER>& tm, int g, int cnt, Body&& body) {
    switch (g) {
      case 1: rows<1>(tm, cnt, body); break;
      case 2: rows<2>(tm, cnt, body); break;
      case 4: rows<4>(tm, cnt, body); break;
      case 8: rows<8>(tm, cnt, body); break;
      case 16: rows<16>(tm, cnt, body); break;
      default: rows<32>(tm, cnt, body); break;
    }
  }
  struct FwdGather {  // t_i = y_i − Σ_{j < s0} L_ij·y_j
    const InstanceDev& I; const Team<CLUSTER>& tm; const float* Y; float* T; int beg, cnt;
    __device__ void accumulate(int idx, int lane, int G, float& a0, float& a1, float& a2) const {
      if (idx >= cnt) return;
      const int i = I.lvlRows[beg + idx];
#pragma unroll 4
      for (int p = I.Lrp[i] + lane; p < I.offEnd[i]; p += G) {
        const int j = I.Lci[p];
        const float lv = I.Lrv32[p];
        a0 = fmaf(lv, tm.ld(Y + 3 * j), a0);
        a1 = fmaf(lv, tm.ld(Y + 3 * j + 1), a1);
        a2 = fmaf(lv, tm.ld(Y + 3 * j + 2), a2);
      }
    }
    __device__ void finish(int idx, float a0, float a1, float a2) const {
      if (idx >= cnt) return;
      const int i = I.lvlRows[beg + idx];
      T[3 * i] = tm.ld(Y + 3 * i) - a0;
      T[3 * i + 1] = tm.ld(Y + 3 * i + 1) - a1;
      T[3 * i + 2] = tm.ld(Y + 3 * i + 2) - a2;
    }
  };
  struct FwdDense {  // y_i = Σ_{c ≤ r} (L_SS⁻¹)_{rc}·t_{s0+c}
    const InstanceDev& I; const Team<CLUSTER>& tm; float* Y; const float* T; int beg, cnt;
    __device__ void accumulate(int idx, int lane, int G, float& a0, float& a1, float& a2) const {
      if (idx >= cnt) return;
      const int i = I.lvlRows[beg + idx];
      const int s = I.rowSn[i];
      const int s0 = I.snStart[s];
      const int r = i - s0;
      const float* X = I.invL32 + I.snInvOff[s] + (int64_t)r * (r + 1) / 2;
#pragma unroll 4
      for (int c = lane; c <= r; c += G) {
        const float xv = X[c];
        const int j = s0 + c;
        a0 = fmaf(xv, tm.ld(T + 3 * j), a0);
        a1 = fmaf(xv, tm.ld(T + 3 * j + 1), a1);
        a2 = fmaf(xv, tm.ld(T + 3 * j + 2), a2);
      }
    }
    __device__ void finish(int idx, float a0, float a1, float a2) const {
      if (idx >= cnt) return;
      const int i = I.lvlRows[beg + idx];
      Y[3 * i] = a0;
      Y[3 * i + 1] = a1;
      Y[3 * i + 2] = a2;
    }
  };
  struct BwdGather {  // t_k = D⁻¹_k·y_k − Σ_{i ≥ s1} L_ik·x_i
    const InstanceDev& I; const Team<CLUSTER>& tm; const float* Y; float* T; int beg, cnt;
    __device__ void accumulate(int idx, int lane, int G, float& a0, float& a1, float& a2) const {
      if (idx >= cnt) return;
      const int k = I.lvlRows[beg + idx];
#pragma unroll 4
      for (int p = I.offBeg[k] + lane; p < I.Lcp[k + 1]; p += G) {
        const int i = I.Lri[p];
        const float lv = I.Lcv32[p];
        a0 = fmaf(lv, tm.ld(Y + 3 * i), a0);
        a1 = fmaf(lv, tm.ld(Y + 3 * i + 1), a1);
        a2 = fmaf(lv, tm.ld(Y + 3 * i + 2), a2);
      }
    }
    __device__ void finish(int idx, float a0, float a1, float a2) const {
      if (idx >= cnt) return;
      const int k = I.lvlRows[beg + idx];
      const float di = I.dinv32[k];
      T[3 * k] = fmaf(tm.ld(Y + 3 * k), di, -a0);
      T[3 * k + 1] = fmaf(tm.ld(Y + 3 * k + 1), di, -a1);
      T[3 * k + 2] = fmaf(tm.ld(Y + 3 * k + 2), di, -a2);
    }
  };
  struct BwdDense {  // x_k = Σ_{c ≥ r} (L_SS⁻¹)_{cr}·t_{s0+c}
    const InstanceDev& I; const Team<CLUSTER>& tm; float* Y; const float* T; int beg, cnt;
    __device__ void accumulate(int idx, int lane, int G, float& a0, float& a1, float& a2) const {
      if (idx >= cnt) return;
      const int k = I.lvlRows[beg + idx];
      const int s = I.rowSn[k];
      const int s0 = I.snStart[s];
      const int sz = I.snStart[s + 1] - s0;
      const int r = k - s0;
      const float* XT = I.invLT32 + I.snInvOff[s] + (int64_t)r * sz - (int64_t)r * (r - 1) / 2;
#pragma unroll 4
      for (int c = lane; c < sz - r; c += G) {
        const float xv = XT[c];
        const int j = k + c;
        a0 = fmaf(xv, tm.ld(T + 3 * j), a0);
        a1 = fmaf(xv, tm.ld(T + 3 * j + 1), a1);
        a2 = fmaf(xv, tm.ld(T + 3 * j + 2), a2);
      }
    }
    __device__ void finish(int idx, float a0, float a1, float a2) const {
      if (idx >= cnt) return;
      const int k = I.lvlRows[beg + idx];
      Y[3 * k] = a0;
      Y[3 * k + 1] = a1;
      Y[3 * k + 2] = a2;
    }
  };
  static __device__ void run(const InstanceDev& I, const Team<CLUSTER>& tm, float* Y, float* T) {
    for (int l = 0; l < I.nlevS; ++l) {
      const int beg = I.lvlRowPtr[l], cnt = I.lvlRowPtr[l + 1] - beg;
      dispatch(tm, I.lvlG32[4 * l + 0], cnt, FwdGather{I, tm, Y, T, beg, cnt});
      tm.sync();
      dispatch(tm, I.lvlG32[4 * l + 1], cnt, FwdDense{I, tm, Y, T, beg, cnt});
      tm.sync();
    }
    for (int l = I.nlevS - 1; l >= 0; --l) {
      const int beg = I.lvlRowPtr[l], cnt = I.lvlRowPtr[l + 1] - beg;
      dispatch(tm, I.lvlG32[4 * l + 2], cnt, BwdGather{I, tm, Y, T, beg, cnt});
      tm.sync();
      dispatch(tm, I.lvlG32[4 * l + 3], cnt, BwdDense{I, tm, Y, T, beg, cnt});
      tm.sync();
    }
  }
};

}  // namespace pdg
