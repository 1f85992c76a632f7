// solve32.cuh — FP32 supernodal solve of one cloth by one CTA.
//
// The factor's nested-dissection tree is walked level by level: per level, the rows' off-block
// entries are gathered (forward: columns in descendant supernodes; backward: rows in ancestor
// supernodes) and the level's diagonal blocks are applied as their dense inverses. Each row gets
// G ∈ {1, 2, 4, …, 32} lanes per phase (the host's choice in lvlG32) and the three components
// (x, y, z) are carried together.
#pragma once

#include "device.cuh"

namespace pdg {

template <int G>
__device__ __forceinline__ float groupSumF(float v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, G);
  return v;
}

// One-CTA FP32 supernodal solve in place: Y holds the right-hand side on entry and the solution
// on exit (elimination order), T is a temporary of the same size.
struct LocalSolve32 {
  template <int G, class Body>
  static __device__ __forceinline__ void rows(int cnt, Body&& body) {
    const int lane = threadIdx.x & (G - 1);
    const int groups = (int)blockDim.x / G;
    const int gid = (int)threadIdx.x / G;
    for (int base = 0; base < cnt; base += groups) {  // block-uniform trip count
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
  static __device__ __forceinline__ void dispatch(int g, int cnt, Body&& body) {
    switch (g) {
      case 1: rows<1>(cnt, body); break;
      case 2: rows<2>(cnt, body); break;
      case 4: rows<4>(cnt, body); break;
      case 8: rows<8>(cnt, body); break;
      case 16: rows<16>(cnt, body); break;
      default: rows<32>(cnt, body); break;
    }
  }
  struct FwdGather {
    const InstanceDev& I; const float* Y; float* T; int beg, cnt;
    __device__ void accumulate(int idx, int lane, int G, float& a0, float& a1, float& a2) const {
      if (idx >= cnt) return;
      const int i = I.lvlRows[beg + idx];
#pragma unroll 4
      for (int p = I.Lrp[i] + lane; p < I.offEnd[i]; p += G) {
        const int j = I.Lci[p];
        const float lv = I.Lrv32[p];
        a0 = fmaf(lv, Y[3 * j], a0);
        a1 = fmaf(lv, Y[3 * j + 1], a1);
        a2 = fmaf(lv, Y[3 * j + 2], a2);
      }
    }
    __device__ void finish(int idx, float a0, float a1, float a2) const {
      if (idx >= cnt) return;
      const int i = I.lvlRows[beg + idx];
      T[3 * i] = Y[3 * i] - a0;
      T[3 * i + 1] = Y[3 * i + 1] - a1;
      T[3 * i + 2] = Y[3 * i + 2] - a2;
    }
  };
  struct FwdDense {
    const InstanceDev& I; float* Y; const float* T; int beg, cnt;
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
        a0 = fmaf(xv, T[3 * j], a0);
        a1 = fmaf(xv, T[3 * j + 1], a1);
        a2 = fmaf(xv, T[3 * j + 2], a2);
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
  struct BwdGather {
    const InstanceDev& I; const float* Y; float* T; int beg, cnt;
    __device__ void accumulate(int idx, int lane, int G, float& a0, float& a1, float& a2) const {
      if (idx >= cnt) return;
      const int k = I.lvlRows[beg + idx];
#pragma unroll 4
      for (int p = I.offBeg[k] + lane; p < I.Lcp[k + 1]; p += G) {
        const int i = I.Lri[p];
        const float lv = I.Lcv32[p];
        a0 = fmaf(lv, Y[3 * i], a0);
        a1 = fmaf(lv, Y[3 * i + 1], a1);
        a2 = fmaf(lv, Y[3 * i + 2], a2);
      }
    }
    __device__ void finish(int idx, float a0, float a1, float a2) const {
      if (idx >= cnt) return;
      const int k = I.lvlRows[beg + idx];
      const float di = I.dinv32[k];
      T[3 * k] = fmaf(Y[3 * k], di, -a0);
      T[3 * k + 1] = fmaf(Y[3 * k + 1], di, -a1);
      T[3 * k + 2] = fmaf(Y[3 * k + 2], di, -a2);
    }
  };
  struct BwdDense {
    const InstanceDev& I; float* Y; const float* T; int beg, cnt;
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
        a0 = fmaf(xv, T[3 * j], a0);
        a1 = fmaf(xv, T[3 * j + 1], a1);
        a2 = fmaf(xv, T[3 * j + 2], a2);
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
  static __device__ void run(const InstanceDev& I, float* Y, float* T) {
    for (int l = 0; l < I.nlevS; ++l) {
      const int beg = I.lvlRowPtr[l], cnt = I.lvlRowPtr[l + 1] - beg;
      dispatch(I.lvlG32[4 * l + 0], cnt, FwdGather{I, Y, T, beg, cnt});
      __syncthreads();
      dispatch(I.lvlG32[4 * l + 1], cnt, FwdDense{I, Y, T, beg, cnt});
      __syncthreads();
    }
    for (int l = I.nlevS - 1; l >= 0; --l) {
      const int beg = I.lvlRowPtr[l], cnt = I.lvlRowPtr[l + 1] - beg;
      dispatch(I.lvlG32[4 * l + 2], cnt, BwdGather{I, Y, T, beg, cnt});
      __syncthreads();
      dispatch(I.lvlG32[4 * l + 3], cnt, BwdDense{I, Y, T, beg, cnt});
      __syncthreads();
    }
  }
};

}  // namespace pdg
