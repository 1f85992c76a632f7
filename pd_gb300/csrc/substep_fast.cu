// substep_fast.cu — FP64 substep with the supernodal triangular solve.
//
// The reference-order solve is a chain of dependent FP64 subtractions as long as the
// elimination tree is deep (dense separator rows of ~100 terms, one after another). Here the
// nested-dissection tree is walked level by level instead; every supernode S = [s0, s1) does
//   forward:  t_S = w_S − L_{S,desc}·y_desc      (off-block gather, parallel per row)
//             y_S = L_SS⁻¹ · t_S                  (dense mat-vec with the precomputed inverse)
//   backward: t_S = D⁻¹_S·y_S − L_{anc,S}ᵀ·x_anc  (off-block gather per column)
//             x_S = L_SS⁻ᵀ · t_S
// so a solve costs 4 × (tree depth) block-wide steps of short parallel reductions. Each row's sum
// is split over a group of G lanes and reduced with shuffles; all accumulation is FMA in FP64.
// The summation order differs from the reference, so results match it to rounding (~1e-15
// relative per solve), not bit for bit.
#include "substep_common.cuh"

namespace pdg {
namespace {

template <int G>
__device__ __forceinline__ double groupSum(double v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, G);
  return v;
}

template <int G>
struct SupernodalSolve {
  static __device__ void run(const InstanceDev& I, double* w, double* t) {
    const int lane = threadIdx.x & (G - 1);
    const int group = threadIdx.x / G;
    const int ngroups = blockDim.x / G;
    // ---- forward: leaves → root
    for (int l = 0; l < I.nlevS; ++l) {
      const int beg = I.lvlRowPtr[l], cnt = I.lvlRowPtr[l + 1] - beg;
      for (int base = 0; base < cnt; base += ngroups) {  // block-uniform trip count: shuffles are safe
        const int idx = base + group;
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        int i = 0;
        if (idx < cnt) {
          i = I.lvlRows[beg + idx];
          for (int p = I.Lrp[i] + lane; p < I.offEnd[i]; p += G) {
            const int j = I.Lci[p];
            const double lv = I.Lrv[p];
            a0 = fma(lv, w[3 * j], a0);
            a1 = fma(lv, w[3 * j + 1], a1);
            a2 = fma(lv, w[3 * j + 2], a2);
          }
        }
        a0 = groupSum<G>(a0);
        a1 = groupSum<G>(a1);
        a2 = groupSum<G>(a2);
        if (idx < cnt && lane == 0) {
          t[3 * i] = w[3 * i] - a0;
          t[3 * i + 1] = w[3 * i + 1] - a1;
          t[3 * i + 2] = w[3 * i + 2] - a2;
        }
      }
      __syncthreads();
      for (int base = 0; base < cnt; base += ngroups) {
        const int idx = base + group;
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        int i = 0;
        if (idx < cnt) {
          i = I.lvlRows[beg + idx];
          const int s = I.rowSn[i];
          const int s0 = I.snStart[s];
          const int r = i - s0;
          const double* X = I.invL + I.snInvOff[s] + (int64_t)r * (r + 1) / 2;
          for (int c = lane; c <= r; c += G) {
            const double xv = X[c];
            const int j = s0 + c;
            a0 = fma(xv, t[3 * j], a0);
            a1 = fma(xv, t[3 * j + 1], a1);
            a2 = fma(xv, t[3 * j + 2], a2);
          }
        }
        a0 = groupSum<G>(a0);
        a1 = groupSum<G>(a1);
        a2 = groupSum<G>(a2);
        if (idx < cnt && lane == 0) {
          w[3 * i] = a0;
          w[3 * i + 1] = a1;
          w[3 * i + 2] = a2;
        }
      }
      __syncthreads();
    }
    // ---- backward: root → leaves
    for (int l = I.nlevS - 1; l >= 0; --l) {
      const int beg = I.lvlRowPtr[l], cnt = I.lvlRowPtr[l + 1] - beg;
      for (int base = 0; base < cnt; base += ngroups) {
        const int idx = base + group;
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        int k = 0;
        if (idx < cnt) {
          k = I.lvlRows[beg + idx];
          for (int p = I.offBeg[k] + lane; p < I.Lcp[k + 1]; p += G) {
            const int i = I.Lri[p];
            const double lv = I.Lcv[p];
            a0 = fma(lv, w[3 * i], a0);
            a1 = fma(lv, w[3 * i + 1], a1);
            a2 = fma(lv, w[3 * i + 2], a2);
          }
        }
        a0 = groupSum<G>(a0);
        a1 = groupSum<G>(a1);
        a2 = groupSum<G>(a2);
        if (idx < cnt && lane == 0) {
          const double di = I.dinv[k];
          t[3 * k] = fma(w[3 * k], di, -a0);
          t[3 * k + 1] = fma(w[3 * k + 1], di, -a1);
          t[3 * k + 2] = fma(w[3 * k + 2], di, -a2);
        }
      }
      __syncthreads();
      for (int base = 0; base < cnt; base += ngroups) {
        const int idx = base + group;
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        int k = 0;
        if (idx < cnt) {
          k = I.lvlRows[beg + idx];
          const int s = I.rowSn[k];
          const int s0 = I.snStart[s];
          const int sz = I.snStart[s + 1] - s0;
          const int r = k - s0;
          const double* XT = I.invLT + I.snInvOff[s] + (int64_t)r * sz - (int64_t)r * (r - 1) / 2;
          for (int c = lane; c < sz - r; c += G) {
            const double xv = XT[c];
            const int j = k + c;
            a0 = fma(xv, t[3 * j], a0);
            a1 = fma(xv, t[3 * j + 1], a1);
            a2 = fma(xv, t[3 * j + 2], a2);
          }
        }
        a0 = groupSum<G>(a0);
        a1 = groupSum<G>(a1);
        a2 = groupSum<G>(a2);
        if (idx < cnt && lane == 0) {
          w[3 * k] = a0;
          w[3 * k + 1] = a1;
          w[3 * k + 2] = a2;
        }
      }
      __syncthreads();
    }
  }
};

constexpr int kGroup = 8;

__global__ void __launch_bounds__(kBlockThreads) substepFastKernel(const InstanceDev* __restrict__ insts,
                                                                   int substeps, int smemBytes) {
  extern __shared__ double smem[];
  __shared__ double red[32];
  __shared__ int flag;
  const InstanceDev& I = insts[blockIdx.x];
  const bool inSmem = 6 * I.n * (int)sizeof(double) <= smemBytes;
  double* w = inSmem ? smem : I.w;
  double* t = inSmem ? smem + 3 * I.n : I.tbuf;
  runSubsteps<FastArith, SupernodalSolve<kGroup>>(I, substeps, w, t, red, &flag);
}

__global__ void __launch_bounds__(kBlockThreads) solveFastKernel(const InstanceDev* __restrict__ inst,
                                                                 const double* __restrict__ b,
                                                                 double* __restrict__ x, int smemBytes) {
  extern __shared__ double smem[];
  const InstanceDev& I = *inst;
  const bool inSmem = 6 * I.n * (int)sizeof(double) <= smemBytes;
  double* w = inSmem ? smem : I.w;
  double* t = inSmem ? smem + 3 * I.n : I.tbuf;
  for (int v = threadIdx.x; v < I.n; v += blockDim.x) {
    const int r = I.iperm[v];
    w[3 * r] = b[3 * v];
    w[3 * r + 1] = b[3 * v + 1];
    w[3 * r + 2] = b[3 * v + 2];
  }
  __syncthreads();
  SupernodalSolve<kGroup>::run(I, w, t);
  for (int v = threadIdx.x; v < I.n; v += blockDim.x) {
    const int r = I.iperm[v];
    x[3 * v] = w[3 * r];
    x[3 * v + 1] = w[3 * r + 1];
    x[3 * v + 2] = w[3 * r + 2];
  }
}

}  // namespace

int launchSubstepFast(const InstanceDev* d, int count, int substeps, int smemBytes, void* stream) {
  if (count <= 0 || substeps <= 0) return 0;
  static bool attrSet = false;
  if (!attrSet) {
    cudaFuncSetAttribute(substepFastKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attrSet = true;
  }
  substepFastKernel<<<count, kBlockThreads, smemBytes, static_cast<cudaStream_t>(stream)>>>(d, substeps, smemBytes);
  return static_cast<int>(cudaGetLastError());
}

int launchSolveFast(const InstanceDev* d, const double* b, double* x, int smemBytes, void* stream) {
  static bool attrSet = false;
  if (!attrSet) {
    cudaFuncSetAttribute(solveFastKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attrSet = true;
  }
  solveFastKernel<<<1, kBlockThreads, smemBytes, static_cast<cudaStream_t>(stream)>>>(d, b, x, smemBytes);
  return static_cast<int>(cudaGetLastError());
}

}  // namespace pdg
