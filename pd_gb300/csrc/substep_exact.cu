// substep_exact.cu — the per-substep PD loop in the reference's exact FP64 arithmetic order.
//
// Every product and sum rounds on its own (ExactArith; the unit is also built with
// -fmad=false) and every per-vertex / per-row sum runs in the reference's order, so the result
// is bit-identical to the reference CPU path. The solve is level-scheduled: forward rows gather
// in ascending column order (the reference's column-scatter form gives each row its terms in
// that order), backward columns gather in ascending row order (EigenDirectSolver.cpp:411-448);
// one thread per row, the three components together.
#include "substep_common.cuh"

namespace pdg {
namespace {

struct ExactSolve {
  static __device__ void run(const InstanceDev& I, double* w, double*) {
    for (int l = 0; l < I.nlevF; ++l) {
      const int beg = I.fwdPtr[l], end = I.fwdPtr[l + 1];
      for (int t = beg + threadIdx.x; t < end; t += blockDim.x) {
        const int r = I.fwdRows[t];
        double a0 = w[3 * r], a1 = w[3 * r + 1], a2 = w[3 * r + 2];
        for (int p = I.Lrp[r]; p < I.Lrp[r + 1]; ++p) {
          const int j = I.Lci[p];
          const double lv = I.Lrv[p];
          a0 = __dsub_rn(a0, __dmul_rn(lv, w[3 * j]));
          a1 = __dsub_rn(a1, __dmul_rn(lv, w[3 * j + 1]));
          a2 = __dsub_rn(a2, __dmul_rn(lv, w[3 * j + 2]));
        }
        w[3 * r] = a0;
        w[3 * r + 1] = a1;
        w[3 * r + 2] = a2;
      }
      __syncthreads();
    }
    for (int l = 0; l < I.nlevB; ++l) {
      const int beg = I.bwdPtr[l], end = I.bwdPtr[l + 1];
      for (int t = beg + threadIdx.x; t < end; t += blockDim.x) {
        const int k = I.bwdRows[t];
        const double di = I.dinv[k];
        double a0 = __dmul_rn(w[3 * k], di), a1 = __dmul_rn(w[3 * k + 1], di), a2 = __dmul_rn(w[3 * k + 2], di);
        for (int p = I.Lcp[k]; p < I.Lcp[k + 1]; ++p) {
          const int i = I.Lri[p];
          const double lv = I.Lcv[p];
          a0 = __dsub_rn(a0, __dmul_rn(lv, w[3 * i]));
          a1 = __dsub_rn(a1, __dmul_rn(lv, w[3 * i + 1]));
          a2 = __dsub_rn(a2, __dmul_rn(lv, w[3 * i + 2]));
        }
        w[3 * k] = a0;
        w[3 * k + 1] = a1;
        w[3 * k + 2] = a2;
      }
      __syncthreads();
    }
  }
};

template <bool TIMED>
__global__ void __launch_bounds__(kBlockThreads) substepExactKernel(const InstanceDev* __restrict__ insts,
                                                                    int substeps, int smemBytes) {
  extern __shared__ double smem[];
  __shared__ double red[32];
  __shared__ int flag;
  const InstanceDev& I = insts[blockIdx.x];
  double* w = (3 * I.n * (int)sizeof(double) <= smemBytes) ? smem : I.w;
  runSubsteps<ExactArith, ExactSolve, TIMED>(I, substeps, w, nullptr, red, &flag);
}

__global__ void __launch_bounds__(kBlockThreads) solveExactKernel(const InstanceDev* __restrict__ inst,
                                                                  const double* __restrict__ b,
                                                                  double* __restrict__ x, int smemBytes) {
  extern __shared__ double smem[];
  const InstanceDev& I = *inst;
  double* w = (3 * I.n * (int)sizeof(double) <= smemBytes) ? smem : I.w;
  for (int v = threadIdx.x; v < I.n; v += blockDim.x) {
    const int r = I.iperm[v];
    w[3 * r] = b[3 * v];
    w[3 * r + 1] = b[3 * v + 1];
    w[3 * r + 2] = b[3 * v + 2];
  }
  __syncthreads();
  ExactSolve::run(I, w, nullptr);
  for (int v = threadIdx.x; v < I.n; v += blockDim.x) {
    const int r = I.iperm[v];
    x[3 * v] = w[3 * r];
    x[3 * v + 1] = w[3 * r + 1];
    x[3 * v + 2] = w[3 * r + 2];
  }
}

// One column of the solve (IGlobalSolver::solveComponent): the same level schedule and the same
// per-row order as the three-column solve, so each column's bits equal that column of it.
__global__ void __launch_bounds__(kBlockThreads) solveColumnExactKernel(const InstanceDev* __restrict__ inst,
                                                                        const double* __restrict__ b,
                                                                        double* __restrict__ x,
                                                                        double* __restrict__ wGlobal, int smemBytes) {
  extern __shared__ double smem[];
  const InstanceDev& I = *inst;
  double* w = (I.n * (int)sizeof(double) <= smemBytes) ? smem : wGlobal;
  for (int v = threadIdx.x; v < I.n; v += blockDim.x) w[I.iperm[v]] = b[v];
  __syncthreads();
  for (int l = 0; l < I.nlevF; ++l) {
    const int beg = I.fwdPtr[l], end = I.fwdPtr[l + 1];
    for (int t = beg + threadIdx.x; t < end; t += blockDim.x) {
      const int r = I.fwdRows[t];
      double a = w[r];
      for (int p = I.Lrp[r]; p < I.Lrp[r + 1]; ++p) a = __dsub_rn(a, __dmul_rn(I.Lrv[p], w[I.Lci[p]]));
      w[r] = a;
    }
    __syncthreads();
  }
  for (int l = 0; l < I.nlevB; ++l) {
    const int beg = I.bwdPtr[l], end = I.bwdPtr[l + 1];
    for (int t = beg + threadIdx.x; t < end; t += blockDim.x) {
      const int k = I.bwdRows[t];
      double a = __dmul_rn(w[k], I.dinv[k]);
      for (int p = I.Lcp[k]; p < I.Lcp[k + 1]; ++p) a = __dsub_rn(a, __dmul_rn(I.Lcv[p], w[I.Lri[p]]));
      w[k] = a;
    }
    __syncthreads();
  }
  for (int v = threadIdx.x; v < I.n; v += blockDim.x) x[v] = w[I.iperm[v]];
}

}  // namespace

int launchSubstepExact(const InstanceDev* d, int count, int substeps, int smemBytes, void* stream, bool timed) {
  if (count <= 0 || substeps <= 0) return 0;
  static bool attrSet = false;
  if (!attrSet) {
    cudaFuncSetAttribute(substepExactKernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(substepExactKernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attrSet = true;
  }
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (timed) substepExactKernel<true><<<count, kBlockThreads, smemBytes, st>>>(d, substeps, smemBytes);
  else substepExactKernel<false><<<count, kBlockThreads, smemBytes, st>>>(d, substeps, smemBytes);
  return static_cast<int>(cudaGetLastError());
}

int launchSolveColumnExact(const InstanceDev* d, const double* b, double* x, double* w, int smemBytes,
                           void* stream) {
  // set once, from whichever thread launches first (thread-safe static initialisation): the
  // three component solves of one solver may be launched from three threads
  static const cudaError_t attr =
      cudaFuncSetAttribute(solveColumnExactKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (attr != cudaSuccess) return static_cast<int>(attr);
  solveColumnExactKernel<<<1, kBlockThreads, smemBytes, static_cast<cudaStream_t>(stream)>>>(d, b, x, w, smemBytes);
  return static_cast<int>(cudaGetLastError());  // the runtime keeps the last error per host thread
}

int launchSolveExact(const InstanceDev* d, const double* b, double* x, int smemBytes, void* stream) {
  static bool attrSet = false;
  if (!attrSet) {
    cudaFuncSetAttribute(solveExactKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attrSet = true;
  }
  solveExactKernel<<<1, kBlockThreads, smemBytes, static_cast<cudaStream_t>(stream)>>>(d, b, x, smemBytes);
  return static_cast<int>(cudaGetLastError());
}

}  // namespace pdg
