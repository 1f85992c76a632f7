// substep_fast.cu — FP64 substep with the supernodal triangular solve, run by one CTA per
// cloth (batches) or by a thread-block cluster per cloth (a few large or single cloths).
//
// The reference-order solve is a chain of dependent FP64 subtractions as long as the
// elimination tree is deep. Here the nested-dissection tree is walked level by level; every
// supernode S = [s0, s1) does
//   forward:  t_S = w_S − L_{S,desc}·y_desc      (off-block gather, parallel per row)
//             y_S = L_SS⁻¹ · t_S                  (dense mat-vec with the precomputed inverse)
//   backward: t_S = D⁻¹_S·y_S − L_{anc,S}ᵀ·x_anc  (off-block gather per column)
//             x_S = L_SS⁻ᵀ · t_S
// with each row's sum split over G lanes (G per level and phase from the host's cost model).
// Sums are reordered and contracted (FMA), so results match the reference to rounding, not bit
// for bit (the tests hold them to 1e-10 relative after the full scene).
#include "substep_team.cuh"

namespace pdg {
namespace {

template <bool TIMED>
__global__ void __launch_bounds__(kBlockThreads) substepFastKernel(const InstanceDev* __restrict__ insts,
                                                                   int substeps, int smemBytes) {
  extern __shared__ double smem[];
  __shared__ double red[32];
  __shared__ double slots[2];
  const InstanceDev& I = insts[blockIdx.x];
  const bool inSmem = 6 * I.n * (int)sizeof(double) <= smemBytes;
  double* w = inSmem ? smem : I.w;
  double* t = inSmem ? smem + 3 * I.n : I.tbuf;
  const Team<false> tm{0, 1};
  runSubstepsTeam<false, TIMED>(I, tm, substeps, w, t, red, slots);
}

template <bool TIMED>
__global__ void __launch_bounds__(kBlockThreads) substepClusterKernel(const InstanceDev* __restrict__ insts,
                                                                      int substeps) {
  __shared__ double red[32];
  __shared__ double slots[2];
  cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
  const int cs = static_cast<int>(cl.num_blocks());
  const InstanceDev& I = insts[blockIdx.x / cs];
  const Team<true> tm{static_cast<int>(cl.block_rank()), cs};
  runSubstepsTeam<true, TIMED>(I, tm, substeps, I.w, I.tbuf, red, slots);
}

// One large cloth on a cooperative grid of CTAs: the cluster code with grid barriers; the
// instance's FP64 refinement workspace x0 (unused in the FP64 modes) holds the team-maximum slots.
template <bool TIMED>
__global__ void __launch_bounds__(kBlockThreads) substepGridKernel(const InstanceDev* __restrict__ insts,
                                                                   int substeps) {
  __shared__ double red[32];
  __shared__ double slots[2];
  const InstanceDev& I = insts[0];
  Team<true> tm{static_cast<int>(blockIdx.x), static_cast<int>(gridDim.x)};
  tm.gslots = I.x0;
  runSubstepsTeam<true, TIMED>(I, tm, substeps, I.w, I.tbuf, red, slots);
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
  const Team<false> tm{0, 1};
  TeamSolve<false>::run(I, tm, w, t);
  for (int v = threadIdx.x; v < I.n; v += blockDim.x) {
    const int r = I.iperm[v];
    x[3 * v] = w[3 * r];
    x[3 * v + 1] = w[3 * r + 1];
    x[3 * v + 2] = w[3 * r + 2];
  }
}

// Rows 3b, 3b+1, 3b+2 of Ã⁻¹ for b = blockIdx.x: the FP64 supernodal solve of three unit vectors
// at once (column 3b + c in component c). Ã is symmetric, so a solved column is the row stored.
__global__ void __launch_bounds__(kBlockThreads) denseInverseKernel(const InstanceDev* __restrict__ inst) {
  extern __shared__ double smem[];
  const InstanceDev& I = *inst;
  const int n = I.n, v0 = 3 * static_cast<int>(blockIdx.x);
  double* w = smem;
  double* t = smem + 3 * n;
  for (int i = threadIdx.x; i < 3 * n; i += blockDim.x) w[i] = 0.0;
  __syncthreads();
  if (threadIdx.x < 3 && v0 + static_cast<int>(threadIdx.x) < n)
    w[3 * I.iperm[v0 + threadIdx.x] + threadIdx.x] = 1.0;
  __syncthreads();
  const Team<false> tm{0, 1};
  TeamSolve<false>::run(I, tm, w, t);
  float* A = const_cast<float*>(I.Ainv);
  float* Alo = const_cast<float*>(I.AinvLo);  // the FP64 team kernel also keeps the FP32 remainder
  for (int c = 0; c < 3 && v0 + c < n; ++c) {
    float* row = A + static_cast<size_t>(v0 + c) * I.denseLd;
    float* rowLo = Alo ? Alo + static_cast<size_t>(v0 + c) * I.denseLd : nullptr;
    for (int u = threadIdx.x; u < n; u += blockDim.x) {
      const double a = w[3 * I.iperm[u] + c];
      const float hi = static_cast<float>(a);
      row[u] = hi;
      if (rowLo) rowLo[u] = static_cast<float>(a - static_cast<double>(hi));
    }
  }
}

cudaLaunchConfig_t clusterConfig(int blocks, int clusterSize, int smemBytes, void* stream, cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(kBlockThreads);
  cfg.dynamicSmemBytes = smemBytes;
  cfg.stream = static_cast<cudaStream_t>(stream);
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = clusterSize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

}  // namespace

int launchSubstepFast(const InstanceDev* d, int count, int substeps, int smemBytes, void* stream, bool timed) {
  if (count <= 0 || substeps <= 0) return 0;
  static bool attrSet = false;
  if (!attrSet) {
    cudaFuncSetAttribute(substepFastKernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(substepFastKernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attrSet = true;
  }
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (timed) substepFastKernel<true><<<count, kBlockThreads, smemBytes, st>>>(d, substeps, smemBytes);
  else substepFastKernel<false><<<count, kBlockThreads, smemBytes, st>>>(d, substeps, smemBytes);
  return static_cast<int>(cudaGetLastError());
}

int clusterSizeSupported(int want) {
  static int cached[17] = {0};
  if (want < 1 || want > 16) return 0;
  if (cached[want]) return cached[want] > 0 ? want : 0;
  bool ok = true;
  for (auto kernel : {substepClusterKernel<false>, substepClusterKernel<true>}) {  // both must run
    if (want > 8) cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = clusterConfig(want, want, 0, nullptr, attr);
    int clusters = 0;
    const cudaError_t e = cudaOccupancyMaxActiveClusters(&clusters, kernel, &cfg);
    if (e != cudaSuccess) cudaGetLastError();
    ok = ok && e == cudaSuccess && clusters > 0;
  }
  cached[want] = ok ? 1 : -1;
  return ok ? want : 0;
}

int gridCapacity() {
  static int cached = -1;
  if (cached >= 0) return cached;
  int dev = 0, sms = 0, least = 1 << 30;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return cached = 0;
  }
  for (auto kernel : {substepGridKernel<false>, substepGridKernel<true>}) {  // both must fit
    int perSm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kernel, kBlockThreads, 0) != cudaSuccess) {
      cudaGetLastError();
      return cached = 0;
    }
    least = least < perSm ? least : perSm;
  }
  return cached = least * sms;
}

int launchSubstepGrid(const InstanceDev* d, int ctas, int substeps, void* stream, bool timed) {
  if (substeps <= 0) return 0;
  if (ctas < 2 || ctas > gridCapacity()) return static_cast<int>(cudaErrorCooperativeLaunchTooLarge);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ctas);
  cfg.blockDim = dim3(kBlockThreads);
  cfg.stream = static_cast<cudaStream_t>(stream);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const cudaError_t e = timed ? cudaLaunchKernelEx(&cfg, substepGridKernel<true>, d, substeps)
                              : cudaLaunchKernelEx(&cfg, substepGridKernel<false>, d, substeps);
  return static_cast<int>(e != cudaSuccess ? e : cudaGetLastError());
}

int launchSubstepCluster(const InstanceDev* d, int count, int clusterSize, int substeps, void* stream, bool timed) {
  if (count <= 0 || substeps <= 0) return 0;
  if (clusterSizeSupported(clusterSize) != clusterSize) return static_cast<int>(cudaErrorInvalidConfiguration);
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = clusterConfig(count * clusterSize, clusterSize, 0, stream, attr);
  const cudaError_t e = timed ? cudaLaunchKernelEx(&cfg, substepClusterKernel<true>, d, substeps)
                              : cudaLaunchKernelEx(&cfg, substepClusterKernel<false>, d, substeps);
  return static_cast<int>(e != cudaSuccess ? e : cudaGetLastError());
}

int launchDenseInverse(const InstanceDev* d, int n, void* stream) {
  if (n <= 0) return 0;
  const int smem = 48 * n;
  if (smem > 200 * 1024) return static_cast<int>(cudaErrorInvalidValue);
  static bool attrSet = false;
  if (!attrSet) {
    cudaFuncSetAttribute(denseInverseKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attrSet = true;
  }
  denseInverseKernel<<<(n + 2) / 3, kBlockThreads, smem, static_cast<cudaStream_t>(stream)>>>(d);
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
