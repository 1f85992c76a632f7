// substep_mixed_grid.cu — FP32_SOLVE substeps of one large cloth on a cooperative grid of CTAs.
//
// The FP32-solve mode does, in every PD iteration,
//   x₀ = solve₃₂(b);  r = b − Ã·x₀ (FP64);  x = x₀ + solve₃₂(r)
// — one step of iterative refinement on an FP32 supernodal solve (substep_mixed.cu). The one-CTA
// and cluster kernels there solve the whole system redundantly in each CTA's shared memory, which a
// 256 × 256 cloth (65,536 vertices) does not fit: one CTA then walks the factor alone (≈0.85 s a
// substep). Here the whole grid shares the cloth instead, as the FP64 and correction grid teams do:
// the FP64 substep of substep_team.cuh (right-hand side gather, unpack, edge terms, residual gate)
// with its solve replaced by the two FP32 team solves of team_solve32.cuh around the FP64 residual,
// every row loop strided over every thread of the grid and every phase closed by a grid barrier.
#include <algorithm>

#include "team_solve32.cuh"

namespace pdg {
namespace {

// w holds b (elimination order, FP64) on entry and x on exit; t (3n doubles) keeps x₀ between the
// two solves. The FP32 vectors are the instance's y32 / t32 workspaces.
template <bool CLUSTER>
struct RefinedTeamSolve32 {
  static __device__ void run(const InstanceDev& I, const Team<CLUSTER>& tm, double* w, double* t) {
    const int T = tm.tid(), NT = tm.count(), n3 = 3 * I.n;
    float* Y = I.y32;
    float* Z = I.t32;
    for (int i = T; i < n3; i += NT) Y[i] = static_cast<float>(tm.ld(w + i));
    tm.sync();
    TeamSolve32<CLUSTER>::run(I, tm, Y, Z);  // Y ← x₀
    // r = b − Ã·x₀ per row in FP64 (Ã in elimination order), into Z; x₀ kept in t
    for (int i = T; i < I.n; i += NT) {
      double r0 = tm.ld(w + 3 * i), r1 = tm.ld(w + 3 * i + 1), r2 = tm.ld(w + 3 * i + 2);
#pragma unroll 4
      for (int p = I.Aptr[i]; p < I.Aptr[i + 1]; ++p) {
        const int j = I.Acol[p];
        const double a = -I.Aval[p];
        r0 = fma(a, static_cast<double>(tm.ld(Y + 3 * j)), r0);
        r1 = fma(a, static_cast<double>(tm.ld(Y + 3 * j + 1)), r1);
        r2 = fma(a, static_cast<double>(tm.ld(Y + 3 * j + 2)), r2);
      }
      t[3 * i] = static_cast<double>(tm.ld(Y + 3 * i));
      t[3 * i + 1] = static_cast<double>(tm.ld(Y + 3 * i + 1));
      t[3 * i + 2] = static_cast<double>(tm.ld(Y + 3 * i + 2));
      Z[3 * i] = static_cast<float>(r0);
      Z[3 * i + 1] = static_cast<float>(r1);
      Z[3 * i + 2] = static_cast<float>(r2);
    }
    tm.sync();
    TeamSolve32<CLUSTER>::run(I, tm, Z, Y);  // Z ← solve₃₂(r), Y the temporary
    for (int i = T; i < n3; i += NT) w[i] = tm.ld(t + i) + static_cast<double>(tm.ld(Z + i));
    tm.sync();
  }
};

// The grid's team-maximum slots live in the instance's x0 workspace (2 × CTAs doubles, which the
// planner caps to fit its 3n), as in the FP64 grid kernel; w and t are the FP64 workspaces.
template <bool TIMED>
__global__ void __launch_bounds__(kBlockThreads) substepMixedGridKernel(const InstanceDev* __restrict__ insts,
                                                                        int substeps) {
  __shared__ double red[32];
  __shared__ double slots[2];
  const InstanceDev& I = insts[0];
  Team<true> tm{static_cast<int>(blockIdx.x), static_cast<int>(gridDim.x)};
  tm.gslots = I.x0;
  runSubstepsTeam<true, TIMED, RefinedTeamSolve32<true>>(I, tm, substeps, I.w, I.tbuf, red, slots);
}

}  // namespace

int mixedGridCapacity() {
  static int cached = -1;
  if (cached >= 0) return cached;
  int dev = 0, sms = 0, least = 1 << 30;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return cached = 0;
  }
  for (auto kernel : {substepMixedGridKernel<false>, substepMixedGridKernel<true>}) {  // both must fit
    int perSm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kernel, kBlockThreads, 0) != cudaSuccess) {
      cudaGetLastError();
      return cached = 0;
    }
    least = std::min(least, perSm);
  }
  return cached = least * sms;
}

int launchSubstepMixedGrid(const InstanceDev* d, int ctas, int substeps, void* stream, bool timed) {
  if (substeps <= 0) return 0;
  if (ctas < 2 || ctas > mixedGridCapacity()) return static_cast<int>(cudaErrorCooperativeLaunchTooLarge);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ctas);
  cfg.blockDim = dim3(kBlockThreads);
  cfg.stream = static_cast<cudaStream_t>(stream);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const cudaError_t e = timed ? cudaLaunchKernelEx(&cfg, substepMixedGridKernel<true>, d, substeps)
                              : cudaLaunchKernelEx(&cfg, substepMixedGridKernel<false>, d, substeps);
  return static_cast<int>(e != cudaSuccess ? e : cudaGetLastError());
}

}  // namespace pdg
