// spectrum.cu — spectrum of the linearised PD iteration by power iteration on the GPU (the
// reference's _verify/iteration_spectrum.cpp:126-338, a convergence diagnostic).
//
// At the instance's current positions the PD map x ← A⁻¹(M x̂/h² + Σ κ A_eᵀ d_e(x)) linearises to
// e ← T e with T = I − A⁻¹(M/h² + N + K_b): N = Σ_e κ_e A_eᵀ(n_e n_eᵀ)A_e, n_e = unit(x_a − x_b),
// and K_b = Σ_s k·A_sᵀA_s for the bending stencils, whose projection is constant (the reference's
// tool refuses bending scenes). B = I − T. Power iteration on T gives ρ(T), the predicted
// contraction per plain iteration; on B, λ_max(B); λ_min(B) = 1 − ρ(T) and the Chebyshev rate
// follow on the host. One team (a thread-block cluster, or one CTA) runs the whole iteration:
// matrix-free right-hand side gathered per vertex in edge order (the reference's summation order
// for a free vertex), the FP64 supernodal solve shared with the substep kernels, and deterministic
// team sums for the norms. Pinned rows of the right-hand side are zero, so pinned components
// stay zero (:255-262).
#include <cuda_runtime.h>

#include "substep_team.cuh"

namespace pdg {

namespace {

// Sum over the team of one value per thread: lane 0 of each warp, then CTAs in rank order —
// deterministic for a given launch shape.
template <bool CLUSTER>
__device__ double teamSum(const Team<CLUSTER>& tm, double v, double* red, double* slots, int& parity) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = (lane < static_cast<int>(blockDim.x >> 5)) ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[0] = v;
  }
  __syncthreads();
  const double r = red[0];
  __syncthreads();
  if (!CLUSTER) return r;
  double* slot = slots + parity;
  parity ^= 1;
  if (threadIdx.x == 0) *slot = r;
  cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
  cl.sync();
  double s = 0.0;
  for (int k = 0; k < tm.size; ++k) s += *cl.map_shared_rank(slot, k);
  return s;
}

struct SpectrumArgs {
  const double* x0;  // 3n start vector, zero on pinned vertices
  double* p;         // 3n current vector
  double* y;         // 3n next vector
  double* nE;        // 3E unit edge directions at the current positions
  double* out;       // ρ(T), its previous estimate, λ_max(B), its previous estimate
  int iters;
};

template <bool CLUSTER>
__device__ void spectrumRun(const InstanceDev& I, const Team<CLUSTER>& tm, const SpectrumArgs& a, double* red,
                            double* slots) {
  const int n = I.n;
  double* w = I.w;
  double* t = I.tbuf;
  int parity = 0;
  for (int e = tm.tid(); e < I.ne; e += tm.count()) {  // iteration_spectrum.cpp:133-142
    const int va = I.eab[2 * e], vb = I.eab[2 * e + 1];
    const double rx = I.x[3 * va] - I.x[3 * vb], ry = I.x[3 * va + 1] - I.x[3 * vb + 1];
    const double rz = I.x[3 * va + 2] - I.x[3 * vb + 2];
    const double len = sqrt(rx * rx + ry * ry + rz * rz);
    const double inv = len > 0.0 ? 1.0 / len : 0.0;
    a.nE[3 * e] = len > 0.0 ? rx * inv : 0.0;
    a.nE[3 * e + 1] = len > 0.0 ? ry * inv : 0.0;
    a.nE[3 * e + 2] = len > 0.0 ? rz * inv : 0.0;
  }
  for (int mode = 0; mode < 2; ++mode) {  // 0: T = I − B, 1: B
    for (int i = tm.tid(); i < 3 * n; i += tm.count()) a.p[i] = a.x0[i];
    tm.sync();
    double last = 0.0, prev = 0.0;
    for (int it = 0; it < a.iters; ++it) {
      // (M/h² + N + K_b)·p on free rows, zero on pinned rows, into w in elimination order
      for (int v = tm.tid(); v < n; v += tm.count()) {
        double r0 = 0.0, r1 = 0.0, r2 = 0.0;
        if (!I.pinned[v]) {
          const double d = I.m[v] * I.invH2;
          r0 = d * tm.ld(a.p + 3 * v);
          r1 = d * tm.ld(a.p + 3 * v + 1);
          r2 = d * tm.ld(a.p + 3 * v + 2);
          for (int k = I.rstart[v]; k < I.rstart[v + 1]; ++k) {  // edges in index order (:229-254)
            const int code = I.rinc[k], e = code >> 1;
            const double kap = I.ek[e];
            const double nx = tm.ld(a.nE + 3 * e), ny = tm.ld(a.nE + 3 * e + 1), nz = tm.ld(a.nE + 3 * e + 2);
            if (kap == 0.0 || (nx == 0.0 && ny == 0.0 && nz == 0.0)) continue;
            const int va = I.eab[2 * e], vb = I.eab[2 * e + 1];
            const double dx = tm.ld(a.p + 3 * va) - tm.ld(a.p + 3 * vb);
            const double dy = tm.ld(a.p + 3 * va + 1) - tm.ld(a.p + 3 * vb + 1);
            const double dz = tm.ld(a.p + 3 * va + 2) - tm.ld(a.p + 3 * vb + 2);
            const double dot = nx * dx + ny * dy + nz * dz;
            const double kd = kap * dot;
            if (code & 1) {
              r0 -= nx * kd;
              r1 -= ny * kd;
              r2 -= nz * kd;
            } else {
              r0 += nx * kd;
              r1 += ny * kd;
              r2 += nz * kd;
            }
          }
          for (int k = I.bstart[v]; k < I.bstart[v + 1]; ++k) {  // k·w_v·(A_s p), stencil order
            const int s = I.binc[k];
            const int sa = I.babc[3 * s], sb = I.babc[3 * s + 1], sc = I.babc[3 * s + 2];
            const double fac = I.bfac[k];
            r0 -= fac * (tm.ld(a.p + 3 * sa) - 2.0 * tm.ld(a.p + 3 * sb) + tm.ld(a.p + 3 * sc));
            r1 -= fac * (tm.ld(a.p + 3 * sa + 1) - 2.0 * tm.ld(a.p + 3 * sb + 1) + tm.ld(a.p + 3 * sc + 1));
            r2 -= fac * (tm.ld(a.p + 3 * sa + 2) - 2.0 * tm.ld(a.p + 3 * sb + 2) + tm.ld(a.p + 3 * sc + 2));
          }
        }
        const int r = I.iperm[v];
        w[3 * r] = r0;
        w[3 * r + 1] = r1;
        w[3 * r + 2] = r2;
      }
      tm.sync();
      TeamSolve<CLUSTER>::run(I, tm, w, t);
      double sy = 0.0, sp = 0.0;
      for (int v = tm.tid(); v < n; v += tm.count()) {
        const int r = I.iperm[v];
        for (int c = 0; c < 3; ++c) {
          const double sol = tm.ld(w + 3 * r + c), pv = tm.ld(a.p + 3 * v + c);
          const double yv = mode == 0 ? pv - sol : sol;
          a.y[3 * v + c] = yv;
          sy += yv * yv;
          sp += pv * pv;
        }
      }
      const double ny = sqrt(teamSum(tm, sy, red, slots, parity));
      const double np = sqrt(teamSum(tm, sp, red, slots, parity));
      if (!(ny > 0.0)) break;  // the same value in every thread: a uniform exit
      if (it >= a.iters - 20) {
        prev = last;
        last = ny / np;
      }
      for (int v = tm.tid(); v < n; v += tm.count())
        for (int c = 0; c < 3; ++c) a.p[3 * v + c] = a.y[3 * v + c] / ny;
      tm.sync();
    }
    if (tm.rank == 0 && threadIdx.x == 0) {
      a.out[2 * mode] = last;
      a.out[2 * mode + 1] = prev;
    }
    tm.sync();
  }
}

__global__ void __launch_bounds__(kBlockThreads) spectrumKernel(const InstanceDev* __restrict__ inst, SpectrumArgs a) {
  __shared__ double red[32];
  const Team<false> tm{0, 1};
  spectrumRun<false>(*inst, tm, a, red, nullptr);
}

__global__ void __launch_bounds__(kBlockThreads) spectrumClusterKernel(const InstanceDev* __restrict__ inst,
                                                                       SpectrumArgs a) {
  __shared__ double red[32];
  __shared__ double slots[2];
  cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
  const Team<true> tm{static_cast<int>(cl.block_rank()), static_cast<int>(cl.num_blocks())};
  spectrumRun<true>(*inst, tm, a, red, slots);
}

}  // namespace

int launchSpectrum(const InstanceDev* dInstance, const double* x0, double* p, double* y, double* nE, double* out,
                   int iters, int clusterSize, void* stream) {
  SpectrumArgs a{x0, p, y, nE, out, iters};
  if (clusterSize <= 1) {
    spectrumKernel<<<1, kBlockThreads, 0, static_cast<cudaStream_t>(stream)>>>(dInstance, a);
    return static_cast<int>(cudaGetLastError());
  }
  if (clusterSize > 8) cudaFuncSetAttribute(spectrumClusterKernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(clusterSize);
  cfg.blockDim = dim3(kBlockThreads);
  cfg.stream = static_cast<cudaStream_t>(stream);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = clusterSize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int clusters = 0;
  cudaError_t e = cudaOccupancyMaxActiveClusters(&clusters, spectrumClusterKernel, &cfg);
  if (e != cudaSuccess || clusters < 1) {  // this cluster size cannot run: one CTA
    cudaGetLastError();
    spectrumKernel<<<1, kBlockThreads, 0, static_cast<cudaStream_t>(stream)>>>(dInstance, a);
    return static_cast<int>(cudaGetLastError());
  }
  e = cudaLaunchKernelEx(&cfg, spectrumClusterKernel, dInstance, a);
  return static_cast<int>(e != cudaSuccess ? e : cudaGetLastError());
}

}  // namespace pdg
