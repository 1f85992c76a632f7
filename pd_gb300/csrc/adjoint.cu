// adjoint.cu — loss and gradient of the substep sequence by the adjoint method, FP64.
//
// The differentiable map is the reference's stepOnce (Integrator.cpp:312-797) with the iteration
// count fixed at max_iterations (the convergence gate is not differentiable) and an optional
// external per-vertex force f entering the prediction as x̂ = x + h·v + h²·g + h²·f/m. The loss is
// the mean over free vertices of |x_S − target|² after S substeps. Gradients: per-edge stiffness
// κ_e, initial velocities v_0 and f.
//
// Reverse mode through one PD iteration x^{k+1} = L⁻¹·b(x^k), b = (M/h²)·x̂ + Σ_e κ_e·S_eᵀ·d_e(x^k)
// (+ pins), with L = M/h² + Σ_e κ_e·S_eᵀS_e (+ bends) symmetric, so one solve with the same factor:
//   λ = L⁻¹·x̄^{k+1};  x̂̄ += (M/h²)·λ;
//   x̄^k_v = Σ_{e∋v} ±κ_e·J_e·(λ_a − λ_b),  J_e = ∂d_e/∂rel = ℓ_e/‖rel‖·(I − r̂r̂ᵀ);
//   κ̄_e += (λ_a − λ_b)·(d_e(x^k) − (x^{k+1}_a − x^{k+1}_b))   (∂b/∂κ_e and ∂L/∂κ_e),
// with pinned vertices at q and λ = 0 on pinned rows (they are identity rows of L). The
// velocity update v' = (x^K − x_n)·(1 − k_d)/h and the prediction chain the rest.
//
// Memory: when HBM allows (S·(K+1)·24n bytes a problem, 130 MB for 64² × 120 substeps × 10
// iterations) the forward pass stores every iterate and the reverse pass only reads them: 2·S·K
// solves a gradient. Otherwise the forward pass stores (x, v) at the start of every substep
// (S·48n bytes) and the reverse pass recomputes each substep's K iterates from its checkpoint:
// 3·S·K solves. A problem is run by one CTA or by a thread-block cluster (the FP64 supernodal
// solve strided over the cluster, vectors in L2, sums through distributed shared memory); a batch
// of problems is one launch.
#include "device.cuh"
#include "substep_team.cuh"

namespace pdg {

namespace {

__device__ __forceinline__ double blockSum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) s += red[w];
  return s;
}

// Sum over the team (CTA sums added in rank order, so every CTA gets the same bits). `slots` is
// a 2-entry shared array used alternately, as in teamMax.
template <bool CLUSTER>
__device__ __forceinline__ double teamSum(const Team<CLUSTER>& tm, double v, double* red, double* slots,
                                          int& parity) {
  v = blockSum(v, red);
  if (!CLUSTER) return v;
  double* slot = slots + parity;
  parity ^= 1;
  if (threadIdx.x == 0) *slot = v;
  cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
  cl.sync();
  double s = 0.0;
  for (int r = 0; r < tm.size; ++r) s += *cl.map_shared_rank(slot, r);
  return s;
}

// One substep of the differentiable map from (J.x, J.v) in place; it[k] receives x^k if given.
template <bool CLUSTER>
__device__ void forwardSubstep(const InstanceDev& J, const GradDev& G, const Team<CLUSTER>& tm, double* w, double* t,
                               double* it) {
  const int n = J.n, T = tm.tid(), NT = tm.count();
  const double h2 = J.h * J.h;
  for (int v = T; v < n; v += NT) {  // predict with the external force
    const double m = J.m[v];
    const double mh2 = m * J.invH2;
    for (int c = 0; c < 3; ++c) {
      const double p = tm.ld(J.x + 3 * v + c);
      double xh = (p + tm.ld(J.v + 3 * v + c) * J.h) + J.gh2[c];
      if (G.force && m > 0.0) xh = fma(G.force[3 * v + c], h2 / m, xh);
      J.xn[3 * v + c] = p;
      J.xhat[3 * v + c] = xh;
      J.bbase[3 * v + c] = mh2 * xh;
      if (it) it[3 * v + c] = p;
    }
  }
  tm.sync();
  for (int e = T; e < J.ne; e += NT) edgeTerms(J, tm, J.x, e, false);
  tm.sync();
  for (int k = 0; k < J.maxIter; ++k) {
    for (int v = T; v < n; v += NT) gatherRow(J, tm, v, w);
    tm.sync();
    TeamSolve<CLUSTER>::run(J, tm, w, t);
    for (int v = T; v < n; v += NT) {
      const int r = J.iperm[v];
      for (int c = 0; c < 3; ++c) {
        const double x = tm.ld(w + 3 * r + c);
        J.x[3 * v + c] = x;
        if (it) it[(size_t)(k + 1) * 3 * n + 3 * v + c] = x;
      }
    }
    tm.sync();
    for (int e = T; e < J.ne; e += NT) edgeTerms(J, tm, J.x, e, false);
    tm.sync();
  }
  for (int v = T; v < n; v += NT) {  // velocity, damping, pin resnap
    for (int c = 0; c < 3; ++c) {
      if (J.pinned[v]) {
        J.v[3 * v + c] = 0.0;
        J.x[3 * v + c] = J.q[3 * v + c];
      } else {
        J.v[3 * v + c] = (tm.ld(J.x + 3 * v + c) - tm.ld(J.xn + 3 * v + c)) * J.dampInvH;
      }
    }
  }
  tm.sync();
}

// Loss and gradients of one problem by a team; w, t: the solve's vectors (shared memory for one
// CTA, the instance's L2 workspaces for a cluster).
template <bool CLUSTER>
__device__ void gradientOf(const InstanceDev& I, const GradDev& G, const Team<CLUSTER>& tm, int substeps, double* w,
                           double* t, double* red, double* slots) {
  InstanceDev J = I;  // the instance with its state redirected to the work arrays
  J.x = G.xs;
  J.v = G.vs;
  const int n = J.n, n3 = 3 * n, K = J.maxIter;
  const int T = tm.tid(), NT = tm.count();
  int parity = 0;
  for (int i = T; i < n3; i += NT) {
    G.xs[i] = I.x[i];
    G.vs[i] = I.v[i];
  }
  tm.sync();
  const size_t itStride = static_cast<size_t>(K + 1) * n3;
  for (int s = 0; s < substeps; ++s) {
    if (!G.itAll) {
      for (int i = T; i < n3; i += NT) {
        G.ckX[(size_t)s * n3 + i] = tm.ld(G.xs + i);
        G.ckV[(size_t)s * n3 + i] = tm.ld(G.vs + i);
      }
      tm.sync();
    }
    forwardSubstep(J, G, tm, w, t, G.itAll ? G.itAll + s * itStride : nullptr);
  }
  // loss and its gradient w.r.t. the final positions
  double l = 0.0, nfree = 0.0;
  for (int v = T; v < n; v += NT) {
    if (J.pinned[v]) continue;
    nfree += 1.0;
    for (int c = 0; c < 3; ++c) {
      const double d = tm.ld(G.xs + 3 * v + c) - G.target[3 * v + c];
      l = fma(d, d, l);
    }
  }
  l = teamSum(tm, l, red, slots, parity);
  nfree = teamSum(tm, nfree, red, slots, parity);
  if (T == 0) *G.loss = nfree > 0.0 ? l / nfree : 0.0;
  if (!G.wantGrad) return;
  for (int v = T; v < n; v += NT) {
    for (int c = 0; c < 3; ++c) {
      const int i = 3 * v + c;
      G.xb[i] = J.pinned[v] ? 0.0 : 2.0 * (tm.ld(G.xs + i) - G.target[i]) / nfree;
      G.vb[i] = 0.0;
      G.fb[i] = 0.0;
    }
  }
  for (int e = T; e < J.ne; e += NT) G.kb[e] = 0.0;
  tm.sync();
  for (int s = substeps - 1; s >= 0; --s) {
    const double* its = G.itAll ? G.itAll + s * itStride : G.it;  // x^0 .. x^K of substep s
    if (!G.itAll) {
      for (int i = T; i < n3; i += NT) {
        G.xs[i] = G.ckX[(size_t)s * n3 + i];
        G.vs[i] = G.ckV[(size_t)s * n3 + i];
      }
      tm.sync();
      forwardSubstep(J, G, tm, w, t, G.it);
    }
    for (int v = T; v < n; v += NT) {
      const bool p = J.pinned[v] != 0;
      for (int c = 0; c < 3; ++c) {
        const int i = 3 * v + c;
        G.xkb[i] = p ? 0.0 : fma(J.dampInvH, G.vb[i], G.xb[i]);
        G.xnb[i] = p ? 0.0 : -J.dampInvH * G.vb[i];
        G.xhb[i] = 0.0;
      }
    }
    tm.sync();
    for (int k = K - 1; k >= 0; --k) {
      // λ = L⁻¹·x̄^{k+1} (pinned rows zero), in elimination order in w
      for (int v = T; v < n; v += NT) {
        const int r = J.iperm[v];
        for (int c = 0; c < 3; ++c) w[3 * r + c] = G.xkb[3 * v + c];
      }
      tm.sync();
      TeamSolve<CLUSTER>::run(J, tm, w, t);
      for (int v = T; v < n; v += NT) {
        if (J.pinned[v]) continue;
        const double mh2 = J.m[v] * J.invH2;
        const int r = J.iperm[v];
        for (int c = 0; c < 3; ++c) G.xhb[3 * v + c] = fma(mh2, tm.ld(w + 3 * r + c), G.xhb[3 * v + c]);
      }
      const double* xk = its + (size_t)k * n3;
      const double* xk1 = its + (size_t)(k + 1) * n3;
      for (int e = T; e < J.ne; e += NT) {
        const int a = J.eab[2 * e], b = J.eab[2 * e + 1];
        const bool ap = J.pinned[a] != 0, bp = J.pinned[b] != 0;
        double g0 = 0.0, g1 = 0.0, g2 = 0.0, kbe = 0.0;
        if (!(ap && bp)) {
          const int ra = J.iperm[a], rb = J.iperm[b];
          const double l0 = (ap ? 0.0 : tm.ld(w + 3 * ra)) - (bp ? 0.0 : tm.ld(w + 3 * rb));
          const double l1 = (ap ? 0.0 : tm.ld(w + 3 * ra + 1)) - (bp ? 0.0 : tm.ld(w + 3 * rb + 1));
          const double l2 = (ap ? 0.0 : tm.ld(w + 3 * ra + 2)) - (bp ? 0.0 : tm.ld(w + 3 * rb + 2));
          const double r0 = tm.ld(xk + 3 * a) - tm.ld(xk + 3 * b), r1 = tm.ld(xk + 3 * a + 1) - tm.ld(xk + 3 * b + 1),
                       r2 = tm.ld(xk + 3 * a + 2) - tm.ld(xk + 3 * b + 2);
          const double len = sqrt(r0 * r0 + r1 * r1 + r2 * r2);
          double d0 = 0.0, d1 = 0.0, d2 = 0.0;
          if (!(len <= 1e-12)) {
            const double s = J.erest[e] / len;
            d0 = r0 * s;
            d1 = r1 * s;
            d2 = r2 * s;
            const double u0 = r0 / len, u1 = r1 / len, u2 = r2 / len;
            const double ul = u0 * l0 + u1 * l1 + u2 * l2;
            const double ks = J.ek[e] * s;  // κ·J·λ_e = κ·(ℓ/len)·(λ_e − r̂(r̂·λ_e))
            g0 = ks * (l0 - u0 * ul);
            g1 = ks * (l1 - u1 * ul);
            g2 = ks * (l2 - u2 * ul);
          }
          const double q0 = tm.ld(xk1 + 3 * a) - tm.ld(xk1 + 3 * b), q1 = tm.ld(xk1 + 3 * a + 1) - tm.ld(xk1 + 3 * b + 1),
                       q2 = tm.ld(xk1 + 3 * a + 2) - tm.ld(xk1 + 3 * b + 2);
          kbe = l0 * (d0 - q0) + l1 * (d1 - q1) + l2 * (d2 - q2);
        }
        G.kb[e] += kbe;
        G.ge[3 * e] = g0;
        G.ge[3 * e + 1] = g1;
        G.ge[3 * e + 2] = g2;
      }
      tm.sync();
      for (int v = T; v < n; v += NT) {  // x̄^k, gathered per vertex
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        if (!J.pinned[v]) {
          for (int q = J.rstart[v]; q < J.rstart[v + 1]; ++q) {
            const int p = J.rinc[q];
            const int e = p >> 1;
            const double sg = (p & 1) ? -1.0 : 1.0;
            a0 = fma(sg, tm.ld(G.ge + 3 * e), a0);
            a1 = fma(sg, tm.ld(G.ge + 3 * e + 1), a1);
            a2 = fma(sg, tm.ld(G.ge + 3 * e + 2), a2);
          }
        }
        G.xkb[3 * v] = a0;
        G.xkb[3 * v + 1] = a1;
        G.xkb[3 * v + 2] = a2;
      }
      tm.sync();
    }
    // x^0 = x_n and x̂ = x_n + h·v_n + h²·g + h²·f/m
    const double h2 = J.h * J.h;
    for (int v = T; v < n; v += NT) {
      const bool p = J.pinned[v] != 0;
      const double m = J.m[v];
      for (int c = 0; c < 3; ++c) {
        const int i = 3 * v + c;
        if (p) {
          G.xb[i] = G.vb[i] = 0.0;
          continue;
        }
        G.xb[i] = G.xnb[i] + G.xkb[i] + G.xhb[i];
        G.vb[i] = J.h * G.xhb[i];
        if (m > 0.0) G.fb[i] = fma(h2 / m, G.xhb[i], G.fb[i]);
      }
    }
    tm.sync();
  }
}

__global__ void __launch_bounds__(kBlockThreads, 1) gradientKernel(const InstanceDev* __restrict__ insts,
                                                               const GradDev* __restrict__ grads, int substeps,
                                                               int smemBytes) {
  extern __shared__ double smem[];
  __shared__ double red[32];
  __shared__ double slots[2];
  const InstanceDev& I = insts[blockIdx.x];
  const bool inSmem = 6 * I.n * static_cast<int>(sizeof(double)) <= smemBytes;
  double* w = inSmem ? smem : I.w;
  double* t = inSmem ? smem + 3 * I.n : I.tbuf;
  const Team<false> tm{0, 1};
  gradientOf<false>(I, grads[blockIdx.x], tm, substeps, w, t, red, slots);
}

__global__ void __launch_bounds__(kBlockThreads, 1) gradientClusterKernel(const InstanceDev* __restrict__ insts,
                                                                      const GradDev* __restrict__ grads,
                                                                      int substeps) {
  __shared__ double red[32];
  __shared__ double slots[2];
  cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
  const int cs = static_cast<int>(cl.num_blocks());
  const int p = static_cast<int>(blockIdx.x) / cs;
  const InstanceDev& I = insts[p];
  const Team<true> tm{static_cast<int>(cl.block_rank()), cs};
  gradientOf<true>(I, grads[p], tm, substeps, I.w, I.tbuf, red, slots);
}

cudaLaunchConfig_t gradClusterConfig(int blocks, int clusterSize, void* stream, cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(kBlockThreads);
  cfg.dynamicSmemBytes = 0;
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

int gradClusterSupported(int want) {
  static int cached[17] = {0};
  if (want < 2 || want > 16) return 0;
  if (cached[want]) return cached[want] > 0 ? want : 0;
  if (want > 8) cudaFuncSetAttribute(gradientClusterKernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = gradClusterConfig(want, want, nullptr, attr);
  int clusters = 0;
  const cudaError_t e = cudaOccupancyMaxActiveClusters(&clusters, gradientClusterKernel, &cfg);
  if (e != cudaSuccess) cudaGetLastError();
  cached[want] = (e == cudaSuccess && clusters > 0) ? 1 : -1;
  return cached[want] > 0 ? want : 0;
}

int launchGradient(const InstanceDev* d, const GradDev* g, int count, int clusterSize, int substeps, int smemBytes,
                   void* stream) {
  if (count <= 0) return 0;
  if (clusterSize > 1) {
    if (gradClusterSupported(clusterSize) != clusterSize) return static_cast<int>(cudaErrorInvalidConfiguration);
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = gradClusterConfig(count * clusterSize, clusterSize, stream, attr);
    const cudaError_t e = cudaLaunchKernelEx(&cfg, gradientClusterKernel, d, g, substeps);
    return static_cast<int>(e != cudaSuccess ? e : cudaGetLastError());
  }
  static bool attrSet = false;
  if (!attrSet) {
    cudaFuncSetAttribute(gradientKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attrSet = true;
  }
  gradientKernel<<<count, kBlockThreads, smemBytes, static_cast<cudaStream_t>(stream)>>>(d, g, substeps, smemBytes);
  return static_cast<int>(cudaGetLastError());
}

}  // namespace pdg
