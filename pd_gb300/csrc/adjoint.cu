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
// 3·S·K solves. One CTA per cloth runs it all with the FP64 supernodal solve; a batch of problems
// is one launch.
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

// One substep of the differentiable map from (J.x, J.v) in place; it[k] receives x^k if given.
__device__ void forwardSubstep(const InstanceDev& J, const GradDev& G, const Team<false>& tm, double* w, double* t,
                               double* it) {
  const int n = J.n;
  const double h2 = J.h * J.h;
  for (int v = threadIdx.x; v < n; v += blockDim.x) {  // predict with the external force
    const double m = J.m[v];
    const double mh2 = m * J.invH2;
    for (int c = 0; c < 3; ++c) {
      const double p = J.x[3 * v + c];
      double xh = (p + J.v[3 * v + c] * J.h) + J.gh2[c];
      if (G.force && m > 0.0) xh = fma(G.force[3 * v + c], h2 / m, xh);
      J.xn[3 * v + c] = p;
      J.xhat[3 * v + c] = xh;
      J.bbase[3 * v + c] = mh2 * xh;
      if (it) it[3 * v + c] = p;
    }
  }
  for (int e = threadIdx.x; e < J.ne; e += blockDim.x) edgeTerms(J, tm, J.x, e, false);
  __syncthreads();
  for (int k = 0; k < J.maxIter; ++k) {
    for (int v = threadIdx.x; v < n; v += blockDim.x) gatherRow(J, tm, v, w);
    __syncthreads();
    TeamSolve<false>::run(J, tm, w, t);
    for (int v = threadIdx.x; v < n; v += blockDim.x) {
      const int r = J.iperm[v];
      for (int c = 0; c < 3; ++c) {
        J.x[3 * v + c] = w[3 * r + c];
        if (it) it[(size_t)(k + 1) * 3 * n + 3 * v + c] = w[3 * r + c];
      }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < J.ne; e += blockDim.x) edgeTerms(J, tm, J.x, e, false);
    __syncthreads();
  }
  for (int v = threadIdx.x; v < n; v += blockDim.x) {  // velocity, damping, pin resnap
    for (int c = 0; c < 3; ++c) {
      if (J.pinned[v]) {
        J.v[3 * v + c] = 0.0;
        J.x[3 * v + c] = J.q[3 * v + c];
      } else {
        J.v[3 * v + c] = (J.x[3 * v + c] - J.xn[3 * v + c]) * J.dampInvH;
      }
    }
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kBlockThreads) gradientKernel(const InstanceDev* __restrict__ insts,
                                                               const GradDev* __restrict__ grads, int substeps,
                                                               int smemBytes) {
  extern __shared__ double smem[];
  __shared__ double red[32];
  const GradDev& G = grads[blockIdx.x];
  InstanceDev J = insts[blockIdx.x];  // the instance with its state redirected to the work arrays
  J.x = G.xs;
  J.v = G.vs;
  const int n = J.n, n3 = 3 * n, K = J.maxIter;
  const bool inSmem = 6 * n * static_cast<int>(sizeof(double)) <= smemBytes;
  double* w = inSmem ? smem : J.w;
  double* t = inSmem ? smem + n3 : J.tbuf;
  const Team<false> tm{0, 1};
  const InstanceDev& I = insts[blockIdx.x];
  for (int i = threadIdx.x; i < n3; i += blockDim.x) {
    G.xs[i] = I.x[i];
    G.vs[i] = I.v[i];
  }
  __syncthreads();
  const size_t itStride = static_cast<size_t>(K + 1) * n3;
  for (int s = 0; s < substeps; ++s) {
    if (!G.itAll) {
      for (int i = threadIdx.x; i < n3; i += blockDim.x) {
        G.ckX[(size_t)s * n3 + i] = G.xs[i];
        G.ckV[(size_t)s * n3 + i] = G.vs[i];
      }
      __syncthreads();
    }
    forwardSubstep(J, G, tm, w, t, G.itAll ? G.itAll + s * itStride : nullptr);
  }
  // loss and its gradient w.r.t. the final positions
  double l = 0.0, nfree = 0.0;
  for (int v = threadIdx.x; v < n; v += blockDim.x) {
    if (J.pinned[v]) continue;
    nfree += 1.0;
    for (int c = 0; c < 3; ++c) {
      const double d = G.xs[3 * v + c] - G.target[3 * v + c];
      l = fma(d, d, l);
    }
  }
  l = blockSum(l, red);
  nfree = blockSum(nfree, red);
  if (threadIdx.x == 0) *G.loss = nfree > 0.0 ? l / nfree : 0.0;
  if (!G.wantGrad) return;
  for (int v = threadIdx.x; v < n; v += blockDim.x) {
    for (int c = 0; c < 3; ++c) {
      const int i = 3 * v + c;
      G.xb[i] = J.pinned[v] ? 0.0 : 2.0 * (G.xs[i] - G.target[i]) / nfree;
      G.vb[i] = 0.0;
      G.fb[i] = 0.0;
    }
  }
  for (int e = threadIdx.x; e < J.ne; e += blockDim.x) G.kb[e] = 0.0;
  __syncthreads();
  for (int s = substeps - 1; s >= 0; --s) {
    const double* its = G.itAll ? G.itAll + s * itStride : G.it;  // x^0 .. x^K of substep s
    if (!G.itAll) {
      for (int i = threadIdx.x; i < n3; i += blockDim.x) {
        G.xs[i] = G.ckX[(size_t)s * n3 + i];
        G.vs[i] = G.ckV[(size_t)s * n3 + i];
      }
      __syncthreads();
      forwardSubstep(J, G, tm, w, t, G.it);
    }
    for (int v = threadIdx.x; v < n; v += blockDim.x) {
      const bool p = J.pinned[v] != 0;
      for (int c = 0; c < 3; ++c) {
        const int i = 3 * v + c;
        G.xkb[i] = p ? 0.0 : fma(J.dampInvH, G.vb[i], G.xb[i]);
        G.xnb[i] = p ? 0.0 : -J.dampInvH * G.vb[i];
        G.xhb[i] = 0.0;
      }
    }
    __syncthreads();
    for (int k = K - 1; k >= 0; --k) {
      // λ = L⁻¹·x̄^{k+1} (pinned rows zero), in elimination order in w
      for (int v = threadIdx.x; v < n; v += blockDim.x) {
        const int r = J.iperm[v];
        for (int c = 0; c < 3; ++c) w[3 * r + c] = G.xkb[3 * v + c];
      }
      __syncthreads();
      TeamSolve<false>::run(J, tm, w, t);
      for (int v = threadIdx.x; v < n; v += blockDim.x) {
        if (J.pinned[v]) continue;
        const double mh2 = J.m[v] * J.invH2;
        const int r = J.iperm[v];
        for (int c = 0; c < 3; ++c) G.xhb[3 * v + c] = fma(mh2, w[3 * r + c], G.xhb[3 * v + c]);
      }
      const double* xk = its + (size_t)k * n3;
      const double* xk1 = its + (size_t)(k + 1) * n3;
      for (int e = threadIdx.x; e < J.ne; e += blockDim.x) {
        const int a = J.eab[2 * e], b = J.eab[2 * e + 1];
        const bool ap = J.pinned[a] != 0, bp = J.pinned[b] != 0;
        double g0 = 0.0, g1 = 0.0, g2 = 0.0, kbe = 0.0;
        if (!(ap && bp)) {
          const int ra = J.iperm[a], rb = J.iperm[b];
          const double l0 = (ap ? 0.0 : w[3 * ra]) - (bp ? 0.0 : w[3 * rb]);
          const double l1 = (ap ? 0.0 : w[3 * ra + 1]) - (bp ? 0.0 : w[3 * rb + 1]);
          const double l2 = (ap ? 0.0 : w[3 * ra + 2]) - (bp ? 0.0 : w[3 * rb + 2]);
          const double r0 = xk[3 * a] - xk[3 * b], r1 = xk[3 * a + 1] - xk[3 * b + 1], r2 = xk[3 * a + 2] - xk[3 * b + 2];
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
          const double q0 = xk1[3 * a] - xk1[3 * b], q1 = xk1[3 * a + 1] - xk1[3 * b + 1],
                       q2 = xk1[3 * a + 2] - xk1[3 * b + 2];
          kbe = l0 * (d0 - q0) + l1 * (d1 - q1) + l2 * (d2 - q2);
        }
        G.kb[e] += kbe;
        G.ge[3 * e] = g0;
        G.ge[3 * e + 1] = g1;
        G.ge[3 * e + 2] = g2;
      }
      __syncthreads();
      for (int v = threadIdx.x; v < n; v += blockDim.x) {  // x̄^k, gathered per vertex
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        if (!J.pinned[v]) {
          for (int q = J.rstart[v]; q < J.rstart[v + 1]; ++q) {
            const int p = J.rinc[q];
            const int e = p >> 1;
            const double sg = (p & 1) ? -1.0 : 1.0;
            a0 = fma(sg, G.ge[3 * e], a0);
            a1 = fma(sg, G.ge[3 * e + 1], a1);
            a2 = fma(sg, G.ge[3 * e + 2], a2);
          }
        }
        G.xkb[3 * v] = a0;
        G.xkb[3 * v + 1] = a1;
        G.xkb[3 * v + 2] = a2;
      }
      __syncthreads();
    }
    // x^0 = x_n and x̂ = x_n + h·v_n + h²·g + h²·f/m
    const double h2 = J.h * J.h;
    for (int v = threadIdx.x; v < n; v += blockDim.x) {
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
    __syncthreads();
  }
}

}  // namespace

int launchGradient(const InstanceDev* d, const GradDev* g, int count, int substeps, int smemBytes, void* stream) {
  if (count <= 0) return 0;
  static bool attrSet = false;
  if (!attrSet) {
    cudaFuncSetAttribute(gradientKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attrSet = true;
  }
  gradientKernel<<<count, kBlockThreads, smemBytes, static_cast<cudaStream_t>(stream)>>>(d, g, substeps, smemBytes);
  return static_cast<int>(cudaGetLastError());
}

}  // namespace pdg
