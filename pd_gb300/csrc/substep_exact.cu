// substep_exact.cu — the per-substep PD loop in the reference's exact FP64 arithmetic order.
//
// One block (256 threads) owns one cloth instance and runs whole substeps on it:
//   predict → [edge pass → colour-ordered gather of b → forward / backward level-scheduled
//   solves → unpack → edge pass → residual gather → gate]^K → velocity.
// Every product and sum uses __dmul_rn / __dadd_rn / __dsub_rn so no FMA contraction can
// occur, and every per-vertex / per-row sum runs in the reference's order, which makes the
// result bit-identical to the reference CPU path (core/sim/Integrator.cpp:312-797).
//
// GB300 note: FP64 issues at ~1.6 ops/clk/SM with ~64-cycle latency, so this kernel is bound
// by the FP64 pipe. Each edge projection (sqrt + divide) is therefore computed once per
// iteration and reused by the residual of iteration k and the scatter of iteration k+1, which
// read the same positions (the reference computes it in both places).
#include <cuda_runtime.h>

#include "device.cuh"

namespace pdg {
namespace {

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

// max over a block of non-negative values, NaN-skipping (reference: running std::max from 0)
__device__ double blockMax(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) red[0] = v;
  }
  __syncthreads();
  const double r = red[0];
  __syncthreads();
  return r;
}

// d_e = ℓ·(x_a − x_b)/‖x_a − x_b‖ (0 when degenerate), DistanceTerm.cpp:94-102.
// kd = κ·d (scatter term, DistanceTerm.cpp:121-152); rc = κ·rel − κ·d (Integrator.cpp:246-248).
__device__ void edgePass(const InstanceDev& I, bool wantRc) {
  for (int e = threadIdx.x; e < I.ne; e += blockDim.x) {
    const int a = I.eab[2 * e], b = I.eab[2 * e + 1];
    const double rx = dsub(I.x[3 * a], I.x[3 * b]);
    const double ry = dsub(I.x[3 * a + 1], I.x[3 * b + 1]);
    const double rz = dsub(I.x[3 * a + 2], I.x[3 * b + 2]);
    const double len = __dsqrt_rn(dadd(dadd(dmul(rx, rx), dmul(ry, ry)), dmul(rz, rz)));
    double dx = 0.0, dy = 0.0, dz = 0.0;
    if (!(len <= 1e-12)) {
      const double s = __ddiv_rn(I.erest[e], len);
      dx = dmul(rx, s);
      dy = dmul(ry, s);
      dz = dmul(rz, s);
    }
    const double k = I.ek[e];
    const double cx = dmul(dx, k), cy = dmul(dy, k), cz = dmul(dz, k);
    I.kd[3 * e] = cx;
    I.kd[3 * e + 1] = cy;
    I.kd[3 * e + 2] = cz;
    if (wantRc) {
      I.rc[3 * e] = dsub(dmul(rx, k), cx);
      I.rc[3 * e + 1] = dsub(dmul(ry, k), cy);
      I.rc[3 * e + 2] = dsub(dmul(rz, k), cz);
    }
  }
}

// b_v = bBase_v + bendRhs_v, then the edge terms in colour order (DistanceTerm.cpp:279-317),
// pinned rows = q (Assembler.cpp:319-332); written to w at the vertex's elimination position.
__device__ void gatherRhs(const InstanceDev& I, double* w) {
  for (int v = threadIdx.x; v < I.n; v += blockDim.x) {
    double b0, b1, b2;
    if (I.pinned[v]) {
      b0 = I.q[3 * v];
      b1 = I.q[3 * v + 1];
      b2 = I.q[3 * v + 2];
    } else {
      b0 = I.bbase[3 * v];
      b1 = I.bbase[3 * v + 1];
      b2 = I.bbase[3 * v + 2];
      if (I.hasBendRhs) {
        b0 = dadd(b0, I.bendRhs[3 * v]);
        b1 = dadd(b1, I.bendRhs[3 * v + 1]);
        b2 = dadd(b2, I.bendRhs[3 * v + 2]);
      } else {
        b0 = dadd(b0, 0.0);
        b1 = dadd(b1, 0.0);
        b2 = dadd(b2, 0.0);
      }
      for (int k = I.sstart[v]; k < I.sstart[v + 1]; ++k) {
        const int p = I.sinc[k];
        const int e = p >> 1;
        const int other = I.eab[2 * e + ((p & 1) ^ 1)];
        const double c0 = I.kd[3 * e], c1 = I.kd[3 * e + 1], c2 = I.kd[3 * e + 2];
        if ((p & 1) == 0) {  // v is endpoint a: b_a += κd
          b0 = dadd(b0, c0);
          b1 = dadd(b1, c1);
          b2 = dadd(b2, c2);
        } else {             // v is endpoint b: b_b −= κd
          b0 = dsub(b0, c0);
          b1 = dsub(b1, c1);
          b2 = dsub(b2, c2);
        }
        if (I.pinned[other]) {  // pin elimination: b_free += κ·q_pinned
          const double k = I.ek[e];
          b0 = dadd(b0, dmul(k, I.q[3 * other]));
          b1 = dadd(b1, dmul(k, I.q[3 * other + 1]));
          b2 = dadd(b2, dmul(k, I.q[3 * other + 2]));
        }
      }
    }
    const int r = I.iperm[v];
    w[3 * r] = b0;
    w[3 * r + 1] = b1;
    w[3 * r + 2] = b2;
  }
}

// Forward L·y = w (unit lower; each row subtracts in ascending column order, as the reference's
// column-scatter form does), then backward Lᵀ·x = D⁻¹·y (each column subtracts in ascending row
// order) — EigenDirectSolver.cpp:411-448. One thread per row, the three components together.
__device__ void solveExact(const InstanceDev& I, double* w) {
  for (int l = 0; l < I.nlevF; ++l) {
    const int beg = I.fwdPtr[l], end = I.fwdPtr[l + 1];
    for (int t = beg + threadIdx.x; t < end; t += blockDim.x) {
      const int r = I.fwdRows[t];
      double a0 = w[3 * r], a1 = w[3 * r + 1], a2 = w[3 * r + 2];
      for (int p = I.Lrp[r]; p < I.Lrp[r + 1]; ++p) {
        const int j = I.Lci[p];
        const double lv = I.Lrv[p];
        a0 = dsub(a0, dmul(lv, w[3 * j]));
        a1 = dsub(a1, dmul(lv, w[3 * j + 1]));
        a2 = dsub(a2, dmul(lv, w[3 * j + 2]));
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
      double a0 = dmul(w[3 * k], di), a1 = dmul(w[3 * k + 1], di), a2 = dmul(w[3 * k + 2], di);
      for (int p = I.Lcp[k]; p < I.Lcp[k + 1]; ++p) {
        const int i = I.Lri[p];
        const double lv = I.Lcv[p];
        a0 = dsub(a0, dmul(lv, w[3 * i]));
        a1 = dsub(a1, dmul(lv, w[3 * i + 1]));
        a2 = dsub(a2, dmul(lv, w[3 * i + 2]));
      }
      w[3 * k] = a0;
      w[3 * k + 1] = a1;
      w[3 * k + 2] = a2;
    }
    __syncthreads();
  }
}

__device__ __forceinline__ double maxAbs3(double a, double b, double c) {
  return fmax(fabs(a), fmax(fabs(b), fabs(c)));
}

// Nonlinear residual of vertex v at the current positions (Integrator.cpp:230-263).
__device__ double vertexResidual(const InstanceDev& I, int v) {
  double f0 = 0.0, f1 = 0.0, f2 = 0.0;
  for (int k = I.rstart[v]; k < I.rstart[v + 1]; ++k) {
    const int p = I.rinc[k];
    const int e = p >> 1;
    if ((p & 1) == 0) {
      f0 = dadd(f0, I.rc[3 * e]);
      f1 = dadd(f1, I.rc[3 * e + 1]);
      f2 = dadd(f2, I.rc[3 * e + 2]);
    } else {
      f0 = dsub(f0, I.rc[3 * e]);
      f1 = dsub(f1, I.rc[3 * e + 1]);
      f2 = dsub(f2, I.rc[3 * e + 2]);
    }
  }
  double g0 = 0.0, g1 = 0.0, g2 = 0.0;
  for (int k = I.bstart[v]; k < I.bstart[v + 1]; ++k) {
    const int s = I.binc[k];
    const int a = I.babc[3 * s], b = I.babc[3 * s + 1], c = I.babc[3 * s + 2];
    const double fac = I.bfac[k];
    const double s0 = dadd(dsub(I.x[3 * a], dmul(2.0, I.x[3 * b])), I.x[3 * c]);
    const double s1 = dadd(dsub(I.x[3 * a + 1], dmul(2.0, I.x[3 * b + 1])), I.x[3 * c + 1]);
    const double s2 = dadd(dsub(I.x[3 * a + 2], dmul(2.0, I.x[3 * b + 2])), I.x[3 * c + 2]);
    g0 = dadd(g0, dmul(s0, fac));
    g1 = dadd(g1, dmul(s1, fac));
    g2 = dadd(g2, dmul(s2, fac));
  }
  f0 = dadd(f0, g0);
  f1 = dadd(f1, g1);
  f2 = dadd(f2, g2);
  const double mass = I.m[v];
  const double mh2 = dmul(mass, I.invH2);
  const double t0 = dadd(dmul(dsub(I.x[3 * v], I.xhat[3 * v]), mh2), f0);
  const double t1 = dadd(dmul(dsub(I.x[3 * v + 1], I.xhat[3 * v + 1]), mh2), f1);
  const double t2 = dadd(dmul(dsub(I.x[3 * v + 2], I.xhat[3 * v + 2]), mh2), f2);
  const double len = __dsqrt_rn(dadd(dadd(dmul(t0, t0), dmul(t1, t1)), dmul(t2, t2)));
  return __ddiv_rn(len, mass);
}

__global__ void __launch_bounds__(kBlockThreads) substepExactKernel(const InstanceDev* __restrict__ insts,
                                                                    int substeps, int smemBytes) {
  extern __shared__ double smem[];
  __shared__ double red[32];
  __shared__ int flag;
  const InstanceDev& I = insts[blockIdx.x];
  double* w = (3 * I.n * (int)sizeof(double) <= smemBytes) ? smem : I.w;

  for (int step = 0; step < substeps; ++step) {
    // predict x̂ = x + h·v + h²·g, x_n = x, bBase = (M/h²)·x̂ (Integrator.cpp:447-472)
    // The displacement scale max|x̂ − x_n|∞ is the same in every iteration of the substep.
    double scale = 0.0;
    for (int v = threadIdx.x; v < I.n; v += blockDim.x) {
      const double mh2 = dmul(I.m[v], I.invH2);
      double d[3];
      for (int c = 0; c < 3; ++c) {
        const double p = I.x[3 * v + c];
        const double xh = dadd(dadd(p, dmul(I.v[3 * v + c], I.h)), I.gh2[c]);
        I.xn[3 * v + c] = p;
        I.xhat[3 * v + c] = xh;
        I.bbase[3 * v + c] = dmul(mh2, xh);
        d[c] = dsub(xh, p);
      }
      scale = fmax(scale, maxAbs3(d[0], d[1], d[2]));
    }
    scale = blockMax(scale, red);
    scale = (scale < I.gScaleHH) ? I.gScaleHH : scale;

    edgePass(I, false);  // projection of x_n for the first scatter
    __syncthreads();
    int used = 0;
    bool conv = false;
    double lastRes = I.useResidual ? 0.0 : -1.0;
    for (int k = 0; k < I.maxIter; ++k) {
      gatherRhs(I, w);
      __syncthreads();
      solveExact(I, w);
      // unpack + displacement scan (Integrator.cpp:618-663)
      double diff = 0.0;
      for (int v = threadIdx.x; v < I.n; v += blockDim.x) {
        const int r = I.iperm[v];
        const double x0 = w[3 * r], x1 = w[3 * r + 1], x2 = w[3 * r + 2];
        diff = fmax(diff, maxAbs3(dsub(x0, I.x[3 * v]), dsub(x1, I.x[3 * v + 1]), dsub(x2, I.x[3 * v + 2])));
        I.x[3 * v] = x0;
        I.x[3 * v + 1] = x1;
        I.x[3 * v + 2] = x2;
      }
      __syncthreads();
      edgePass(I, I.useResidual != 0);
      __syncthreads();
      double res = 0.0;
      if (I.useResidual) {
        for (int v = threadIdx.x; v < I.n; v += blockDim.x) {
          if (I.pinned[v] || !(I.m[v] > 0.0)) continue;
          const double r = vertexResidual(I, v);
          if (r > res) res = r;
        }
        res = blockMax(res, red);
      }
      diff = blockMax(diff, red);
      // gate (Integrator.cpp:676-747)
      if (threadIdx.x == 0) {
        const double rel = (scale > 0.0) ? __ddiv_rn(diff, scale) : diff;
        const bool absHit = (I.absTol > 0.0) && (diff <= I.absTol);
        const bool relHit = (I.relTol > 0.0) && (rel <= I.relTol);
        bool c;
        if (I.useResidual) c = (res <= I.resThreshold);
        else c = absHit || relHit;
        flag = c ? 1 : 0;
      }
      __syncthreads();
      used = k + 1;
      lastRes = I.useResidual ? res : -1.0;
      conv = flag != 0;
      __syncthreads();
      if (conv) break;
    }
    // velocity, damping, pin resnap (Integrator.cpp:774-791)
    for (int v = threadIdx.x; v < I.n; v += blockDim.x) {
      if (I.pinned[v]) {
        for (int c = 0; c < 3; ++c) {
          I.v[3 * v + c] = 0.0;
          I.x[3 * v + c] = I.q[3 * v + c];
        }
      } else {
        for (int c = 0; c < 3; ++c) I.v[3 * v + c] = dmul(dsub(I.x[3 * v + c], I.xn[3 * v + c]), I.dampInvH);
      }
    }
    if (threadIdx.x == 0) {
      if (I.iterLog) I.iterLog[step] = used;
      if (I.convLog) I.convLog[step] = conv ? 1 : 0;
      *I.lastResidual = lastRes;
      *I.iterationsUsed = used;
      *I.converged = conv ? 1 : 0;
      if (conv) *I.earlyExits += 1;
    }
    __syncthreads();
  }
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
  solveExact(I, w);
  for (int v = threadIdx.x; v < I.n; v += blockDim.x) {
    const int r = I.iperm[v];
    x[3 * v] = w[3 * r];
    x[3 * v + 1] = w[3 * r + 1];
    x[3 * v + 2] = w[3 * r + 2];
  }
}

}  // namespace

int launchSubstepExact(const InstanceDev* d, int count, int substeps, int smemBytes, void* stream) {
  if (count <= 0 || substeps <= 0) return 0;
  static bool attrSet = false;
  if (!attrSet) {
    cudaFuncSetAttribute(substepExactKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attrSet = true;
  }
  substepExactKernel<<<count, kBlockThreads, smemBytes, static_cast<cudaStream_t>(stream)>>>(d, substeps, smemBytes);
  return static_cast<int>(cudaGetLastError());
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
