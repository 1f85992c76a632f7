// substep_common.cuh — the per-substep PD loop shared by the FP64 kernels.
//
// One block owns one cloth instance and runs whole substeps:
//   predict → [gather of b in colour order → solve → unpack → edge pass → residual gather →
//   gate]^K → velocity,
// with the edge pass of x_n before the first iteration (reference: core/sim/Integrator.cpp:312-797).
// `A` is the arithmetic policy (ExactArith: every product and sum rounds on its own, as the
// reference; FastArith: the compiler may contract into FMA). `Solve` runs L x = b on the
// block's workspace w (elimination order, 3 doubles per row).
//
// GB300: FP64 issues at ~1.6 ops/clk/SM with ~64-cycle latency, so the edge projection (sqrt +
// divide) is computed once per iteration and reused by the residual of iteration k and by the
// scatter of iteration k+1, which read the same positions.
#pragma once

#include <cuda_runtime.h>

#include "device.cuh"

namespace pdg {

struct ExactArith {
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
  static __device__ __forceinline__ double sqrt(double a) { return __dsqrt_rn(a); }
};

struct FastArith {
  static __device__ __forceinline__ double mul(double a, double b) { return a * b; }
  static __device__ __forceinline__ double add(double a, double b) { return a + b; }
  static __device__ __forceinline__ double sub(double a, double b) { return a - b; }
  static __device__ __forceinline__ double div(double a, double b) { return a / b; }
  static __device__ __forceinline__ double sqrt(double a) { return ::sqrt(a); }
};

// max over the block of non-negative values, NaN-skipping (the reference's running std::max from 0)
__device__ __forceinline__ double blockMax(double v, double* red) {
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

__device__ __forceinline__ double maxAbs3(double a, double b, double c) {
  return fmax(fabs(a), fmax(fabs(b), fabs(c)));
}

// d_e = ℓ·(x_a − x_b)/‖x_a − x_b‖ (0 when degenerate), DistanceTerm.cpp:94-102;
// kd = κ·d (scatter term, DistanceTerm.cpp:121-152); rc = κ·rel − κ·d (Integrator.cpp:246-248).
// X: the positions (I.x, or I.xsol for the residual of an over-relaxed iteration).
template <class A>
__device__ void edgePass(const InstanceDev& I, const double* X, bool wantRc) {
  for (int e = threadIdx.x; e < I.ne; e += blockDim.x) {
    const int a = I.eab[2 * e], b = I.eab[2 * e + 1];
    const double rx = A::sub(X[3 * a], X[3 * b]);
    const double ry = A::sub(X[3 * a + 1], X[3 * b + 1]);
    const double rz = A::sub(X[3 * a + 2], X[3 * b + 2]);
    const double len = A::sqrt(A::add(A::add(A::mul(rx, rx), A::mul(ry, ry)), A::mul(rz, rz)));
    double dx = 0.0, dy = 0.0, dz = 0.0;
    if (!(len <= 1e-12)) {
      const double s = A::div(I.erest[e], len);
      dx = A::mul(rx, s);
      dy = A::mul(ry, s);
      dz = A::mul(rz, s);
    }
    const double k = I.ek[e];
    const double cx = A::mul(dx, k), cy = A::mul(dy, k), cz = A::mul(dz, k);
    I.kd[3 * e] = cx;
    I.kd[3 * e + 1] = cy;
    I.kd[3 * e + 2] = cz;
    if (wantRc) {
      I.rc[3 * e] = A::sub(A::mul(rx, k), cx);
      I.rc[3 * e + 1] = A::sub(A::mul(ry, k), cy);
      I.rc[3 * e + 2] = A::sub(A::mul(rz, k), cz);
    }
  }
}

// b_v = bBase_v + bendRhs_v, then the edge terms in colour order (DistanceTerm.cpp:279-317),
// pinned rows = q (Assembler.cpp:319-332); written to w at the vertex's elimination position.
template <class A>
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
        b0 = A::add(b0, I.bendRhs[3 * v]);
        b1 = A::add(b1, I.bendRhs[3 * v + 1]);
        b2 = A::add(b2, I.bendRhs[3 * v + 2]);
      } else {
        b0 = A::add(b0, 0.0);
        b1 = A::add(b1, 0.0);
        b2 = A::add(b2, 0.0);
      }
      for (int k = I.sstart[v]; k < I.sstart[v + 1]; ++k) {
        const int p = I.sinc[k];
        const int e = p >> 1;
        const int other = I.eab[2 * e + ((p & 1) ^ 1)];
        const double c0 = I.kd[3 * e], c1 = I.kd[3 * e + 1], c2 = I.kd[3 * e + 2];
        if ((p & 1) == 0) {  // v is endpoint a: b_a += κd
          b0 = A::add(b0, c0);
          b1 = A::add(b1, c1);
          b2 = A::add(b2, c2);
        } else {             // v is endpoint b: b_b −= κd
          b0 = A::sub(b0, c0);
          b1 = A::sub(b1, c1);
          b2 = A::sub(b2, c2);
        }
        if (I.pinned[other]) {  // pin elimination: b_free += κ·q_pinned
          const double k = I.ek[e];
          b0 = A::add(b0, A::mul(k, I.q[3 * other]));
          b1 = A::add(b1, A::mul(k, I.q[3 * other + 1]));
          b2 = A::add(b2, A::mul(k, I.q[3 * other + 2]));
        }
      }
    }
    const int r = I.iperm[v];
    w[3 * r] = b0;
    w[3 * r + 1] = b1;
    w[3 * r + 2] = b2;
  }
}

// Nonlinear residual of vertex v at positions X (Integrator.cpp:230-263).
template <class A>
__device__ double vertexResidual(const InstanceDev& I, const double* X, int v) {
  double f0 = 0.0, f1 = 0.0, f2 = 0.0;
  for (int k = I.rstart[v]; k < I.rstart[v + 1]; ++k) {
    const int p = I.rinc[k];
    const int e = p >> 1;
    if ((p & 1) == 0) {
      f0 = A::add(f0, I.rc[3 * e]);
      f1 = A::add(f1, I.rc[3 * e + 1]);
      f2 = A::add(f2, I.rc[3 * e + 2]);
    } else {
      f0 = A::sub(f0, I.rc[3 * e]);
      f1 = A::sub(f1, I.rc[3 * e + 1]);
      f2 = A::sub(f2, I.rc[3 * e + 2]);
    }
  }
  double g0 = 0.0, g1 = 0.0, g2 = 0.0;
  for (int k = I.bstart[v]; k < I.bstart[v + 1]; ++k) {
    const int s = I.binc[k];
    const int a = I.babc[3 * s], b = I.babc[3 * s + 1], c = I.babc[3 * s + 2];
    const double fac = I.bfac[k];
    const double s0 = A::add(A::sub(X[3 * a], A::mul(2.0, X[3 * b])), X[3 * c]);
    const double s1 = A::add(A::sub(X[3 * a + 1], A::mul(2.0, X[3 * b + 1])), X[3 * c + 1]);
    const double s2 = A::add(A::sub(X[3 * a + 2], A::mul(2.0, X[3 * b + 2])), X[3 * c + 2]);
    g0 = A::add(g0, A::mul(s0, fac));
    g1 = A::add(g1, A::mul(s1, fac));
    g2 = A::add(g2, A::mul(s2, fac));
  }
  f0 = A::add(f0, g0);
  f1 = A::add(f1, g1);
  f2 = A::add(f2, g2);
  const double mass = I.m[v];
  const double mh2 = A::mul(mass, I.invH2);
  const double t0 = A::add(A::mul(A::sub(X[3 * v], I.xhat[3 * v]), mh2), f0);
  const double t1 = A::add(A::mul(A::sub(X[3 * v + 1], I.xhat[3 * v + 1]), mh2), f1);
  const double t2 = A::add(A::mul(A::sub(X[3 * v + 2], I.xhat[3 * v + 2]), mh2), f2);
  const double len = A::sqrt(A::add(A::add(A::mul(t0, t0), A::mul(t1, t1)), A::mul(t2, t2)));
  return A::div(len, mass);
}

// Whole substeps of one instance. `w` holds the RHS / solution in elimination order; the
// solver may use `t` as a second workspace of the same size.
template <class A, class Solve, bool TIMED = false>
__device__ void runSubsteps(const InstanceDev& I, int substeps, double* w, double* t, double* red, int* flag) {
  const StageClock<TIMED> clk(I, threadIdx.x == 0);
  for (int step = 0; step < substeps; ++step) {
    // predict x̂ = x + h·v + h²·g, x_n = x, bBase = (M/h²)·x̂ (Integrator.cpp:447-472); the
    // displacement scale max|x̂ − x_n|∞ is the same in every iteration of the substep.
    double scale = 0.0;
    for (int v = threadIdx.x; v < I.n; v += blockDim.x) {
      const double mh2 = A::mul(I.m[v], I.invH2);
      double d[3];
      for (int c = 0; c < 3; ++c) {
        const double p = I.x[3 * v + c];
        const double xh = A::add(A::add(p, A::mul(I.v[3 * v + c], I.h)), I.gh2[c]);
        I.xn[3 * v + c] = p;
        I.xhat[3 * v + c] = xh;
        I.bbase[3 * v + c] = A::mul(mh2, xh);
        d[c] = A::sub(xh, p);
      }
      scale = fmax(scale, maxAbs3(d[0], d[1], d[2]));
    }
    scale = blockMax(scale, red);
    scale = (scale < I.gScaleHH) ? I.gScaleHH : scale;
    clk.lap(I, threadIdx.x == 0, kStagePredict);

    edgePass<A>(I, I.x, false);  // projection of x_n for the first scatter
    __syncthreads();
    clk.lap(I, threadIdx.x == 0, kStageLocal);
    int used = 0;
    bool conv = false;
    double lastRes = I.useResidual ? 0.0 : -1.0;
    for (int k = 0; k < I.maxIter; ++k) {
      gatherRhs<A>(I, w);
      __syncthreads();
      clk.lap(I, threadIdx.x == 0, kStageScatter);
      Solve::run(I, w, t);
      if (TIMED) __syncthreads();
      clk.lap(I, threadIdx.x == 0, kStageSolve);
      // unpack + displacement scan (Integrator.cpp:618-663); an over-relaxed iteration puts
      // x_prev + (x_solve − x_prev)·ω and keeps x_solve for the residual (:631-641)
      const bool blend = k >= I.chebFrom;
      const bool split = blend && I.useResidual;
      const double om = blend ? I.omega[k] : 1.0;
      double diff = 0.0;
      for (int v = threadIdx.x; v < I.n; v += blockDim.x) {
        const int r = I.iperm[v];
        double xs[3] = {w[3 * r], w[3 * r + 1], w[3 * r + 2]};
        if (blend) {
          double d[3];
          for (int c = 0; c < 3; ++c) {
            const double p = I.x[3 * v + c];
            const double put = A::add(p, A::mul(A::sub(xs[c], p), om));
            d[c] = A::sub(put, p);
            if (split) I.xsol[3 * v + c] = xs[c];
            I.x[3 * v + c] = put;
          }
          diff = fmax(diff, maxAbs3(d[0], d[1], d[2]));
        } else {
          diff = fmax(diff, maxAbs3(A::sub(xs[0], I.x[3 * v]), A::sub(xs[1], I.x[3 * v + 1]),
                                    A::sub(xs[2], I.x[3 * v + 2])));
          I.x[3 * v] = xs[0];
          I.x[3 * v + 1] = xs[1];
          I.x[3 * v + 2] = xs[2];
        }
      }
      __syncthreads();
      clk.lap(I, threadIdx.x == 0, kStageUnpack);
      const double* X = split ? I.xsol : I.x;
      edgePass<A>(I, X, I.useResidual != 0);
      __syncthreads();
      clk.lap(I, threadIdx.x == 0, kStageLocal);
      double res = 0.0;
      if (I.useResidual) {
        for (int v = threadIdx.x; v < I.n; v += blockDim.x) {
          if (I.pinned[v] || !(I.m[v] > 0.0)) continue;
          const double r = vertexResidual<A>(I, X, v);
          if (r > res) res = r;
        }
        res = blockMax(res, red);  // ends with a barrier: rc is no longer read below
      }
      if (split) {  // the next scatter projects the over-relaxed positions
        edgePass<A>(I, I.x, false);
        __syncthreads();
      }
      clk.lap(I, threadIdx.x == 0, kStageUnpack);  // the residual scan and the gate belong to the convergence scan
      diff = blockMax(diff, red);
      // gate (Integrator.cpp:676-747)
      if (threadIdx.x == 0) {
        const double rel = (scale > 0.0) ? A::div(diff, scale) : diff;
        const bool absHit = (I.absTol > 0.0) && (diff <= I.absTol);
        const bool relHit = (I.relTol > 0.0) && (rel <= I.relTol);
        const bool c = I.useResidual ? (res <= I.resThreshold) : (absHit || relHit);
        *flag = c ? 1 : 0;
      }
      __syncthreads();
      used = k + 1;
      lastRes = I.useResidual ? res : -1.0;
      if (I.resTrace && I.useResidual && threadIdx.x == 0) I.resTrace[(size_t)step * I.maxIter + k] = res;
      conv = *flag != 0;
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
        for (int c = 0; c < 3; ++c) I.v[3 * v + c] = A::mul(A::sub(I.x[3 * v + c], I.xn[3 * v + c]), I.dampInvH);
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
    clk.lap(I, threadIdx.x == 0, kStageVelocity);
    clk.finish(I, threadIdx.x == 0);
  }
}

}  // namespace pdg
