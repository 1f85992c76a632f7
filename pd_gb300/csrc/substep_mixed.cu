// substep_mixed.cu — mixed-precision substep: FP32 supernodal solve + one FP64 refinement step.
//
// GB300 issues FP32 FMAs ~69× faster than FP64 ones, and the triangular solves are most of the
// FP64 work. Each PD iteration here does
//   x₀ = solve₃₂(b);  r = b − Ã·x₀ (FP64);  x = x₀ + solve₃₂(r)
// — one step of iterative refinement, which brings the FP32 solve's ~κ(L)·2⁻²⁴ relative error
// down to about its square. Everything outside the solve (projection accumulated into b, the
// residual gate, the velocity update) stays FP64; with proj32 the projection d_e itself is FP32.
//
// A cloth is run by one CTA, or by a thread-block cluster whose CTAs each solve the whole system
// redundantly in their own shared memory (so the solve needs no cluster barrier at all) while
// the FP64 work — right-hand side, refinement residual, edge pass, residual gate — is split over
// the cluster and exchanged through L2 between cluster barriers.
#include "solve32.cuh"
#include "substep_team.cuh"

namespace pdg {
namespace {

// Edge e at positions held in elimination order (X0): κ·d_e and κ·rel − κ·d_e into global memory.
__device__ __forceinline__ void edgeTermsElim(const InstanceDev& I, const double* X0, int e, bool wantRc) {
  const int a = I.iperm[I.eab[2 * e]], b = I.iperm[I.eab[2 * e + 1]];
  const double rx = X0[3 * a] - X0[3 * b];
  const double ry = X0[3 * a + 1] - X0[3 * b + 1];
  const double rz = X0[3 * a + 2] - X0[3 * b + 2];
  double dx = 0.0, dy = 0.0, dz = 0.0;
  projectEdge(I, e, rx, ry, rz, dx, dy, dz);
  const double k = I.ek[e];
  const double cx = dx * k, cy = dy * k, cz = dz * k;
  __stcg(I.kd + 3 * e, cx);
  __stcg(I.kd + 3 * e + 1, cy);
  __stcg(I.kd + 3 * e + 2, cz);
  if (wantRc) {
    __stcg(I.rc + 3 * e, fma(rx, k, -cx));
    __stcg(I.rc + 3 * e + 1, fma(ry, k, -cy));
    __stcg(I.rc + 3 * e + 2, fma(rz, k, -cz));
  }
}

// Whole mixed-precision substeps of one instance. B, X0 (doubles) and Y, T (floats) are this
// CTA's private 3n workspaces; with a cluster they are in shared memory and I.w / I.tbuf carry
// the right-hand side and the refinement residual between the CTAs.
template <bool CLUSTER>
__device__ void runSubstepsMixed(const InstanceDev& I, const Team<CLUSTER>& tm, int substeps, double* B, double* X0,
                                 float* Y, float* Tt, double* red, double* slots) {
  int parity = 0;
  const int T = tm.tid(), NT = tm.count();
  const int n3 = 3 * I.n;
  for (int step = 0; step < substeps; ++step) {
    double scale = 0.0;
    for (int v = T; v < I.n; v += NT) {  // predict (Integrator.cpp:447-472)
      const double mh2 = I.m[v] * I.invH2;
      double d[3];
      for (int c = 0; c < 3; ++c) {
        const double p = tm.ld(I.x + 3 * v + c);
        const double xh = (p + tm.ld(I.v + 3 * v + c) * I.h) + I.gh2[c];
        I.xn[3 * v + c] = p;
        I.xhat[3 * v + c] = xh;
        I.bbase[3 * v + c] = mh2 * xh;
        d[c] = xh - p;
      }
      scale = fmax(scale, maxAbs3(d[0], d[1], d[2]));
    }
    scale = teamMax(tm, scale, red, slots, parity);
    scale = (scale < I.gScaleHH) ? I.gScaleHH : scale;
    for (int e = T; e < I.ne; e += NT) edgeTerms(I, tm, I.x, e, false);  // projection of x_n
    tm.sync();
    int used = 0;
    bool conv = false;
    double lastRes = I.useResidual ? 0.0 : -1.0;
    for (int k = 0; k < I.maxIter; ++k) {
      // right-hand side (FP64) of this CTA's vertices
      for (int v = T; v < I.n; v += NT) {
        double b[3];
        if (I.pinned[v]) {
          for (int c = 0; c < 3; ++c) b[c] = I.q[3 * v + c];
        } else {
          for (int c = 0; c < 3; ++c) b[c] = tm.ld(I.bbase + 3 * v + c) + (I.hasBendRhs ? I.bendRhs[3 * v + c] : 0.0);
          for (int q = I.sstart[v]; q < I.sstart[v + 1]; ++q) {
            const int p = I.sinc[q];
            const int e = p >> 1;
            const double sgn = (p & 1) ? -1.0 : 1.0;
            for (int c = 0; c < 3; ++c) b[c] = fma(sgn, tm.ld(I.kd + 3 * e + c), b[c]);
            const int other = I.eab[2 * e + ((p & 1) ^ 1)];
            if (I.pinned[other])
              for (int c = 0; c < 3; ++c) b[c] = fma(I.ek[e], I.q[3 * other + c], b[c]);
          }
        }
        const int r = I.iperm[v];
        for (int c = 0; c < 3; ++c) {
          if (CLUSTER) {
            __stcg(I.w + 3 * r + c, b[c]);
          } else {
            B[3 * r + c] = b[c];
            Y[3 * r + c] = static_cast<float>(b[c]);
          }
        }
      }
      if (CLUSTER) {
        tm.sync();
        for (int i = threadIdx.x; i < n3; i += blockDim.x) {
          const double b = __ldcg(I.w + i);
          B[i] = b;
          Y[i] = static_cast<float>(b);
        }
      }
      __syncthreads();
      LocalSolve32::run(I, Y, Tt);
      for (int i = threadIdx.x; i < n3; i += blockDim.x) X0[i] = static_cast<double>(Y[i]);
      __syncthreads();
      // refinement residual r = b − Ã·x₀ (FP64) of this CTA's rows
      for (int i = T; i < I.n; i += NT) {
        double r0 = B[3 * i], r1 = B[3 * i + 1], r2 = B[3 * i + 2];
#pragma unroll 4
        for (int p = I.Aptr[i]; p < I.Aptr[i + 1]; ++p) {
          const int j = I.Acol[p];
          const double a = -I.Aval[p];
          r0 = fma(a, X0[3 * j], r0);
          r1 = fma(a, X0[3 * j + 1], r1);
          r2 = fma(a, X0[3 * j + 2], r2);
        }
        if (CLUSTER) {
          __stcg(I.tbuf + 3 * i, r0);
          __stcg(I.tbuf + 3 * i + 1, r1);
          __stcg(I.tbuf + 3 * i + 2, r2);
        } else {
          Y[3 * i] = static_cast<float>(r0);
          Y[3 * i + 1] = static_cast<float>(r1);
          Y[3 * i + 2] = static_cast<float>(r2);
        }
      }
      if (CLUSTER) {
        tm.sync();
        for (int i = threadIdx.x; i < n3; i += blockDim.x) Y[i] = static_cast<float>(__ldcg(I.tbuf + i));
      }
      __syncthreads();
      LocalSolve32::run(I, Y, Tt);
      for (int i = threadIdx.x; i < n3; i += blockDim.x) X0[i] += static_cast<double>(Y[i]);
      __syncthreads();
      // unpack this CTA's vertices + displacement scan (Integrator.cpp:618-663); an over-relaxed
      // iteration puts x_prev + (x_solve − x_prev)·ω, the residual below stays that of x_solve (X0)
      const bool blend = k >= I.chebFrom;
      const double om = blend ? I.omega[k] : 1.0;
      double diff = 0.0;
      for (int v = T; v < I.n; v += NT) {
        const int r = I.iperm[v];
        double dm = 0.0;
        for (int c = 0; c < 3; ++c) {
          const double xs = X0[3 * r + c], p = tm.ld(I.x + 3 * v + c);
          const double put = blend ? p + (xs - p) * om : xs;
          dm = fmax(dm, fabs(put - p));
          I.x[3 * v + c] = put;
        }
        diff = fmax(diff, dm);
      }
      for (int e = T; e < I.ne; e += NT) edgeTermsElim(I, X0, e, I.useResidual != 0);
      tm.sync();
      if (blend) {  // the next right-hand side projects the over-relaxed positions (rc is kept)
        for (int e = T; e < I.ne; e += NT) edgeTerms(I, tm, I.x, e, false);
        tm.sync();
      }
      double res = 0.0;
      if (I.useResidual) {
        for (int v = T; v < I.n; v += NT) {
          if (I.pinned[v] || !(I.m[v] > 0.0)) continue;
          double f[3] = {0.0, 0.0, 0.0};
          for (int q = I.rstart[v]; q < I.rstart[v + 1]; ++q) {
            const int p = I.rinc[q];
            const int e = p >> 1;
            const double sgn = (p & 1) ? -1.0 : 1.0;
            for (int c = 0; c < 3; ++c) f[c] = fma(sgn, tm.ld(I.rc + 3 * e + c), f[c]);
          }
          for (int q = I.bstart[v]; q < I.bstart[v + 1]; ++q) {
            const int s = I.binc[q];
            const int a = I.iperm[I.babc[3 * s]], b = I.iperm[I.babc[3 * s + 1]], cc = I.iperm[I.babc[3 * s + 2]];
            for (int c = 0; c < 3; ++c)
              f[c] = fma(X0[3 * a + c] - 2.0 * X0[3 * b + c] + X0[3 * cc + c], I.bfac[q], f[c]);
          }
          const double mass = I.m[v];
          const double mh2 = mass * I.invH2;
          const int r = I.iperm[v];
          double s2 = 0.0;
          for (int c = 0; c < 3; ++c) {
            const double t = fma(X0[3 * r + c] - I.xhat[3 * v + c], mh2, f[c]);
            s2 = fma(t, t, s2);
          }
          const double rv = sqrt(s2) / mass;
          if (rv > res) res = rv;
        }
        res = teamMax(tm, res, red, slots, parity);
      }
      diff = teamMax(tm, diff, red, slots, parity);
      const double rel = (scale > 0.0) ? diff / scale : diff;
      const bool absHit = (I.absTol > 0.0) && (diff <= I.absTol);
      const bool relHit = (I.relTol > 0.0) && (rel <= I.relTol);
      conv = I.useResidual ? (res <= I.resThreshold) : (absHit || relHit);
      used = k + 1;
      lastRes = I.useResidual ? res : -1.0;
      if (I.resTrace && I.useResidual && T == 0) I.resTrace[(size_t)step * I.maxIter + k] = res;
      if (conv) break;
    }
    for (int v = T; v < I.n; v += NT) {  // velocity, damping, pin resnap (Integrator.cpp:774-791)
      if (I.pinned[v]) {
        for (int c = 0; c < 3; ++c) {
          I.v[3 * v + c] = 0.0;
          I.x[3 * v + c] = I.q[3 * v + c];
        }
      } else {
        for (int c = 0; c < 3; ++c) I.v[3 * v + c] = (tm.ld(I.x + 3 * v + c) - tm.ld(I.xn + 3 * v + c)) * I.dampInvH;
      }
    }
    if (T == 0) {
      if (I.iterLog) I.iterLog[step] = used;
      if (I.convLog) I.convLog[step] = conv ? 1 : 0;
      *I.lastResidual = lastRes;
      *I.iterationsUsed = used;
      *I.converged = conv ? 1 : 0;
      if (conv) *I.earlyExits += 1;
    }
    tm.sync();
  }
}

// Rows [rb, re) of Ã⁻¹·s for the three components, one warp per row: float4 loads of the row
// (L2-resident), s in shared memory as three padded FP32 arrays. Calls emit(i, a0, a1, a2).
template <class Emit>
__device__ __forceinline__ void denseRows(const InstanceDev& I, int rb, int re, const float* Sx, const float* Sy,
                                          const float* Sz, Emit&& emit) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int ld4 = I.denseLd / 4;
  const float4* sx = reinterpret_cast<const float4*>(Sx);
  const float4* sy = reinterpret_cast<const float4*>(Sy);
  const float4* sz = reinterpret_cast<const float4*>(Sz);
  for (int i = rb + warp; i < re; i += nw) {
    const float4* row = reinterpret_cast<const float4*>(I.Ainv + static_cast<size_t>(i) * I.denseLd);
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
#pragma unroll 4
    for (int j = lane; j < ld4; j += 32) {
      const float4 m = __ldg(row + j);
      const float4 x = sx[j], y = sy[j], z = sz[j];
      a0 = fmaf(m.x, x.x, fmaf(m.y, x.y, fmaf(m.z, x.z, fmaf(m.w, x.w, a0))));
      a1 = fmaf(m.x, y.x, fmaf(m.y, y.y, fmaf(m.z, y.z, fmaf(m.w, y.w, a1))));
      a2 = fmaf(m.x, z.x, fmaf(m.y, z.y, fmaf(m.z, z.z, fmaf(m.w, z.w, a2))));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (lane == 0) emit(i, a0, a1, a2);
  }
}

// Mixed-precision substeps of a small cloth by a cluster, with the solve as two FP32 products
// with the explicit inverse around one FP64 refinement: x₀ = Ã⁻¹b, r = b − Ã·x₀, x = x₀ + Ã⁻¹r.
// Vectors are in vertex order. Each CTA owns a block of rows of every product; b, x₀, r and x
// pass between the CTAs through L2 (I.w, I.tbuf, I.x0, I.x) between cluster barriers.
__device__ void runSubstepsDense(const InstanceDev& I, const Team<true>& tm, int substeps, double* Bd, double* X0,
                                 float* Sx, float* Sy, float* Sz, double* red, double* slots) {
  int parity = 0;
  const int T = tm.tid(), NT = tm.count();
  const int n = I.n;
  const int chunk = (n + tm.size - 1) / tm.size;
  const int rb = min(n, tm.rank * chunk), re = min(n, rb + chunk);
  for (int j = n + threadIdx.x; j < I.denseLd; j += blockDim.x) Sx[j] = Sy[j] = Sz[j] = 0.f;  // padding
  for (int step = 0; step < substeps; ++step) {
    double scale = 0.0;
    for (int v = T; v < n; v += NT) {  // predict (Integrator.cpp:447-472)
      const double mh2 = I.m[v] * I.invH2;
      double d[3];
      for (int c = 0; c < 3; ++c) {
        const double p = tm.ld(I.x + 3 * v + c);
        const double xh = (p + tm.ld(I.v + 3 * v + c) * I.h) + I.gh2[c];
        I.xn[3 * v + c] = p;
        I.xhat[3 * v + c] = xh;
        I.bbase[3 * v + c] = mh2 * xh;
        d[c] = xh - p;
      }
      scale = fmax(scale, maxAbs3(d[0], d[1], d[2]));
    }
    scale = teamMax(tm, scale, red, slots, parity);
    scale = (scale < I.gScaleHH) ? I.gScaleHH : scale;
    for (int e = T; e < I.ne; e += NT) edgeTerms(I, tm, I.x, e, false);  // projection of x_n
    tm.sync();
    int used = 0;
    bool conv = false;
    double lastRes = I.useResidual ? 0.0 : -1.0;
    for (int k = 0; k < I.maxIter; ++k) {
      for (int v = T; v < n; v += NT) {  // right-hand side (FP64), published in I.w
        double b[3];
        if (I.pinned[v]) {
          for (int c = 0; c < 3; ++c) b[c] = I.q[3 * v + c];
        } else {
          for (int c = 0; c < 3; ++c) b[c] = tm.ld(I.bbase + 3 * v + c) + (I.hasBendRhs ? I.bendRhs[3 * v + c] : 0.0);
          for (int q = I.sstart[v]; q < I.sstart[v + 1]; ++q) {
            const int p = I.sinc[q];
            const int e = p >> 1;
            const double sgn = (p & 1) ? -1.0 : 1.0;
            for (int c = 0; c < 3; ++c) b[c] = fma(sgn, tm.ld(I.kd + 3 * e + c), b[c]);
            const int other = I.eab[2 * e + ((p & 1) ^ 1)];
            if (I.pinned[other])
              for (int c = 0; c < 3; ++c) b[c] = fma(I.ek[e], I.q[3 * other + c], b[c]);
          }
        }
        for (int c = 0; c < 3; ++c) __stcg(I.w + 3 * v + c, b[c]);
      }
      tm.sync();
      for (int v = threadIdx.x; v < n; v += blockDim.x) {
        const double b0 = __ldcg(I.w + 3 * v), b1 = __ldcg(I.w + 3 * v + 1), b2 = __ldcg(I.w + 3 * v + 2);
        Bd[3 * v] = b0;
        Bd[3 * v + 1] = b1;
        Bd[3 * v + 2] = b2;
        Sx[v] = static_cast<float>(b0);
        Sy[v] = static_cast<float>(b1);
        Sz[v] = static_cast<float>(b2);
      }
      __syncthreads();
      denseRows(I, rb, re, Sx, Sy, Sz, [&](int i, float a0, float a1, float a2) {  // x₀ = Ã⁻¹·b
        __stcg(I.tbuf + 3 * i, static_cast<double>(a0));
        __stcg(I.tbuf + 3 * i + 1, static_cast<double>(a1));
        __stcg(I.tbuf + 3 * i + 2, static_cast<double>(a2));
      });
      tm.sync();
      for (int i = threadIdx.x; i < 3 * n; i += blockDim.x) X0[i] = __ldcg(I.tbuf + i);
      __syncthreads();
      for (int i = rb + (int)threadIdx.x; i < re; i += blockDim.x) {  // r = b − Ã·x₀ (FP64)
        double r0 = Bd[3 * i], r1 = Bd[3 * i + 1], r2 = Bd[3 * i + 2];
        for (int p = I.Vptr[i]; p < I.Vptr[i + 1]; ++p) {
          const int j = I.Vcol[p];
          const double a = -I.Vval[p];
          r0 = fma(a, X0[3 * j], r0);
          r1 = fma(a, X0[3 * j + 1], r1);
          r2 = fma(a, X0[3 * j + 2], r2);
        }
        __stcg(I.x0 + 3 * i, r0);
        __stcg(I.x0 + 3 * i + 1, r1);
        __stcg(I.x0 + 3 * i + 2, r2);
      }
      tm.sync();
      for (int v = threadIdx.x; v < n; v += blockDim.x) {
        Sx[v] = static_cast<float>(__ldcg(I.x0 + 3 * v));
        Sy[v] = static_cast<float>(__ldcg(I.x0 + 3 * v + 1));
        Sz[v] = static_cast<float>(__ldcg(I.x0 + 3 * v + 2));
      }
      __syncthreads();
      // x_solve = x₀ + Ã⁻¹·r; an over-relaxed iteration puts x_prev + (x_solve − x_prev)·ω and
      // keeps x_solve for the residual (Integrator.cpp:631-641)
      const bool blend = k >= I.chebFrom;
      const bool split = blend && I.useResidual;
      const double om = blend ? I.omega[k] : 1.0;
      double diff = 0.0;
      denseRows(I, rb, re, Sx, Sy, Sz, [&](int i, float a0, float a1, float a2) {
        const float a[3] = {a0, a1, a2};
        for (int c = 0; c < 3; ++c) {
          const double xs = X0[3 * i + c] + a[c], p = __ldcg(I.x + 3 * i + c);
          double put = xs;
          if (blend) {
            put = p + (xs - p) * om;
            if (split) __stcg(I.xsol + 3 * i + c, xs);
          }
          diff = fmax(diff, fabs(put - p));
          __stcg(I.x + 3 * i + c, put);
        }
      });
      tm.sync();
      const double* X = split ? I.xsol : I.x;
      for (int e = T; e < I.ne; e += NT) edgeTerms(I, tm, X, e, I.useResidual != 0);
      tm.sync();
      double res = 0.0;
      if (I.useResidual) {
        for (int v = T; v < n; v += NT) {
          if (I.pinned[v] || !(I.m[v] > 0.0)) continue;
          const double r = residualAt(I, tm, X, v);
          if (r > res) res = r;
        }
        res = teamMax(tm, res, red, slots, parity);
      }
      if (split) {  // the next right-hand side projects the over-relaxed positions
        for (int e = T; e < I.ne; e += NT) edgeTerms(I, tm, I.x, e, false);
        tm.sync();
      }
      diff = teamMax(tm, diff, red, slots, parity);
      const double rel = (scale > 0.0) ? diff / scale : diff;
      const bool absHit = (I.absTol > 0.0) && (diff <= I.absTol);
      const bool relHit = (I.relTol > 0.0) && (rel <= I.relTol);
      conv = I.useResidual ? (res <= I.resThreshold) : (absHit || relHit);
      used = k + 1;
      lastRes = I.useResidual ? res : -1.0;
      if (I.resTrace && I.useResidual && T == 0) I.resTrace[(size_t)step * I.maxIter + k] = res;
      if (conv) break;
    }
    for (int v = T; v < n; v += NT) {  // velocity, damping, pin resnap (Integrator.cpp:774-791)
      if (I.pinned[v]) {
        for (int c = 0; c < 3; ++c) {
          I.v[3 * v + c] = 0.0;
          __stcg(I.x + 3 * v + c, I.q[3 * v + c]);
        }
      } else {
        for (int c = 0; c < 3; ++c) I.v[3 * v + c] = (tm.ld(I.x + 3 * v + c) - tm.ld(I.xn + 3 * v + c)) * I.dampInvH;
      }
    }
    if (T == 0) {
      if (I.iterLog) I.iterLog[step] = used;
      if (I.convLog) I.convLog[step] = conv ? 1 : 0;
      *I.lastResidual = lastRes;
      *I.iterationsUsed = used;
      *I.converged = conv ? 1 : 0;
      if (conv) *I.earlyExits += 1;
    }
    tm.sync();
  }
}

__global__ void __launch_bounds__(kClusterThreads) substepDenseClusterKernel(const InstanceDev* __restrict__ insts,
                                                                           int substeps) {
  extern __shared__ double smem[];
  __shared__ double red[32];
  __shared__ double slots[2];
  cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
  const int cs = static_cast<int>(cl.num_blocks());
  const InstanceDev& I = insts[blockIdx.x / cs];
  double* Bd = smem;
  double* X0 = smem + 3 * I.n;
  float* Sx = reinterpret_cast<float*>(smem + 6 * I.n);
  float* Sy = Sx + I.denseLd;
  float* Sz = Sy + I.denseLd;
  const Team<true> tm{static_cast<int>(cl.block_rank()), cs};
  runSubstepsDense(I, tm, substeps, Bd, X0, Sx, Sy, Sz, red, slots);
}

__global__ void __launch_bounds__(kBlockThreads) substepMixedKernel(const InstanceDev* __restrict__ insts,
                                                                    int substeps, int smemBytes) {
  extern __shared__ double smem[];
  __shared__ double red[32];
  __shared__ double slots[2];
  const InstanceDev& I = insts[blockIdx.x];
  const int n3 = 3 * I.n;
  const bool inSmem = 72 * I.n <= smemBytes;  // B, X0 (doubles) + Y, T (floats): 72·n bytes
  double* B = inSmem ? smem : I.w;
  double* X0 = inSmem ? smem + n3 : I.x0;
  float* Y = inSmem ? reinterpret_cast<float*>(smem + 2 * n3) : I.y32;
  float* Tt = inSmem ? Y + n3 : I.t32;
  const Team<false> tm{0, 1};
  runSubstepsMixed<false>(I, tm, substeps, B, X0, Y, Tt, red, slots);
}

__global__ void __launch_bounds__(kClusterThreads) substepMixedClusterKernel(const InstanceDev* __restrict__ insts,
                                                                           int substeps) {
  extern __shared__ double smem[];
  __shared__ double red[32];
  __shared__ double slots[2];
  cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
  const int cs = static_cast<int>(cl.num_blocks());
  const InstanceDev& I = insts[blockIdx.x / cs];
  const int n3 = 3 * I.n;
  double* B = smem;
  double* X0 = smem + n3;
  float* Y = reinterpret_cast<float*>(smem + 2 * n3);
  float* Tt = Y + n3;
  const Team<true> tm{static_cast<int>(cl.block_rank()), cs};
  runSubstepsMixed<true>(I, tm, substeps, B, X0, Y, Tt, red, slots);
}

cudaLaunchConfig_t clusterLaunch(int blocks, int clusterSize, int smemBytes, void* stream, cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(kClusterThreads);
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

int launchSubstepMixed(const InstanceDev* d, int count, int substeps, int smemBytes, void* stream) {
  if (count <= 0 || substeps <= 0) return 0;
  static bool attrSet = false;
  if (!attrSet) {
    cudaFuncSetAttribute(substepMixedKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attrSet = true;
  }
  substepMixedKernel<<<count, kBlockThreads, smemBytes, static_cast<cudaStream_t>(stream)>>>(d, substeps, smemBytes);
  return static_cast<int>(cudaGetLastError());
}

int mixedClusterSupported(int clusterSize, int smemBytes) {
  if (clusterSize < 2 || clusterSize > 16 || smemBytes > 200 * 1024) return 0;
  cudaFuncSetAttribute(substepMixedClusterKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (clusterSize > 8) cudaFuncSetAttribute(substepMixedClusterKernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = clusterLaunch(clusterSize, clusterSize, smemBytes, nullptr, attr);
  int clusters = 0;
  const cudaError_t e = cudaOccupancyMaxActiveClusters(&clusters, substepMixedClusterKernel, &cfg);
  if (e != cudaSuccess) cudaGetLastError();
  return (e == cudaSuccess && clusters > 0) ? clusterSize : 0;
}

int denseClusterSupported(int clusterSize, int smemBytes) {
  if (clusterSize < 2 || clusterSize > 16 || smemBytes > 200 * 1024) return 0;
  cudaFuncSetAttribute(substepDenseClusterKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (clusterSize > 8) cudaFuncSetAttribute(substepDenseClusterKernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = clusterLaunch(clusterSize, clusterSize, smemBytes, nullptr, attr);
  int clusters = 0;
  const cudaError_t e = cudaOccupancyMaxActiveClusters(&clusters, substepDenseClusterKernel, &cfg);
  if (e != cudaSuccess) cudaGetLastError();
  return (e == cudaSuccess && clusters > 0) ? clusterSize : 0;
}

int launchSubstepDenseCluster(const InstanceDev* d, int count, int clusterSize, int smemBytes, int substeps,
                              void* stream) {
  if (count <= 0 || substeps <= 0) return 0;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = clusterLaunch(count * clusterSize, clusterSize, smemBytes, stream, attr);
  const cudaError_t e = cudaLaunchKernelEx(&cfg, substepDenseClusterKernel, d, substeps);
  return static_cast<int>(e != cudaSuccess ? e : cudaGetLastError());
}

int launchSubstepMixedCluster(const InstanceDev* d, int count, int clusterSize, int smemBytes, int substeps,
                              void* stream) {
  if (count <= 0 || substeps <= 0) return 0;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = clusterLaunch(count * clusterSize, clusterSize, smemBytes, stream, attr);
  const cudaError_t e = cudaLaunchKernelEx(&cfg, substepMixedClusterKernel, d, substeps);
  return static_cast<int>(e != cudaSuccess ? e : cudaGetLastError());
}

}  // namespace pdg
