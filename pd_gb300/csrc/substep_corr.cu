// substep_corr.cu — MIXED substeps of cloths above the explicit-inverse limit, one CTA per cloth.
//
// Each PD iteration is taken in correction form, x^{k+1} = x^k + L⁻¹·(b(x^k) − Ã·x^k): the
// correction r = b − Ã·x comes matrix-free from one FP32 pass over each vertex's incidences
// (correction.cuh, which also yields the reference's residual of x^k for the gate), one FP32
// supernodal solve (solve32.cuh) turns it into Δ, and positions — FP32 hi/lo pairs — take Δ by an
// exact two-sum. The solve's FP32 rounding is relative to Δ, not to x, and the fixed point (r = 0)
// is the reference's; the iteration loop has no FP64 instruction (FP64 is left for the
// once-per-substep prediction and velocity update), and there is one solve per iteration.
//
// One 256-thread CTA per cloth, four CTAs per SM, so a batch of cloths fills the GPU; the host
// orders a batch's descriptors by cost so that the largest cloths start first.
// Positions and x̂ (as pairs) live in the instance's arrays (L2); the solve's two FP32 vectors
// sit in shared memory when they fit.
#include "correction.cuh"
#include "solve32.cuh"

namespace pdg {
namespace {

constexpr int kLanesPerVertex = 8;  // lanes sharing one vertex's incidences

__device__ __forceinline__ float warpMax(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Max over the CTA of non-negative values (NaN-skipping); `red` holds one slot per warp.
__device__ __forceinline__ float blockMaxF(float v, float* red) {
  v = warpMax(v);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float m = 0.f;
  for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) m = fmaxf(m, red[w]);
  return m;
}

__global__ void __launch_bounds__(kBlockThreads, 4) substepCorrKernel(const InstanceDev* __restrict__ insts,
                                                                  int substeps, int smemBytes) {
  extern __shared__ float sm[];
  __shared__ float red[32];
  const InstanceDev& I = insts[blockIdx.x];
  const int n = I.n, n3 = 3 * n;
  const bool inSmem = 24 * n <= smemBytes;  // Y, T: 3n floats each
  float* Y = inSmem ? sm : I.y32;
  float* T = inSmem ? sm + n3 : I.t32;
  float4* X = reinterpret_cast<float4*>(I.xhl);     // vertex v: hi at X[2v], lo at X[2v + 1]
  float4* Xh = reinterpret_cast<float4*>(I.xhathl);  // x̂ the same way
  float* xf = I.xhl;
  float* xhf = I.xhathl;

  for (int v = threadIdx.x; v < n; v += blockDim.x) {
    float4 h, l;
    split(I.x[3 * v], h.x, l.x);
    split(I.x[3 * v + 1], h.y, l.y);
    split(I.x[3 * v + 2], h.z, l.z);
    h.w = l.w = 0.f;
    X[2 * v] = h;
    X[2 * v + 1] = l;
  }
  __syncthreads();

  const int gl = threadIdx.x & (kLanesPerVertex - 1), group = threadIdx.x / kLanesPerVertex;
  const int ngroups = blockDim.x / kLanesPerVertex;
  for (int step = 0; step < substeps; ++step) {
    // predict (Integrator.cpp:447-472): x_n in FP64, x̂ as a pair
    float sc = 0.f;
    for (int t = threadIdx.x; t < n3; t += blockDim.x) {
      const int v = t / 3, c = t - 3 * v;
      const double p = static_cast<double>(xf[8 * v + c]) + static_cast<double>(xf[8 * v + 4 + c]);
      const double xh = (p + I.v[t] * I.h) + I.gh2[c];
      I.xn[t] = p;
      float hi, lo;
      split(xh, hi, lo);
      xhf[8 * v + c] = hi;
      xhf[8 * v + 4 + c] = lo;
      sc = fmaxf(sc, static_cast<float>(fabs(xh - p)));
    }
    const float scMax = blockMaxF(sc, red);
    const double scale = (scMax < I.gScaleHH) ? I.gScaleHH : scMax;
    int used = 0;
    bool conv = false;
    double lastRes = I.useResidual ? 0.0 : -1.0;
    for (int k = 0;; ++k) {
      // correction (elimination order, into Y) and residual of x^k
      float res = 0.f;
      for (int base = 0; base < n; base += ngroups) {
        const int v = base + group;
        const bool active = v < n;
        const float4 vc = active ? __ldg(I.tVtx + v) : make_float4(0.f, 0.f, 1.f, 0.f);
        CorrectionSums cs;
        if (vc.z == 0.f) {
          const float4 vh = X[2 * v], vl = X[2 * v + 1];
          cs.accumulate(I, I.tEdge, I.rstart[v], I.rstart[v + 1], I.tBend, I.bstart[v], I.bstart[v + 1], X, vh, vl,
                        gl, kLanesPerVertex);
          if (gl == 0) cs.addMass(vh, vl, Xh[2 * v], Xh[2 * v + 1], vc.x);
        }
        cs.reduce<kLanesPerVertex>();
        if (active && gl == 0) {
          float3 r = make_float3(0.f, 0.f, 0.f);
          if (vc.z == 0.f) {
            if (vc.y > 0.f) res = fmaxf(res, cs.residual(vc.y));
            r = cs.correction();
          }
          const int e = I.iperm[v];
          Y[3 * e] = r.x;
          Y[3 * e + 1] = r.y;
          Y[3 * e + 2] = r.z;
        }
      }
      const float resMax = blockMaxF(res, red);
      bool stop = k == I.maxIter;
      if (I.useResidual && k >= 1) {
        lastRes = resMax;
        used = k;
        conv = resMax <= I.resThreshold;
        stop = stop || conv;
      }
      if (stop) break;
      LocalSolve32::run(I, Y, T);  // Y ← Δ
      // x^{k+1} = x^k + Δ as pairs; pinned rows take q
      float dmax = 0.f;
      for (int t = threadIdx.x; t < n3; t += blockDim.x) {
        const int v = t / 3, c = t - 3 * v;
        float hi = xf[8 * v + c], lo = xf[8 * v + 4 + c];
        if (I.pinned[v]) {
          const float* qf = reinterpret_cast<const float*>(I.qhl);
          const float qh = __ldg(qf + 8 * v + c), ql = __ldg(qf + 8 * v + 4 + c);
          dmax = fmaxf(dmax, fabsf((qh - hi) + (ql - lo)));
          hi = qh;
          lo = ql;
        } else {
          const float d = Y[3 * I.iperm[v] + c];
          dmax = fmaxf(dmax, fabsf(d));
          addHL(hi, lo, d);
        }
        xf[8 * v + c] = hi;
        xf[8 * v + 4 + c] = lo;
      }
      const float diff = blockMaxF(dmax, red);
      if (!I.useResidual) {
        const double rel = (scale > 0.0) ? diff / scale : diff;
        const bool absHit = (I.absTol > 0.0) && (diff <= I.absTol);
        const bool relHit = (I.relTol > 0.0) && (rel <= I.relTol);
        used = k + 1;
        conv = absHit || relHit;
        if (conv) break;
      }
    }
    // velocity, damping, pin resnap (Integrator.cpp:774-791)
    for (int t = threadIdx.x; t < n3; t += blockDim.x) {
      const int v = t / 3, c = t - 3 * v;
      if (I.pinned[v]) {
        I.v[t] = 0.0;
        if (used == 0) {  // no update ran: the pair is resnapped here
          const float* qf = reinterpret_cast<const float*>(I.qhl);
          xf[8 * v + c] = __ldg(qf + 8 * v + c);
          xf[8 * v + 4 + c] = __ldg(qf + 8 * v + 4 + c);
        }
      } else {
        const double x = static_cast<double>(xf[8 * v + c]) + static_cast<double>(xf[8 * v + 4 + c]);
        I.v[t] = (x - I.xn[t]) * I.dampInvH;
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
  for (int t = threadIdx.x; t < n3; t += blockDim.x) {
    const int v = t / 3, c = t - 3 * v;
    I.x[t] = I.pinned[v] ? I.q[t] : static_cast<double>(xf[8 * v + c]) + static_cast<double>(xf[8 * v + 4 + c]);
  }
}

}  // namespace

int launchSubstepCorr(const InstanceDev* d, int count, int substeps, int smemBytes, void* stream) {
  if (count <= 0 || substeps <= 0) return 0;
  static bool attrSet = false;
  if (!attrSet) {
    cudaFuncSetAttribute(substepCorrKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attrSet = true;
  }
  substepCorrKernel<<<count, kBlockThreads, smemBytes, static_cast<cudaStream_t>(stream)>>>(d, substeps, smemBytes);
  return static_cast<int>(cudaGetLastError());
}

}  // namespace pdg
