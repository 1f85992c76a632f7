// substep_corr.cu — MIXED substeps of cloths above the explicit-inverse limit: the correction form
// with the FP32 supernodal solve, by one CTA per cloth or by a thread-block cluster per cloth.
//
// Each PD iteration is taken in correction form, x^{k+1} = x^k + L⁻¹·(b(x^k) − Ã·x^k): the
// correction r = b − Ã·x comes matrix-free from one FP32 pass over each vertex's incidences
// (correction.cuh, which also yields the reference's residual of x^k for the gate), one FP32
// supernodal solve turns it into Δ, and positions — FP32 hi/lo pairs — take Δ by an exact
// two-sum. The solve's FP32 rounding is relative to Δ, not to x, and the fixed point (r = 0) is the
// reference's; the iteration loop has no FP64 instruction (FP64 is left for the once-per-substep
// prediction and velocity update), and there is one solve per iteration.
//
// One 256-thread CTA per cloth (four per SM, so a batch fills the GPU; the host orders a batch's
// descriptors by cost so that the largest cloths start first), or a cluster of up to 16 CTAs per
// cloth for large single cloths: vertex, edge and row loops are strided over the cluster, phases
// are separated by cluster barriers, data other CTAs write are read through L2, and reductions go
// through distributed shared memory. Positions and x̂ (as pairs) and the solve's two vectors live
// in the instance's arrays; a one-CTA cloth keeps the solve vectors in shared memory when they fit.
#include <algorithm>

#include "correction.cuh"
#include "team_solve32.cuh"

namespace pdg {
namespace {

// Lanes sharing one vertex's incidences in the correction pass. The pass is bound by the latency of
// its dependent loads (incidence records, then the neighbours' positions) once per round of vertices,
// so fewer lanes a vertex — more vertices a round, fewer rounds — is faster where the team is small:
// measured on the 512-cloth batch (one CTA or a 4-CTA cluster per cloth) 28.8 / 26.8 / 26.4 / 25.6 ms a
// substep with 8 / 4 / 2 / 1 lanes, and on one 256×256 cloth over a 456-CTA grid 10.33 / 10.23 / 10.09 ms
// with 8 / 4 / 2 (one lane costs the grid kernel registers and with them a third of its CTAs). The
// cluster kernel takes two: with one it needs 128 registers a thread and fits two CTAs an SM; the
// autotuned batch (8-CTA clusters for the large cloths) 23.4 ms a substep with one lane, 20.8 with two.
constexpr int kLanesOneCta = 1;
constexpr int kLanesCluster = 2;
constexpr int kLanesGrid = 2;

template <int LANES, bool CLUSTER, bool TIMED = false>
__device__ void runSubstepsCorr(const InstanceDev& I, const Team<CLUSTER>& tm, int substeps, float* Y, float* T,
                                double* red, double* slots) {
  int parity = 0;
  const int n = I.n, n3 = 3 * n;
  const int TID = tm.tid(), NT = tm.count();
  float4* X = reinterpret_cast<float4*>(I.xhl);     // vertex v: hi at X[2v], lo at X[2v + 1]
  float4* Xh = reinterpret_cast<float4*>(I.xhathl);  // x̂ the same way
  float* xf = I.xhl;
  float* xhf = I.xhathl;

  for (int v = TID; v < n; v += NT) {
    float4 h, l;
    split(I.x[3 * v], h.x, l.x);
    split(I.x[3 * v + 1], h.y, l.y);
    split(I.x[3 * v + 2], h.z, l.z);
    h.w = l.w = 0.f;
    X[2 * v] = h;
    X[2 * v + 1] = l;
  }
  tm.sync();

  const int gl = TID & (LANES - 1), group = TID / LANES, ngroups = NT / LANES;
  const StageClock<TIMED> clk(I, TID == 0);
  for (int step = 0; step < substeps; ++step) {
    // predict (Integrator.cpp:447-472): x_n in FP64, x̂ as a pair
    double sc = 0.0;
    for (int t = TID; t < n3; t += NT) {
      const int v = t / 3, c = t - 3 * v;
      const double p = static_cast<double>(tm.ld(xf + 8 * v + c)) + static_cast<double>(tm.ld(xf + 8 * v + 4 + c));
      const double xh = (p + I.v[t] * I.h) + I.gh2[c];
      I.xn[t] = p;
      float hi, lo;
      split(xh, hi, lo);
      xhf[8 * v + c] = hi;
      xhf[8 * v + 4 + c] = lo;
      sc = fmax(sc, fabs(xh - p));
    }
    const double scMax = teamMax(tm, sc, red, slots, parity);
    clk.lap(I, TID == 0, kStagePredict);
    const double scale = (scMax < I.gScaleHH) ? I.gScaleHH : scMax;
    int used = 0;
    bool conv = false;
    double lastRes = I.useResidual ? 0.0 : -1.0;
    // correction b − Ã·x (elimination order, into Y when wanted) and the largest residual of the
    // current positions, LANES lanes per vertex
    auto correctionPass = [&](bool wantY) {
      float res = 0.f;
      for (int base = 0; base < n; base += ngroups) {
        const int v = base + group;
        const bool active = v < n;
        const float4 vc = active ? __ldg(I.tVtx + v) : make_float4(0.f, 0.f, 1.f, 0.f);
        CorrectionSums cs;
        if (vc.z == 0.f) {
          const float4 vh = tm.ld(X + 2 * v), vl = tm.ld(X + 2 * v + 1);
          cs.accumulate<CLUSTER>(I, I.tEdge, I.rstart[v], I.rstart[v + 1], I.tBend, I.bstart[v], I.bstart[v + 1], X,
                                 vh, vl, gl, LANES);
          if (gl == 0) cs.addMass(vh, vl, tm.ld(Xh + 2 * v), tm.ld(Xh + 2 * v + 1), vc.x);
        }
        cs.reduce<LANES>();
        if (active && gl == 0) {
          float3 r = make_float3(0.f, 0.f, 0.f);
          if (vc.z == 0.f) {
            if (vc.y > 0.f) res = fmaxf(res, cs.residual(vc.y));
            r = cs.correction();
          }
          if (wantY) {
            const int e = I.iperm[v];
            Y[3 * e] = r.x;
            Y[3 * e + 1] = r.y;
            Y[3 * e + 2] = r.z;
          }
        }
      }
      return teamMax(tm, static_cast<double>(res), red, slots, parity);
    };
    for (int k = 0;; ++k) {
      // correction and residual of x^k; the residual gates iteration k − 1 unless that iteration
      // was over-relaxed and gated on its own solve's residual below
      const double resMax = correctionPass(true);
      clk.lap(I, TID == 0, kStageLocal);
      bool stop = k == I.maxIter;
      if (I.useResidual && k >= 1 && k - 1 < I.chebFrom) {
        lastRes = resMax;
        used = k;
        if (I.resTrace && TID == 0) I.resTrace[(size_t)step * I.maxIter + k - 1] = resMax;
        conv = resMax <= I.resThreshold;
        stop = stop || conv;
      }
      if (stop) break;
      TeamSolve32<CLUSTER>::run(I, tm, Y, T);  // Y ← Δ
      clk.lap(I, TID == 0, kStageSolve);
      // x^{k+1} = x^k + Δ as pairs; pinned rows take q. An over-relaxed iteration
      // (Integrator.cpp:631-641) puts x^k + ω·Δ; with the residual gate it first puts x^k + Δ,
      // takes that point's residual, then adds (ω − 1)·Δ.
      const bool blend = k >= I.chebFrom;
      const bool split = blend && I.useResidual;
      const float om = blend ? static_cast<float>(I.omega[k]) : 1.f;
      double dmax = 0.0;
      for (int t = TID; t < n3; t += NT) {
        const int v = t / 3, c = t - 3 * v;
        float hi = tm.ld(xf + 8 * v + c), lo = tm.ld(xf + 8 * v + 4 + c);
        float* y = Y + 3 * I.iperm[v] + c;
        float d;
        if (I.pinned[v]) {
          const float* qf = reinterpret_cast<const float*>(I.qhl);
          const float qh = __ldg(qf + 8 * v + c), ql = __ldg(qf + 8 * v + 4 + c);
          d = (qh - hi) + (ql - lo);
          hi = qh;
          lo = ql;
          if (blend && !split) addHL(hi, lo, (om - 1.f) * d);
          if (split) *y = d;
        } else {
          d = tm.ld(y);
          addHL(hi, lo, split ? d : om * d);
        }
        dmax = fmax(dmax, static_cast<double>(fabsf(blend ? om * d : d)));
        xf[8 * v + c] = hi;
        xf[8 * v + 4 + c] = lo;
      }
      if (split) {
        tm.sync();
        const double resSolve = correctionPass(false);  // residual of x^k + Δ; ends with a team barrier
        for (int t = TID; t < n3; t += NT) {
          const int v = t / 3, c = t - 3 * v;
          float hi = tm.ld(xf + 8 * v + c), lo = tm.ld(xf + 8 * v + 4 + c);
          addHL(hi, lo, (om - 1.f) * tm.ld(Y + 3 * I.iperm[v] + c));
          xf[8 * v + c] = hi;
          xf[8 * v + 4 + c] = lo;
        }
        tm.sync();
        clk.lap(I, TID == 0, kStageUnpack);
        lastRes = resSolve;
        used = k + 1;
        if (I.resTrace && TID == 0) I.resTrace[(size_t)step * I.maxIter + k] = resSolve;
        conv = resSolve <= I.resThreshold;
        if (conv || k + 1 == I.maxIter) break;
        continue;
      }
      const double diff = teamMax(tm, dmax, red, slots, parity);
      clk.lap(I, TID == 0, kStageUnpack);
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
    for (int t = TID; t < n3; t += NT) {
      const int v = t / 3, c = t - 3 * v;
      if (I.pinned[v]) {
        I.v[t] = 0.0;
        if (used == 0) {  // no update ran: the pair is resnapped here
          const float* qf = reinterpret_cast<const float*>(I.qhl);
          xf[8 * v + c] = __ldg(qf + 8 * v + c);
          xf[8 * v + 4 + c] = __ldg(qf + 8 * v + 4 + c);
        }
      } else {
        const double x = static_cast<double>(tm.ld(xf + 8 * v + c)) + static_cast<double>(tm.ld(xf + 8 * v + 4 + c));
        I.v[t] = (x - I.xn[t]) * I.dampInvH;
      }
    }
    if (TID == 0) {
      if (I.iterLog) I.iterLog[step] = used;
      if (I.convLog) I.convLog[step] = conv ? 1 : 0;
      *I.lastResidual = lastRes;
      *I.iterationsUsed = used;
      *I.converged = conv ? 1 : 0;
      if (conv) *I.earlyExits += 1;
    }
    tm.sync();
    clk.lap(I, TID == 0, kStageVelocity);
    clk.finish(I, TID == 0);
  }
  for (int t = TID; t < n3; t += NT) {
    const int v = t / 3, c = t - 3 * v;
    I.x[t] = I.pinned[v] ? I.q[t]
                         : static_cast<double>(tm.ld(xf + 8 * v + c)) + static_cast<double>(tm.ld(xf + 8 * v + 4 + c));
  }
}

template <bool TIMED>
__global__ void __launch_bounds__(kBlockThreads, 4) substepCorrKernel(const InstanceDev* __restrict__ insts,
                                                                     int substeps, int smemBytes) {
  extern __shared__ float sm[];
  __shared__ double red[32];
  __shared__ double slots[2];
  const InstanceDev& I = insts[blockIdx.x];
  const bool inSmem = 24 * I.n <= smemBytes;  // Y, T: 3n floats each
  float* Y = inSmem ? sm : I.y32;
  float* T = inSmem ? sm + 3 * I.n : I.t32;
  const Team<false> tm{0, 1};
  runSubstepsCorr<kLanesOneCta, false, TIMED>(I, tm, substeps, Y, T, red, slots);
}

template <bool TIMED>
__global__ void __launch_bounds__(kBlockThreads) substepCorrClusterKernel(const InstanceDev* __restrict__ insts,
                                                                         int substeps) {
  __shared__ double red[32];
  __shared__ double slots[2];
  cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
  const int cs = static_cast<int>(cl.num_blocks());
  const InstanceDev& I = insts[blockIdx.x / cs];
  const Team<true> tm{static_cast<int>(cl.block_rank()), cs};
  runSubstepsCorr<kLanesCluster, true, TIMED>(I, tm, substeps, I.y32, I.t32, red, slots);
}

// A batch as a work table: resident CTAs of WT threads each take the next cloth from an integer
// counter (the descriptors come largest first), run all of its substeps, and take another until the
// table is empty. A cloth is run by exactly one CTA, so its bits do not depend on which CTA takes it
// or when; the counter is the only shared word (integer atomics, no waiting on other CTAs). Against
// one 256-thread CTA per cloth all launched at once, a CTA has four times the threads to hide the
// solve's load latency, and no SM idles while another finishes a large cloth.
template <int WT, bool TIMED>
__global__ void __launch_bounds__(WT, 1024 / WT) substepCorrWorkKernel(const InstanceDev* __restrict__ insts,
                                                                       int count, int* counter, int substeps,
                                                                       int smemBytes) {
  extern __shared__ float sm[];
  __shared__ double red[32];
  __shared__ double slots[2];
  __shared__ int taken;
  for (;;) {
    if (threadIdx.x == 0) taken = atomicAdd(counter, 1);
    __syncthreads();
    const int idx = taken;
    __syncthreads();  // every thread has read `taken` before thread 0 takes the next cloth
    if (idx >= count) break;
    const InstanceDev& I = insts[idx];
    const bool inSmem = 24 * I.n <= smemBytes;  // Y, T: 3n floats each
    float* Y = inSmem ? sm : I.y32;
    float* T = inSmem ? sm + 3 * I.n : I.t32;
    const Team<false> tm{0, 1};
    runSubstepsCorr<kLanesOneCta, false, TIMED>(I, tm, substeps, Y, T, red, slots);
    __syncthreads();
  }
}

// One large cloth on a cooperative grid of CTAs (more SMs than a cluster holds): the cluster code
// path with grid barriers; the instance's FP64 solve workspace (unused by the correction kernels)
// holds the per-CTA slots of the team maxima.
template <bool TIMED>
__global__ void __launch_bounds__(kBlockThreads) substepCorrGridKernel(const InstanceDev* __restrict__ insts,
                                                                      int substeps) {
  __shared__ double red[32];
  __shared__ double slots[2];
  const InstanceDev& I = insts[0];
  Team<true> tm{static_cast<int>(blockIdx.x), static_cast<int>(gridDim.x)};
  tm.gslots = I.w;
  runSubstepsCorr<kLanesGrid, true, TIMED>(I, tm, substeps, I.y32, I.t32, red, slots);
}

cudaLaunchConfig_t corrClusterConfig(int blocks, int cs, void* stream, cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(kBlockThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = static_cast<cudaStream_t>(stream);
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

}  // namespace

int launchSubstepCorr(const InstanceDev* d, int count, int substeps, int smemBytes, void* stream, bool timed) {
  if (count <= 0 || substeps <= 0) return 0;
  static bool attrSet = false;
  if (!attrSet) {
    cudaFuncSetAttribute(substepCorrKernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(substepCorrKernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attrSet = true;
  }
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (timed) substepCorrKernel<true><<<count, kBlockThreads, smemBytes, st>>>(d, substeps, smemBytes);
  else substepCorrKernel<false><<<count, kBlockThreads, smemBytes, st>>>(d, substeps, smemBytes);
  return static_cast<int>(cudaGetLastError());
}

namespace {
template <int WT>
int launchWork(const InstanceDev* d, int count, int* counter, int substeps, int smemBytes, cudaStream_t st,
               bool timed) {
  static const bool attrSet = [] {
    cudaFuncSetAttribute(substepCorrWorkKernel<WT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(substepCorrWorkKernel<WT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    return true;
  }();
  (void)attrSet;
  int perSm = 0, dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, substepCorrWorkKernel<WT, false>, WT, smemBytes) !=
          cudaSuccess ||
      perSm <= 0) {
    cudaGetLastError();
    return static_cast<int>(cudaErrorInvalidConfiguration);
  }
  const int grid = std::max(1, std::min(count, perSm * sms));  // resident CTAs only: the rest would idle
  if (timed) substepCorrWorkKernel<WT, true><<<grid, WT, smemBytes, st>>>(d, count, counter, substeps, smemBytes);
  else substepCorrWorkKernel<WT, false><<<grid, WT, smemBytes, st>>>(d, count, counter, substeps, smemBytes);
  return static_cast<int>(cudaGetLastError());
}
}  // namespace

int launchSubstepCorrWork(const InstanceDev* d, int count, int* counter, int threads, int substeps, int smemBytes,
                          void* stream, bool timed) {
  if (count <= 0 || substeps <= 0) return 0;
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  const cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(int), st);  // the table starts at its first cloth
  if (e != cudaSuccess) return static_cast<int>(e);
  if (threads == 512) return launchWork<512>(d, count, counter, substeps, smemBytes, st, timed);
  if (threads == 1024) return launchWork<1024>(d, count, counter, substeps, smemBytes, st, timed);
  return static_cast<int>(cudaErrorInvalidValue);
}

int corrClusterSupported(int cs) {
  if (cs < 2 || cs > 16) return 0;
  for (auto kernel : {substepCorrClusterKernel<false>, substepCorrClusterKernel<true>}) {  // both must run
    if (cs > 8) cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = corrClusterConfig(cs, cs, nullptr, attr);
    int clusters = 0;
    const cudaError_t e = cudaOccupancyMaxActiveClusters(&clusters, kernel, &cfg);
    if (e != cudaSuccess) cudaGetLastError();
    if (e != cudaSuccess || clusters <= 0) return 0;
  }
  return cs;
}

int corrGridCapacity() {
  static int cached = -1;
  if (cached >= 0) return cached;
  int dev = 0, sms = 0, least = 1 << 30;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return cached = 0;
  }
  for (auto kernel : {substepCorrGridKernel<false>, substepCorrGridKernel<true>}) {  // both must fit
    int perSm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kernel, kBlockThreads, 0) != cudaSuccess) {
      cudaGetLastError();
      return cached = 0;
    }
    least = std::min(least, perSm);
  }
  return cached = least * sms;
}

int launchSubstepCorrGrid(const InstanceDev* d, int ctas, int substeps, void* stream, bool timed) {
  if (substeps <= 0) return 0;
  if (ctas < 2 || ctas > corrGridCapacity()) return static_cast<int>(cudaErrorCooperativeLaunchTooLarge);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ctas);
  cfg.blockDim = dim3(kBlockThreads);
  cfg.stream = static_cast<cudaStream_t>(stream);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const cudaError_t e = timed ? cudaLaunchKernelEx(&cfg, substepCorrGridKernel<true>, d, substeps)
                              : cudaLaunchKernelEx(&cfg, substepCorrGridKernel<false>, d, substeps);
  return static_cast<int>(e != cudaSuccess ? e : cudaGetLastError());
}

int launchSubstepCorrCluster(const InstanceDev* d, int count, int cs, int substeps, void* stream, bool timed) {
  if (count <= 0 || substeps <= 0) return 0;
  if (corrClusterSupported(cs) != cs) return static_cast<int>(cudaErrorInvalidConfiguration);
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = corrClusterConfig(count * cs, cs, stream, attr);
  const cudaError_t e = timed ? cudaLaunchKernelEx(&cfg, substepCorrClusterKernel<true>, d, substeps)
                              : cudaLaunchKernelEx(&cfg, substepCorrClusterKernel<false>, d, substeps);
  return static_cast<int>(e != cudaSuccess ? e : cudaGetLastError());
}

}  // namespace pdg
