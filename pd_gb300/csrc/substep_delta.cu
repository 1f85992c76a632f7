// substep_delta.cu — MIXED substeps of small cloths by a team of CTAs, the solve in correction
// form against the explicit FP32 inverse of Ã.
//
// The reference iteration x^{k+1} = L⁻¹·b(x^k) (Integrator.cpp:560-663) is computed here as
//   x^{k+1} = x^k + Ã⁻¹·r,   r = b(x^k) − Ã·x^k,
// which is the same map in exact arithmetic. r is small and smooth once the iteration is under
// way, so an FP32 inverse and FP32 arithmetic for r leave an error of about 2⁻²⁴·|x^{k+1} − x^k|
// per iteration instead of 2⁻²⁴·|x|, while positions keep ≈48-bit significands and the fixed
// point is the reference's (r = 0). r needs no matrix: with the projections d_e at x^k,
//   r_v = m_v/h²·(x̂_v − x_v) − Σ_e κ_e·((x_v − x_o) − d_e) + Σ_s (−k_s w_v)·(w_sᵀx)  (free v),
// the mass, edge and bend terms of Ã (Assembler.cpp:139-278) with pinned neighbours at q, and
// r_v = 0 with x_v = q_v for pinned rows. The same pass gives the reference's residual t_v
// (Integrator.cpp:230-263) of x^k for the convergence gate.
//
// GB300 layout: one cloth is run by `team` CTAs (up to one per SM), each owning a contiguous
// range of vertices, their incidences (in shared memory) and the matching rows of Ã⁻¹ (in shared
// memory when they fit). Per iteration a CTA computes r for its vertices in FP32 (positions as
// FP32 hi/lo pairs, so that differences keep FP64 accuracy) and publishes it; after exchange A it
// holds the whole r, applies its rows of Ã⁻¹ (FP32 FMA from shared memory), updates its positions
// and publishes them; after exchange B it holds the positions its vertices touch. Positions live
// as FP32 hi/lo pairs (≈48-bit significands) updated with an exact two-sum, so the iteration loop
// has no FP64 instruction — FP64 runs at 1/69 of the FP32 rate on this part; FP64 is left for the
// once-per-substep prediction and velocity update.
//
// Exchanges go through L2 as 64-bit words (epoch << 32 | FP32 bits) written and read with
// relaxed gpu-scope accesses: a reader polls the words it needs until each carries the current
// epoch, so an exchange costs about one L2 round trip after the last writer and needs no fence
// (a fence would also drop the L1 lines the CTA reads through). Per-CTA partial maxima (residual,
// displacement, scale) travel the same way, one per L2 line; one warp polls them while the
// others poll the data words. Polling does not back off: a store is visible to another SM about
// 250 ns later on the same die and 370 ns on the other, and a sleep between rounds only adds to
// that; each round waits for its own loads, so a waiting CTA keeps at most a few loads in flight
// per thread.
// Exchange A is a full barrier of the team; with the residual gate exchange B only waits for
// the CTAs whose positions a CTA reads, so r and the A partials alternate between two buffers.
// Every word is rewritten only after a later full barrier, which no CTA passes before every CTA
// has read it. The launch is cooperative so that every CTA of the team is resident, and every
// poll gives up after a bounded number of rounds, setting the instance's error flag.
#include <cstdint>

#include <algorithm>

#include "correction.cuh"
#include "device.cuh"

namespace pdg {
namespace {

constexpr int kWarps = kDeltaThreads / 32;
constexpr long long kSpinLimit = 1ll << 22; // poll rounds before an exchange gives up
constexpr int kMaxTeam = 256;               // partials one polling warp covers (kMaxTeam / 32 a lane)
constexpr int kGroup = 16;                  // lanes per vertex in the correction pass
constexpr int kRowBlock = 11;               // rows of Ã⁻¹ one warp applies together (33 sums, one transpose)
constexpr int kPartStride = 16;             // words between two CTAs' partials: one L2 line each

__device__ __forceinline__ unsigned long long loadRelaxed(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void storeRelaxed(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ unsigned long long tagged(unsigned tag, float v) {
  return (static_cast<unsigned long long>(tag) << 32) | __float_as_uint(v);
}

// Polls src[j] for j in [b, e) until each carries `tag` and hands its value to sink(j, value);
// thread `tid` of `nth` takes every nth word, B loads in flight. False if a word stayed stale for
// kSpinLimit rounds.
template <int B, class Sink>
__device__ __forceinline__ bool pollWords(const unsigned long long* src, int b, int e, unsigned tag, int tid, int nth,
                                          Sink&& sink) {
  for (int j0 = b + tid; j0 < e; j0 += B * nth) {
    unsigned pending = 0;
#pragma unroll
    for (int u = 0; u < B; ++u)
      if (j0 + u * nth < e) pending |= 1u << u;
    long long spins = 0;
    while (pending) {
      unsigned long long w[B];
#pragma unroll
      for (int u = 0; u < B; ++u) w[u] = ((pending >> u) & 1u) ? loadRelaxed(src + j0 + u * nth) : 0ull;
#pragma unroll
      for (int u = 0; u < B; ++u) {
        if (((pending >> u) & 1u) && static_cast<unsigned>(w[u] >> 32) == tag) {
          sink(j0 + u * nth, __uint_as_float(static_cast<unsigned>(w[u])));
          pending &= ~(1u << u);
        }
      }
      if (pending && ++spins > kSpinLimit) return false;
    }
  }
  return true;
}

__device__ __forceinline__ float warpMaxF(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Warp 0: maximum of the partials tagged `tag` of the team's ranks r ≡ first (mod step) into
// *out (other warps return true).
__device__ __forceinline__ bool pollPartials(const unsigned long long* ptag, int team, unsigned tag, float* out,
                                             int first = 0, int step = 1) {
  if (threadIdx.x >= 32) return true;
  const int lane = threadIdx.x;
  unsigned pending = 0;
#pragma unroll
  for (int i = 0; i < kMaxTeam / 32; ++i)
    if (first + step * (lane + 32 * i) < team) pending |= 1u << i;
  float mx = 0.f;
  long long spins = 0;
  bool good = true;
  while (true) {
    unsigned long long w[kMaxTeam / 32];
#pragma unroll
    for (int i = 0; i < kMaxTeam / 32; ++i)
      w[i] = ((pending >> i) & 1u) ? loadRelaxed(ptag + kPartStride * (first + step * (lane + 32 * i))) : 0ull;
#pragma unroll
    for (int i = 0; i < kMaxTeam / 32; ++i) {
      if (((pending >> i) & 1u) && static_cast<unsigned>(w[i] >> 32) == tag) {
        mx = fmaxf(mx, __uint_as_float(static_cast<unsigned>(w[i])));
        pending &= ~(1u << i);
      }
    }
    if (__all_sync(0xffffffffu, pending == 0)) break;
    if (++spins > kSpinLimit) {
      good = false;
      break;
    }
  }
  mx = warpMaxF(mx);
  if (lane == 0) *out = mx;
  return good;
}

template <int G>
__device__ __forceinline__ float groupSum(float v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warpMaxD(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// The displacement gate (Integrator.cpp:676-699) on the FP32 maximum g of the iteration's
// displacements: diff = (double)g passes when diff ≤ absTol or diff / scale ≤ relTol (diff itself
// when scale ≤ 0), each test only when its tolerance is positive. Both are monotone in g, so each
// holds exactly when g is at most the largest float that passes it; those thresholds are found once
// per substep (a failing test gets −∞).
__device__ __noinline__ void displacementThresholds(double absTol, double relTol, double scale, float* absF,
                                                    float* relF) {
  *absF = (absTol > 0.0) ? __double2float_rd(absTol) : -INFINITY;
  if (!(relTol > 0.0)) {
    *relF = -INFINITY;
    return;
  }
  if (!(scale > 0.0)) {
    *relF = __double2float_rd(relTol);
    return;
  }
  auto passes = [&](float g) { return static_cast<double>(g) / scale <= relTol; };
  float t = __double2float_rd(relTol * scale);
  for (int i = 0; i < 64 && !passes(t) && t > -INFINITY; ++i) t = nextafterf(t, -INFINITY);
  for (int i = 0; i < 64 && t < INFINITY && passes(nextafterf(t, INFINITY)); ++i) t = nextafterf(t, INFINITY);
  *relF = t;
}

// One step of a transposing warp reduction: lanes with bit O set keep the upper half of s[0, 2·O),
// the others the lower half, each adding the half its partner sends.
template <int O>
__device__ __forceinline__ void transposeStep(float* s, int lane) {
  const bool up = (lane & O) != 0;
#pragma unroll
  for (int i = 0; i < O; ++i) {
    const float send = up ? s[i] : s[i + O];
    const float keep = up ? s[i + O] : s[i];
    s[i] = keep + __shfl_xor_sync(0xffffffffu, send, O);
  }
}

// Rows [0, nr) (nr ≤ kRowBlock) of Ã⁻¹ starting at A0 (shared or global memory) times the three
// components of R, by warp `w` of `nw`: lane l takes the float4 columns w·32 + l, w·32 + l + 32·nw, ...
// so that R and the rows are read once by the nw warps together; the 3·nr sums are then reduced
// over the warp in 31 + 5 shuffles (a transpose of the first 32 and a butterfly of the last) and
// written to out[3·r + c], the warp's share of the row products.
template <bool SMEM, bool FULL>
__device__ __forceinline__ void rowBlock(const float* A0, int nrArg, const float* Rs, int ld, int w, int nw, float* out) {
  const int nr = FULL ? kRowBlock : nrArg;  // a full block has no per-row predicates
  const int lane = threadIdx.x & 31;
  const float4* a = reinterpret_cast<const float4*>(A0);
  const int ld4 = ld / 4;
  const float4* rx = reinterpret_cast<const float4*>(Rs);
  const float4* ry = reinterpret_cast<const float4*>(Rs + ld);
  const float4* rz = reinterpret_cast<const float4*>(Rs + 2 * ld);
  float s[3 * kRowBlock];
#pragma unroll
  for (int i = 0; i < 3 * kRowBlock; ++i) s[i] = 0.f;
  for (int j = 32 * w + lane; j < ld4; j += 32 * nw) {
    const float4 x = rx[j], y = ry[j], z = rz[j];
#pragma unroll
    for (int r = 0; r < kRowBlock; ++r) {
      if (r < nr) {
        const float4 u = SMEM ? a[r * ld4 + j] : __ldg(a + r * ld4 + j);
        s[3 * r] = fmaf(u.x, x.x, fmaf(u.y, x.y, fmaf(u.z, x.z, fmaf(u.w, x.w, s[3 * r]))));
        s[3 * r + 1] = fmaf(u.x, y.x, fmaf(u.y, y.y, fmaf(u.z, y.z, fmaf(u.w, y.w, s[3 * r + 1]))));
        s[3 * r + 2] = fmaf(u.x, z.x, fmaf(u.y, z.y, fmaf(u.z, z.z, fmaf(u.w, z.w, s[3 * r + 2]))));
      }
    }
  }
  transposeStep<16>(s, lane);
  transposeStep<8>(s, lane);
  transposeStep<4>(s, lane);
  transposeStep<2>(s, lane);
  transposeStep<1>(s, lane);  // lane l now holds the warp's sum of s[l]
  float e = s[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
  if (lane < 3 * nr) out[lane] = s[0];
  if (lane == 0 && 3 * nr > 32) out[32] = e;
}

template <bool TIMED>
__global__ void __launch_bounds__(kDeltaThreads, 1) substepDeltaKernel(const InstanceDev* __restrict__ insts,
                                                                      int team, int substeps) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ float red[kWarps];
  __shared__ float gate;
  __shared__ int gateHit;  // the gate's decision, taken once by thread 0 and read by every thread
  __shared__ float dispAbsF, dispRelF;  // the displacement gate's thresholds on the FP32 maximum
  __shared__ int failed;
  const int rank = static_cast<int>(blockIdx.x) % team;
  const InstanceDev& I = insts[blockIdx.x / team];
  const int n = I.n, ld = I.denseLd;
  const int chunk = (n + team - 1) / team;
  const int rb = min(n, rank * chunk), re = min(n, rb + chunk), m = re - rb;
  const int resRows = min(m, I.denseResRows);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  // shared memory (16-byte items first): positions as hi/lo pairs, the whole correction, resident
  // rows of Ã⁻¹, own incidences, vertex constants and x̂ (hi/lo), x_n and v (FP64), partial sums
  // of Δ per column segment, incidence offsets
  float4* Xs = reinterpret_cast<float4*>(smem);
  float* xf = reinterpret_cast<float*>(Xs);  // vertex v: hi at xf[8v + c], lo at xf[8v + 4 + c]
  float* Rs = reinterpret_cast<float*>(Xs + 2 * n);
  float* As = Rs + 3 * ld;
  int4* sE = reinterpret_cast<int4*>(As + static_cast<size_t>(I.denseResRows) * ld);
  int4* sB = sE + I.teamECap;
  float4* sV = reinterpret_cast<float4*>(sB + I.teamBCap);
  float4* sXh = sV + chunk;
  float4* sXp = sXh + 2 * chunk;  // window positions before an over-relaxed update (teamWCap pairs)
  double* xn64 = reinterpret_cast<double*>(sXp + 2 * I.teamWCap);
  double* v64 = xn64 + 3 * chunk;
  float* dl = reinterpret_cast<float*>(v64 + 3 * chunk);  // kDeltaProductWarps × 3·chunk
  int* sEb = reinterpret_cast<int*>(dl + kDeltaProductWarps * 3 * chunk);
  int* sBb = sEb + chunk + 1;

  if (threadIdx.x == 0) failed = 0;
  const int e0 = (m > 0) ? I.rstart[rb] : 0, b0 = (m > 0) ? I.bstart[rb] : 0;
  const int eN = (m > 0) ? I.rstart[re] - e0 : 0, bN = (m > 0) ? I.bstart[re] - b0 : 0;
  for (int t = threadIdx.x; t < eN; t += blockDim.x) sE[t] = I.tEdge[e0 + t];
  for (int t = threadIdx.x; t < bN; t += blockDim.x) sB[t] = I.tBend[b0 + t];
  for (int t = threadIdx.x; t < m; t += blockDim.x) sV[t] = I.tVtx[rb + t];
  for (int t = threadIdx.x; t <= m; t += blockDim.x) {
    sEb[t] = I.rstart[rb + t] - e0;
    sBb[t] = I.bstart[rb + t] - b0;
  }
  for (int t = threadIdx.x; t < 3 * m; t += blockDim.x) v64[t] = I.v[3 * rb + t];
  for (int v = threadIdx.x; v < n; v += blockDim.x) {
    float4 h, l;
    split(I.x[3 * v], h.x, l.x);
    split(I.x[3 * v + 1], h.y, l.y);
    split(I.x[3 * v + 2], h.z, l.z);
    h.w = l.w = 0.f;
    Xs[2 * v] = h;
    Xs[2 * v + 1] = l;
  }
  for (int j = n + threadIdx.x; j < ld; j += blockDim.x) Rs[j] = Rs[ld + j] = Rs[2 * ld + j] = 0.f;
  {
    const float4* src = reinterpret_cast<const float4*>(I.Ainv + static_cast<size_t>(rb) * ld);
    float4* dst = reinterpret_cast<float4*>(As);
    const int total = resRows * (ld / 4);
    for (int t = threadIdx.x; t < total; t += blockDim.x) dst[t] = __ldg(src + t);
  }
  unsigned epoch = *I.epoch;  // exchanges of this launch continue the previous launch's epochs
  // exchange words: r and the A partials alternate between two buffers (by A epoch), since with
  // the residual gate exchange B only waits for the CTAs whose positions a CTA reads
  unsigned long long* ptagB = I.ptag + 2 * kPartStride * team;
  const int wlo = I.window[2 * rank], whi = I.window[2 * rank + 1];
  // loop invariants kept in registers (the relaxed accesses' memory clobbers would reload them)
  const int useRes = I.useResidual, maxIter = I.maxIter, chebFrom = I.chebFrom, withhold = I.withholdRank;
  unsigned long long* const rtagBase = I.rtag;
  unsigned long long* const ptagBase = I.ptag;
  unsigned long long* const xtag = I.xtag;
  const double* const omegaP = I.omega;
  double* const resTraceP = I.resTrace;
  const float* const qf = reinterpret_cast<const float*>(I.qhl);
  float* const xhf = reinterpret_cast<float*>(sXh);  // x̂ of own vertex li: hi at 8·li + c, lo at 8·li + 4 + c
  // the residual gate in FP32: for a float g, (double)g ≤ T exactly when g ≤ T rounded down to a float
  const float resThrF = __double2float_rd(I.resThreshold);
  __syncthreads();

  const StageClock<TIMED> clk(I, rank == 0 && threadIdx.x == 0);
  for (int step = 0; step < substeps; ++step) {
    // predict own rows (Integrator.cpp:447-472), x̂ kept as a hi/lo pair
    double sc = 0.0;
    for (int t = threadIdx.x; t < 3 * m; t += blockDim.x) {
      const int li = t / 3, c = t - 3 * li, v = rb + li;
      const double p = static_cast<double>(xf[8 * v + c]) + static_cast<double>(xf[8 * v + 4 + c]);
      const double xh = (p + v64[t] * I.h) + I.gh2[c];
      xn64[t] = p;
      float hi, lo;
      split(xh, hi, lo);
      xhf[8 * li + c] = hi;
      xhf[8 * li + 4 + c] = lo;
      sc = fmax(sc, fabs(xh - p));
    }
    const float scW = static_cast<float>(warpMaxD(sc));
    __syncthreads();  // x̂ of own rows is read by other threads below
    clk.lap(I, rank == 0 && threadIdx.x == 0, kStagePredict);
    double scale = 0.0;
    int used = 0;
    bool conv = false;
    float lastRes = I.useResidual ? 0.f : -1.f;  // the gate's FP32 maximum (exact in FP64)
    float resSplit = 0.f;  // residual of the last over-relaxed iteration's solve (per thread)
    for (int k = 0;; ++k) {
      // an over-relaxed iteration with the residual gate (Integrator.cpp:631-663) puts x^k + Δ,
      // takes that point's residual, then adds (ω − 1)·Δ to every window vertex
      const bool blend = k >= chebFrom && k < maxIter;
      const bool split = blend && useRes;
      const bool splitBefore = useRes && k >= 1 && k - 1 >= chebFrom;
      const float om = blend ? static_cast<float>(omegaP[k]) : 1.f;
      if (split)
        for (int t = threadIdx.x; t < 2 * (whi - wlo); t += blockDim.x) sXp[t] = Xs[2 * wlo + t];
      const unsigned tagA = ++epoch;  // odd: epochs are consumed in (A, B) pairs
      const unsigned buf = (tagA >> 1) & 1u;
      unsigned long long* rtag = rtagBase + buf * 3 * n;
      unsigned long long* ptagA = ptagBase + buf * kPartStride * team;
      // correction r and residual of x^k for own vertices, kGroup lanes per vertex (FP32 only)
      float resLocal = 0.f;
      const int gl = threadIdx.x & (kGroup - 1), group = threadIdx.x / kGroup, ngroups = blockDim.x / kGroup;
      for (int base = 0; base < m; base += ngroups) {
        const int li = base + group;
        const bool active = li < m;
        const float4 vc = active ? sV[li] : make_float4(0.f, 0.f, 1.f, 0.f);
        const int v = rb + li;
        CorrectionSums cs;
        if (vc.z == 0.f) {
          const float4 vh = Xs[2 * v], vl = Xs[2 * v + 1];
          cs.accumulate(I, sE, sEb[li], sEb[li + 1], sB, sBb[li], sBb[li + 1], Xs, vh, vl, gl, kGroup);
          if (gl == 0) cs.addMass(vh, vl, sXh[2 * li], sXh[2 * li + 1], vc.x);
        }
        cs.reduce<kGroup>();
        if (active && gl == 0) {
          float3 r = make_float3(0.f, 0.f, 0.f);
          if (vc.z == 0.f) {
            if (vc.y > 0.f) resLocal = fmaxf(resLocal, cs.residual(vc.y));
            r = cs.correction();
          }
          storeRelaxed(rtag + 3 * v, tagged(tagA, r.x));
          storeRelaxed(rtag + 3 * v + 1, tagged(tagA, r.y));
          storeRelaxed(rtag + 3 * v + 2, tagged(tagA, r.z));
        }
      }
      // exchange A, a full barrier of the team: the whole correction (warps 1..) and the maximum
      // of the residuals — at k = 0 of the scale — (warp 0)
      if (splitBefore) resLocal = resSplit;  // iteration k − 1 is gated on its solve's residual
      resLocal = warpMaxF(resLocal);
      if (lane == 0) red[warp] = (k == 0) ? scW : resLocal;
      __syncthreads();
      clk.lap(I, rank == 0 && threadIdx.x == 0, kStageLocal);  // the correction pass: projection, scatter and residual in one
      bool ok = true;
      if (warp == 0) {
        if (lane == 0) {
          float pm = 0.f;
          for (int w = 0; w < kWarps; ++w) pm = fmaxf(pm, red[w]);
          if (!(withhold == rank && step == 0 && k == 0))
            storeRelaxed(ptagA + kPartStride * rank, tagged(tagA, pm));
        }
        __syncwarp();
        ok = pollPartials(ptagA, team, tagA, &gate);
        // the residual gate's decision (the reference's FP64 comparison, taken exactly in FP32), once
        if (lane == 0) gateHit = (k >= 1 && gate <= resThrF) ? 1 : 0;
      } else {
        ok = pollWords<10>(rtag, 0, 3 * n, tagA, threadIdx.x - 32, blockDim.x - 32, [&](int j, float val) {
          const int v = j / 3;
          Rs[(j - 3 * v) * ld + v] = val;
        });
      }
      if (!ok) failed = 1;
      __syncthreads();
      if (failed) break;
      if (k == 0) {
        const double gateA = gate;
        scale = (gateA < I.gScaleHH) ? I.gScaleHH : gateA;
        if (threadIdx.x == 0 && !useRes) displacementThresholds(I.absTol, I.relTol, scale, &dispAbsF, &dispRelF);
      }
      bool stop = k == maxIter;
      if (useRes && k >= 1) {
        used = k;
        if (threadIdx.x == 0) {  // the only thread that reports them
          lastRes = gate;
          if (resTraceP && rank == 0) resTraceP[(size_t)step * maxIter + k - 1] = gate;
        }
        conv = gateHit != 0;
        stop = stop || conv;
      }
      if (stop) {
        ++epoch;  // the unused B epoch: the next A epoch stays odd
        break;
      }

      // this CTA's rows of Ã⁻¹·r: blocks of up to kRowBlock rows, each applied by kDeltaProductWarps
      // warps over interleaved columns (resident rows from shared memory, the rest through L2)
      if (warp < kDeltaProductWarps) {
        for (int li = 0; li < m;) {
          const bool resident = li < resRows;
          const int nr = min(kRowBlock, (resident ? resRows : m) - li);
          float* out = dl + warp * 3 * chunk + 3 * li;
          const float* A0 = resident ? As + static_cast<size_t>(li) * ld : I.Ainv + static_cast<size_t>(rb + li) * ld;
          if (resident && nr == kRowBlock)
            rowBlock<true, true>(A0, nr, Rs, ld, warp, kDeltaProductWarps, out);
          else if (resident)
            rowBlock<true, false>(A0, nr, Rs, ld, warp, kDeltaProductWarps, out);
          else
            rowBlock<false, false>(A0, nr, Rs, ld, warp, kDeltaProductWarps, out);
          li += nr;
        }
      }
      __syncthreads();
      clk.lap(I, rank == 0 && threadIdx.x == 0, kStageSolve);  // exchange A (the whole correction) and this CTA's rows of Ã⁻¹·r
      // x^{k+1} = x^k + Δ as hi/lo pairs (pinned rows: q), published for the team
      const unsigned tagB = ++epoch;
      float dmax = 0.f;
      for (int t = threadIdx.x; t < 3 * m; t += blockDim.x) {
        const int li = t / 3, c = t - 3 * li, v = rb + li;
        float hi = xf[8 * v + c], lo = xf[8 * v + 4 + c];
        if (sV[li].z != 0.f) {
          const float qh = __ldg(qf + 8 * v + c), ql = __ldg(qf + 8 * v + 4 + c);
          const float d = (qh - hi) + (ql - lo);
          dmax = fmaxf(dmax, fabsf(om * d));
          hi = qh;
          lo = ql;
          if (blend && !split) addHL(hi, lo, (om - 1.f) * d);
        } else {
          float d = dl[t];
#pragma unroll
          for (int w = 1; w < kDeltaProductWarps; ++w) d += dl[w * 3 * chunk + t];
          dmax = fmaxf(dmax, fabsf(om * d));
          addHL(hi, lo, (blend && !split) ? om * d : d);
        }
        storeRelaxed(xtag + 6 * v + c, tagged(tagB, hi));
        storeRelaxed(xtag + 6 * v + 3 + c, tagged(tagB, lo));
      }
      // exchange B: the positions this CTA reads; with the displacement gate also the maximum of
      // the displacements (warp 0), which makes it a full barrier — with the residual gate a CTA
      // waits only for the CTAs owning its window
      __syncthreads();  // own positions are read back by other threads below
      if (!useRes) {
        dmax = warpMaxF(dmax);
        if (lane == 0) red[warp] = dmax;
        __syncthreads();
        if (warp == 0) {
          if (lane == 0) {
            float pm = 0.f;
            for (int w = 0; w < kWarps; ++w) pm = fmaxf(pm, red[w]);
            storeRelaxed(ptagB + kPartStride * rank, tagged(tagB, pm));
          }
          __syncwarp();
          ok = pollPartials(ptagB, team, tagB, &gate);
          if (lane == 0)  // the displacement gate's decision, once, on thresholds taken at k = 0
            gateHit = (gate <= dispAbsF) || (gate <= dispRelF) ? 1 : 0;
        } else {
          ok = pollWords<4>(xtag, 6 * wlo, 6 * whi, tagB, threadIdx.x - 32, blockDim.x - 32, [&](int j, float val) {
            const int v = j / 6, c = j - 6 * v;  // c < 3: hi, else lo
            xf[8 * v + (c < 3 ? c : c + 1)] = val;
          });
        }
      } else {
        ok = pollWords<4>(xtag, 6 * wlo, 6 * whi, tagB, threadIdx.x, blockDim.x, [&](int j, float val) {
          const int v = j / 6, c = j - 6 * v;
          xf[8 * v + (c < 3 ? c : c + 1)] = val;
        });
      }
      if (!ok) failed = 1;
      __syncthreads();
      if (failed) break;
      clk.lap(I, rank == 0 && threadIdx.x == 0, kStageUnpack);  // the two-sum update and exchange B (the window's positions)
      if (split) {
        // residual of x^k + Δ for own vertices, sent with the next exchange A
        resSplit = 0.f;
        for (int base = 0; base < m; base += ngroups) {
          const int li = base + group;
          const bool active = li < m;
          const float4 vc = active ? sV[li] : make_float4(0.f, 0.f, 1.f, 0.f);
          const int v = rb + li;
          CorrectionSums cs;
          if (vc.z == 0.f) {
            const float4 vh = Xs[2 * v], vl = Xs[2 * v + 1];
            cs.accumulate(I, sE, sEb[li], sEb[li + 1], sB, sBb[li], sBb[li + 1], Xs, vh, vl, gl, kGroup);
            if (gl == 0) cs.addMass(vh, vl, sXh[2 * li], sXh[2 * li + 1], vc.x);
          }
          cs.reduce<kGroup>();
          if (active && gl == 0 && vc.z == 0.f && vc.y > 0.f) resSplit = fmaxf(resSplit, cs.residual(vc.y));
        }
        __syncthreads();
        // x^{k+1} = (x^k + Δ) + (ω − 1)·Δ over the whole window, Δ recovered from the pairs, so
        // that every CTA reading a vertex computes the same bits as its owner
        for (int j = threadIdx.x; j < whi - wlo; j += blockDim.x) {
          const int v = wlo + j;
          float4 h = Xs[2 * v], l = Xs[2 * v + 1];
          const float3 d = diffHL(h, l, sXp[2 * j], sXp[2 * j + 1]);
          addHL(h.x, l.x, (om - 1.f) * d.x);
          addHL(h.y, l.y, (om - 1.f) * d.y);
          addHL(h.z, l.z, (om - 1.f) * d.z);
          Xs[2 * v] = h;
          Xs[2 * v + 1] = l;
        }
        __syncthreads();
      }
      if (!useRes) {
        used = k + 1;
        conv = gateHit != 0;
        if (conv) break;
      }
    }
    if (failed) {
      if (threadIdx.x == 0) atomicExch(I.err, 1);
      return;
    }
    // velocity, damping, pin resnap (Integrator.cpp:774-791)
    for (int t = threadIdx.x; t < 3 * m; t += blockDim.x) {
      const int li = t / 3, c = t - 3 * li, v = rb + li;
      if (sV[li].z != 0.f) {
        v64[t] = 0.0;
      } else {
        const double x = static_cast<double>(xf[8 * v + c]) + static_cast<double>(xf[8 * v + 4 + c]);
        v64[t] = (x - xn64[t]) * I.dampInvH;
      }
    }
    if (used == 0) {  // no update ran: pinned vertices are resnapped to q everywhere
      for (int v = threadIdx.x; v < n; v += blockDim.x)
        if (I.pinned[v]) pinHL(I, v, Xs[2 * v], Xs[2 * v + 1]);
    }
    if (rank == 0 && threadIdx.x == 0) {
      if (I.iterLog) I.iterLog[step] = used;
      if (I.convLog) I.convLog[step] = conv ? 1 : 0;
      *I.lastResidual = lastRes;
      *I.iterationsUsed = used;
      *I.converged = conv ? 1 : 0;
      if (conv) *I.earlyExits += 1;
    }
    __syncthreads();
    clk.lap(I, rank == 0 && threadIdx.x == 0, kStageVelocity);
    clk.finish(I, rank == 0 && threadIdx.x == 0);
  }
  if (rank == 0 && threadIdx.x == 0) *I.epoch = epoch;
  for (int t = threadIdx.x; t < 3 * m; t += blockDim.x) {
    const int li = t / 3, c = t - 3 * li, v = rb + li;
    I.x[3 * rb + t] = (sV[li].z != 0.f) ? I.q[3 * v + c]
                                         : static_cast<double>(xf[8 * v + c]) + static_cast<double>(xf[8 * v + 4 + c]);
    I.v[3 * rb + t] = v64[t];
    I.xn[3 * rb + t] = xn64[t];
  }
}

}  // namespace

int deltaResidentCtas(int smemBytes) {
  constexpr int kMaxDynamic = 224 * 1024;  // leaves room for the kernel's static shared memory
  if (smemBytes > kMaxDynamic) return 0;
  int least = 1 << 30;
  for (auto kernel : {substepDeltaKernel<false>, substepDeltaKernel<true>}) {  // both must fit
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynamic);
    int perSm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kernel, kDeltaThreads, smemBytes) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    least = std::min(least, perSm);
  }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return least * sms;
}

int launchSubstepDelta(const InstanceDev* d, int count, int team, int smemBytes, int substeps, void* stream,
                       bool timed) {
  if (count <= 0 || substeps <= 0) return 0;
  if (team > kMaxTeam || deltaResidentCtas(smemBytes) < count * team)
    return static_cast<int>(cudaErrorCooperativeLaunchTooLarge);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(count * team);
  cfg.blockDim = dim3(kDeltaThreads);
  cfg.dynamicSmemBytes = smemBytes;
  cfg.stream = static_cast<cudaStream_t>(stream);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const cudaError_t e = timed ? cudaLaunchKernelEx(&cfg, substepDeltaKernel<true>, d, team, substeps)
                              : cudaLaunchKernelEx(&cfg, substepDeltaKernel<false>, d, team, substeps);
  return static_cast<int>(e != cudaSuccess ? e : cudaGetLastError());
}

}  // namespace pdg
