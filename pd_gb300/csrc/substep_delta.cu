// substep_delta.cu — MIXED substeps of small cloths by a team of CTAs, the solve in correction
// form against the explicit FP32 inverse of Ã.
//
// The reference iteration x^{k+1} = L⁻¹·b(x^k) (Integrator.cpp:560-663) is computed here as
//   x^{k+1} = x^k + Ã⁻¹·r,   r = b(x^k) − Ã·x^k,
// which is the same map in exact arithmetic. r is small and smooth once the iteration is under
// way, so an FP32 inverse and FP32 arithmetic for r leave an error of about 2⁻²⁴·|x^{k+1} − x^k|
// per iteration instead of 2⁻²⁴·|x|, while positions stay FP64 and the fixed point is exactly
// the reference's (r = 0). r needs no matrix: with the projections d_e at x^k,
//   r_v = m_v/h²·(x̂_v − x_v) − Σ_e ±κ_e·(x_a − x_b − d_e) + Σ_s (−k_s w_v)·(w_sᵀx)  (free v),
// the mass, edge and bend terms of Ã (Assembler.cpp:139-278) with pinned neighbours at q, and
// r_v = 0 with x_v = q_v for pinned rows. The same pass gives the reference's residual t_v
// (Integrator.cpp:230-263) of x^k for the convergence gate.
//
// GB300 layout: one cloth is run by `team` CTAs (up to one per SM), each owning a contiguous
// range of vertices and the matching rows of Ã⁻¹, kept in its shared memory when they fit. Per
// iteration a CTA computes r for its vertices (FP32, positions as FP32 hi/lo pairs so that
// differences keep FP64 accuracy), publishes them to L2, meets the team at a barrier, reads the
// whole r, applies its rows of Ã⁻¹ (FP32 FMA from shared memory), updates its positions in FP64,
// publishes them and meets the team again. FP64 instructions — 1/69 of the FP32 rate on this
// part — are left only for the per-vertex position updates. The team barrier is an arrival
// counter in global memory polled with acquire loads; the launch is cooperative so that every CTA
// of the team is resident, and every wait gives up after a bounded number of polls, setting the
// instance's error flag.
#include <cstdint>

#include "device.cuh"

namespace pdg {
namespace {

constexpr int kWarps = kDeltaThreads / 32;
constexpr int kGroup = 16;                 // lanes per vertex in the correction pass
constexpr long long kSpinLimit = 1ll << 22; // polls of the team counter before giving up

__device__ __forceinline__ unsigned long long loadAcquire(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Barrier of the team's CTAs. `publish` runs in thread 0 after the CTA's own threads have met and
// before the arrival is released. Returns false in every thread when the wait gave up.
template <class Publish>
__device__ __forceinline__ bool teamBarrier(const InstanceDev& I, int team, unsigned long long& target,
                                            volatile int* flag, Publish&& publish) {
  __syncthreads();
  if (threadIdx.x == 0) {
    publish();
    target += static_cast<unsigned long long>(team);
    __threadfence();
    atomicAdd(I.bar, 1ull);
    int ok = 1;
    long long spins = 0;
    while (loadAcquire(I.bar) < target) {
      if (++spins > kSpinLimit) {
        ok = 0;
        atomicExch(I.err, 1);
        break;
      }
    }
    __threadfence();
    *flag = ok;
  }
  __syncthreads();
  return *flag != 0;
}

template <int G>
__device__ __forceinline__ float groupSum(float v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ float warpMaxF(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ double warpMaxD(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// FP64 value as an FP32 pair with hi + lo = v to ~2⁻⁴⁸ relative.
__device__ __forceinline__ void split(double v, float& hi, float& lo) {
  hi = static_cast<float>(v);
  lo = static_cast<float>(v - static_cast<double>(hi));
}

// Difference of two positions held as hi/lo pairs, to FP32 rounding of the result.
__device__ __forceinline__ float3 diffHL(float4 ah, float4 al, float4 bh, float4 bl) {
  return make_float3((ah.x - bh.x) + (al.x - bl.x), (ah.y - bh.y) + (al.y - bl.y), (ah.z - bh.z) + (al.z - bl.z));
}

__device__ __forceinline__ void pinHL(const InstanceDev& I, int u, float4& h, float4& l) {
  split(I.q[3 * u], h.x, l.x);
  split(I.q[3 * u + 1], h.y, l.y);
  split(I.q[3 * u + 2], h.z, l.z);
  h.w = l.w = 0.f;
}

// Rows of Ã⁻¹ times the three components of R, two rows per warp; A rows from shared or global
// memory. Sums of the pair land in dl[3·li + c].
template <bool SMEM>
__device__ __forceinline__ void rowPair(const float* A0, const float* A1, bool two, const float* Rs, int ld, int li,
                                        float* dl) {
  const int lane = threadIdx.x & 31;
  const float4* a0 = reinterpret_cast<const float4*>(A0);
  const float4* a1 = reinterpret_cast<const float4*>(A1);
  const float4* rx = reinterpret_cast<const float4*>(Rs);
  const float4* ry = reinterpret_cast<const float4*>(Rs + ld);
  const float4* rz = reinterpret_cast<const float4*>(Rs + 2 * ld);
  float s0 = 0.f, s1 = 0.f, s2 = 0.f, t0 = 0.f, t1 = 0.f, t2 = 0.f;
  const int q4 = ld / 4;
#pragma unroll 4
  for (int j = lane; j < q4; j += 32) {
    const float4 x = rx[j], y = ry[j], z = rz[j];
    const float4 u = SMEM ? a0[j] : __ldg(a0 + j);
    const float4 w = SMEM ? a1[j] : __ldg(a1 + j);
    s0 = fmaf(u.x, x.x, fmaf(u.y, x.y, fmaf(u.z, x.z, fmaf(u.w, x.w, s0))));
    s1 = fmaf(u.x, y.x, fmaf(u.y, y.y, fmaf(u.z, y.z, fmaf(u.w, y.w, s1))));
    s2 = fmaf(u.x, z.x, fmaf(u.y, z.y, fmaf(u.z, z.z, fmaf(u.w, z.w, s2))));
    t0 = fmaf(w.x, x.x, fmaf(w.y, x.y, fmaf(w.z, x.z, fmaf(w.w, x.w, t0))));
    t1 = fmaf(w.x, y.x, fmaf(w.y, y.y, fmaf(w.z, y.z, fmaf(w.w, y.w, t1))));
    t2 = fmaf(w.x, z.x, fmaf(w.y, z.y, fmaf(w.z, z.z, fmaf(w.w, z.w, t2))));
  }
  s0 = groupSum<32>(s0);
  s1 = groupSum<32>(s1);
  s2 = groupSum<32>(s2);
  t0 = groupSum<32>(t0);
  t1 = groupSum<32>(t1);
  t2 = groupSum<32>(t2);
  if (lane == 0) {
    dl[3 * li] = s0;
    dl[3 * li + 1] = s1;
    dl[3 * li + 2] = s2;
    if (two) {
      dl[3 * li + 3] = t0;
      dl[3 * li + 4] = t1;
      dl[3 * li + 5] = t2;
    }
  }
}

__global__ void __launch_bounds__(kDeltaThreads, 1) substepDeltaKernel(const InstanceDev* __restrict__ insts,
                                                                      int team, int substeps) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double redD[kWarps];
  __shared__ float redF[kWarps];
  __shared__ double gate[3];
  __shared__ int flag;
  const int rank = static_cast<int>(blockIdx.x) % team;
  const InstanceDev& I = insts[blockIdx.x / team];
  const int n = I.n, ld = I.denseLd;
  const int chunk = (n + team - 1) / team;
  const int rb = min(n, rank * chunk), re = min(n, rb + chunk), m = re - rb;
  const int resRows = min(m, I.denseResRows);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  // shared memory: all positions (hi/lo), the whole correction, resident rows of Ã⁻¹, own FP64 state
  float4* Xs = reinterpret_cast<float4*>(smem);
  float* Rs = reinterpret_cast<float*>(Xs + 2 * n);
  float* As = Rs + 3 * ld;
  double* xo = reinterpret_cast<double*>(As + static_cast<size_t>(I.denseResRows) * ld);
  double* xno = xo + 3 * chunk;
  double* xho = xno + 3 * chunk;
  double* vo = xho + 3 * chunk;
  float* dl = reinterpret_cast<float*>(vo + 3 * chunk);
  float4* xbuf4 = reinterpret_cast<float4*>(I.xbuf);

  for (int t = threadIdx.x; t < 3 * m; t += blockDim.x) {
    xo[t] = I.x[3 * rb + t];
    vo[t] = I.v[3 * rb + t];
  }
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
  // barrier arrivals so far: a multiple of `team` (no CTA can pass the first barrier before this
  // CTA arrives there, so at most team − 1 arrivals of this launch can have been counted)
  unsigned long long target = 0;
  if (threadIdx.x == 0) target = loadAcquire(I.bar) / team * team;
  int parity = 0;
  __syncthreads();

  for (int step = 0; step < substeps; ++step) {
    // predict own rows (Integrator.cpp:447-472)
    double sc = 0.0;
    for (int t = threadIdx.x; t < 3 * m; t += blockDim.x) {
      const int c = t % 3;
      const double p = xo[t];
      const double xh = (p + vo[t] * I.h) + I.gh2[c];
      xno[t] = p;
      xho[t] = xh;
      sc = fmax(sc, fabs(xh - p));
    }
    sc = warpMaxD(sc);
    if (lane == 0) redD[warp] = sc;
    __syncthreads();  // x̂ of own rows is read by other threads below
    double scale = 0.0;
    int used = 0;
    bool conv = false;
    double lastRes = I.useResidual ? 0.0 : -1.0;
    for (int k = 0;; ++k) {
      // correction r and residual of x^k for own vertices, kGroup lanes per vertex
      float resLocal = 0.f;
      const int gl = threadIdx.x & (kGroup - 1), group = threadIdx.x / kGroup, ngroups = blockDim.x / kGroup;
      for (int base = 0; base < m; base += ngroups) {
        const int li = base + group;
        const bool active = li < m;
        const int v = rb + (active ? li : 0);
        // a: mass + edge terms of the residual, f: its bend terms, p: what the matrix adds to
        // −(a) + f because it couples pinned neighbours at q rather than at their positions
        float a0 = 0.f, a1 = 0.f, a2 = 0.f, f0 = 0.f, f1 = 0.f, f2 = 0.f, p0 = 0.f, p1 = 0.f, p2 = 0.f;
        if (active && !I.pinned[v]) {
          for (int q = I.rstart[v] + gl; q < I.rstart[v + 1]; q += kGroup) {
            const int p = I.rinc[q];
            const int e = p >> 1;
            const int a = I.eab[2 * e], b = I.eab[2 * e + 1];
            const float4 ah = Xs[2 * a], al = Xs[2 * a + 1], bh = Xs[2 * b], bl = Xs[2 * b + 1];
            const float3 rel = diffHL(ah, al, bh, bl);
            const float rest = __ldg(I.edge32 + 2 * e), kap = __ldg(I.edge32 + 2 * e + 1);
            const float len = sqrtf(rel.x * rel.x + rel.y * rel.y + rel.z * rel.z);
            float dx = 0.f, dy = 0.f, dz = 0.f;
            if (!(len <= 1e-12f)) {
              const float s = rest / len;
              dx = rel.x * s;
              dy = rel.y * s;
              dz = rel.z * s;
            }
            const float sg = (p & 1) ? -1.f : 1.f;
            // residual: rc_e = κ·(x_a − x_b) − κ·d_e at the current positions
            a0 = fmaf(sg * kap, rel.x - dx, a0);
            a1 = fmaf(sg * kap, rel.y - dy, a1);
            a2 = fmaf(sg * kap, rel.z - dz, a2);
            // the matrix couples a free vertex to a pinned neighbour at q, not at its position
            const int other = (p & 1) ? a : b;
            if (I.pinned[other]) {
              float4 qh, ql;
              pinHL(I, other, qh, ql);
              const float3 relq = (p & 1) ? diffHL(qh, ql, bh, bl) : diffHL(ah, al, qh, ql);
              p0 = fmaf(sg * kap, relq.x - rel.x, p0);
              p1 = fmaf(sg * kap, relq.y - rel.y, p1);
              p2 = fmaf(sg * kap, relq.z - rel.z, p2);
            }
          }
          for (int q = I.bstart[v] + gl; q < I.bstart[v + 1]; q += kGroup) {
            const int s = I.binc[q];
            const int a = I.babc[3 * s], b = I.babc[3 * s + 1], c = I.babc[3 * s + 2];
            const float fac = __ldg(I.bfac32 + q);
            float4 ah = Xs[2 * a], al = Xs[2 * a + 1], bh = Xs[2 * b], bl = Xs[2 * b + 1], ch = Xs[2 * c],
                   cl = Xs[2 * c + 1];
            const float3 u = diffHL(ah, al, bh, bl), w = diffHL(ch, cl, bh, bl);
            f0 = fmaf(fac, u.x + w.x, f0);
            f1 = fmaf(fac, u.y + w.y, f1);
            f2 = fmaf(fac, u.z + w.z, f2);
            const bool pa = I.pinned[a], pb = I.pinned[b], pc = I.pinned[c];
            if (pa || pb || pc) {  // matrix part with pinned members at q
              if (pa) pinHL(I, a, ah, al);
              if (pb) pinHL(I, b, bh, bl);
              if (pc) pinHL(I, c, ch, cl);
              const float3 uq = diffHL(ah, al, bh, bl), wq = diffHL(ch, cl, bh, bl);
              p0 = fmaf(fac, (u.x + w.x) - (uq.x + wq.x), p0);
              p1 = fmaf(fac, (u.y + w.y) - (uq.y + wq.y), p1);
              p2 = fmaf(fac, (u.z + w.z) - (uq.z + wq.z), p2);
            }
          }
        }
        a0 = groupSum<kGroup>(a0);
        a1 = groupSum<kGroup>(a1);
        a2 = groupSum<kGroup>(a2);
        f0 = groupSum<kGroup>(f0);
        f1 = groupSum<kGroup>(f1);
        f2 = groupSum<kGroup>(f2);
        p0 = groupSum<kGroup>(p0);
        p1 = groupSum<kGroup>(p1);
        p2 = groupSum<kGroup>(p2);
        if (active && gl == 0) {
          float r0 = 0.f, r1 = 0.f, r2 = 0.f;
          if (!I.pinned[v]) {
            const float mh2 = __ldg(I.vtx32 + 2 * v), invM = __ldg(I.vtx32 + 2 * v + 1);
            a0 = fmaf(static_cast<float>(xo[3 * li] - xho[3 * li]), mh2, a0);
            a1 = fmaf(static_cast<float>(xo[3 * li + 1] - xho[3 * li + 1]), mh2, a1);
            a2 = fmaf(static_cast<float>(xo[3 * li + 2] - xho[3 * li + 2]), mh2, a2);
            if (invM > 0.f) {
              const float t0 = a0 + f0, t1 = a1 + f1, t2 = a2 + f2;
              resLocal = fmaxf(resLocal, sqrtf(t0 * t0 + t1 * t1 + t2 * t2) * invM);
            }
            // r = −(mass + edge terms) + bend terms with pinned neighbours at q (the pinned part
            // of the bend terms is the reference's constant bending RHS)
            r0 = (f0 - a0) - p0;
            r1 = (f1 - a1) - p1;
            r2 = (f2 - a2) - p2;
          }
          I.rbuf[v] = r0;
          I.rbuf[ld + v] = r1;
          I.rbuf[2 * ld + v] = r2;
        }
      }
      resLocal = warpMaxF(resLocal);
      if (lane == 0) redF[warp] = resLocal;
      // barrier A: the correction is complete; partial maxima of the residual (and at k = 0 the scale)
      double* slotA = I.part + 3 * (parity * team + rank);
      if (!teamBarrier(I, team, target, &flag, [&] {
            double rm = 0.0, sm = 0.0;
            for (int w = 0; w < kWarps; ++w) {
              rm = fmax(rm, static_cast<double>(redF[w]));
              sm = fmax(sm, redD[w]);
            }
            slotA[0] = rm;
            slotA[2] = sm;
          }))
        return;
      if (warp == 0) {
        double rm = 0.0, sm = 0.0;
        for (int r = lane; r < team; r += 32) {
          rm = fmax(rm, __ldcg(I.part + 3 * (parity * team + r)));
          sm = fmax(sm, __ldcg(I.part + 3 * (parity * team + r) + 2));
        }
        rm = warpMaxD(rm);
        sm = warpMaxD(sm);
        if (lane == 0) {
          gate[0] = rm;
          gate[2] = sm;
        }
      }
      __syncthreads();
      parity ^= 1;
      if (k == 0) scale = (gate[2] < I.gScaleHH) ? I.gScaleHH : gate[2];
      if (I.useResidual && k >= 1) {
        lastRes = gate[0];
        used = k;
        conv = gate[0] <= I.resThreshold;
        if (conv) break;
      }
      if (k == I.maxIter) break;

      // whole correction into shared memory, then this CTA's rows of Ã⁻¹·r
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        Rs[j] = __ldcg(I.rbuf + j);
        Rs[ld + j] = __ldcg(I.rbuf + ld + j);
        Rs[2 * ld + j] = __ldcg(I.rbuf + 2 * ld + j);
      }
      __syncthreads();
      for (int li = 2 * warp; li < m; li += 2 * kWarps) {
        const bool two = li + 1 < m;
        if (li < resRows) {  // resRows is even: both rows of the pair are resident
          const float* A0 = As + static_cast<size_t>(li) * ld;
          rowPair<true>(A0, two ? A0 + ld : A0, two, Rs, ld, li, dl);
        } else {
          const float* A0 = I.Ainv + static_cast<size_t>(rb + li) * ld;
          rowPair<false>(A0, two ? A0 + ld : A0, two, Rs, ld, li, dl);
        }
      }
      __syncthreads();
      // x^{k+1} = x^k + Δ in FP64 (pinned rows: q), published as hi/lo pairs
      double dmax = 0.0;
      float* xb = I.xbuf;
      for (int t = threadIdx.x; t < 3 * m; t += blockDim.x) {
        const int li = t / 3, c = t - 3 * li, v = rb + li;
        const double xn = I.pinned[v] ? I.q[3 * v + c] : xo[t] + static_cast<double>(dl[t]);
        dmax = fmax(dmax, fabs(xn - xo[t]));
        xo[t] = xn;
        float hi, lo;
        split(xn, hi, lo);
        __stcg(xb + 8 * v + c, hi);
        __stcg(xb + 8 * v + 4 + c, lo);
      }
      dmax = warpMaxD(dmax);
      if (lane == 0) redD[warp] = dmax;
      // barrier B: new positions complete; partial maxima of the displacement
      double* slotB = I.part + 3 * (parity * team + rank);
      if (!teamBarrier(I, team, target, &flag, [&] {
            double dm = 0.0;
            for (int w = 0; w < kWarps; ++w) dm = fmax(dm, redD[w]);
            slotB[1] = dm;
          }))
        return;
      for (int j = threadIdx.x; j < 2 * n; j += blockDim.x) Xs[j] = __ldcg(xbuf4 + j);
      if (warp == 0) {
        double dm = 0.0;
        for (int r = lane; r < team; r += 32) dm = fmax(dm, __ldcg(I.part + 3 * (parity * team + r) + 1));
        dm = warpMaxD(dm);
        if (lane == 0) gate[1] = dm;
      }
      __syncthreads();
      parity ^= 1;
      if (!I.useResidual) {
        const double diff = gate[1];
        const double rel = (scale > 0.0) ? diff / scale : diff;
        const bool absHit = (I.absTol > 0.0) && (diff <= I.absTol);
        const bool relHit = (I.relTol > 0.0) && (rel <= I.relTol);
        used = k + 1;
        conv = absHit || relHit;
        if (conv) break;
      }
    }
    // velocity, damping, pin resnap (Integrator.cpp:774-791)
    for (int t = threadIdx.x; t < 3 * m; t += blockDim.x) {
      const int v = rb + t / 3;
      if (I.pinned[v]) {
        xo[t] = I.q[3 * rb + t];
        vo[t] = 0.0;
      } else {
        vo[t] = (xo[t] - xno[t]) * I.dampInvH;
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
  }
  for (int t = threadIdx.x; t < 3 * m; t += blockDim.x) {
    I.x[3 * rb + t] = xo[t];
    I.v[3 * rb + t] = vo[t];
    I.xn[3 * rb + t] = xno[t];
    I.xhat[3 * rb + t] = xho[t];
  }
}

}  // namespace

int deltaResidentCtas(int smemBytes) {
  constexpr int kMaxDynamic = 224 * 1024;  // leaves room for the kernel's static shared memory
  if (smemBytes > kMaxDynamic) return 0;
  cudaFuncSetAttribute(substepDeltaKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynamic);
  int perSm = 0, dev = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, substepDeltaKernel, kDeltaThreads, smemBytes) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return perSm * sms;
}

int launchSubstepDelta(const InstanceDev* d, int count, int team, int smemBytes, int substeps, void* stream) {
  if (count <= 0 || substeps <= 0) return 0;
  if (deltaResidentCtas(smemBytes) < count * team) return static_cast<int>(cudaErrorCooperativeLaunchTooLarge);
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
  const cudaError_t e = cudaLaunchKernelEx(&cfg, substepDeltaKernel, d, team, substeps);
  return static_cast<int>(e != cudaSuccess ? e : cudaGetLastError());
}

}  // namespace pdg
