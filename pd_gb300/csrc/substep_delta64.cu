// substep_delta64.cu — FP64 substeps of small cloths by a team of CTAs: the correction form against
// the explicit inverse of Ã, FP64-accurate, with the inverse's product on the FP32 pipes.
//
// The PD iteration x^{k+1} = L⁻¹·b(x^k) (Integrator.cpp:560-663) is computed in correction form,
//   x^{k+1} = x^k + Ã⁻¹·r,   r = b(x^k) − Ã·x^k,
// the same map in exact arithmetic, with r from one matrix-free FP64 pass over each vertex's
// incidences (the mass, edge and bend terms of Ã with pinned neighbours at q, Assembler.cpp:139-278;
// the same sums give the reference's residual t_v of x^k for the gate, Integrator.cpp:230-263).
// Positions and r are FP64 throughout. The one part that is not FP64 arithmetic is Δ = Ã⁻¹·r, the
// bulk of the work: on this part FP64 issues at 1/64 of the FP32 rate, so the product runs as
// double-float arithmetic on the FP32 pipes — Ã⁻¹ held as FP32 pairs (hi + lo = the FP64 inverse to
// ≈2⁻⁴⁸), r split into pairs the same way, each product hi·hi taken exactly (Dekker's two-product
// by FMA) and summed with Knuth's two-sum, the cross terms hi·lo + lo·hi added to the error word —
// which keeps Δ to ≈2⁻⁴⁵ of Σ|Ã⁻¹ᵢⱼ·rⱼ|. Δ is a correction, so that error is relative to |Δ|, not
// to |x|: the iterates stay within FP64 rounding of the reference's (the tests hold them to 1e-10
// after 600 substeps) at a cost close to the FP32 team kernel's.
//
// The team, the exchanges and the gate are those of substep_delta.cu (MIXED): one cloth per team of
// co-resident CTAs (cooperative launch, 512 threads each), each owning a contiguous vertex range,
// its incidences and its rows of Ã⁻¹ in shared memory. Per iteration: the correction pass of own
// vertices → exchange A (the whole r and the maximum of the residuals: a full barrier) → own rows of
// Ã⁻¹·r → update of own positions → exchange B (the positions of the CTA's window: its vertices, edge
// neighbours and bend partners). An exchange word is (epoch << 32 | 32 bits of data), written and
// polled with relaxed gpu-scope accesses; an FP64 value travels as two words (its low and high 32
// bits), each checked for the current epoch. r and the A partials alternate between two buffers.
// Every poll gives up after a bounded number of rounds, sets the instance's error flag and ends the
// CTA. Chebyshev-weighted iterates are not taken here (the planner keeps the supernodal kernel then).
#include <cstdint>

#include <algorithm>

#include "device.cuh"

namespace pdg {
namespace {

constexpr int kWarps = kDeltaThreads / 32;
constexpr int kGroup = 16;                  // lanes per vertex in the correction pass
constexpr long long kSpinLimit = 1ll << 22; // poll rounds before an exchange gives up
constexpr int kMaxTeam = 256;               // partials one polling warp covers (kMaxTeam / 32 a lane)
constexpr int kSegments = kDelta64Segments; // most column segments a row group of Ã⁻¹ is split into
constexpr int kGroupRows = 2;               // rows of Ã⁻¹ one warp applies together
constexpr int kPartStride = 16;             // words between two CTAs' partials: one L2 line each

__device__ __forceinline__ unsigned long long loadRelaxed(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void storeRelaxed(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// The two exchange words of an FP64 value: low 32 bits at p[0], high 32 bits at p[1].
__device__ __forceinline__ void publish(unsigned long long* p, unsigned tag, double v) {
  const unsigned long long t = static_cast<unsigned long long>(tag) << 32;
  storeRelaxed(p, t | static_cast<unsigned>(__double2loint(v)));
  storeRelaxed(p + 1, t | static_cast<unsigned>(__double2hiint(v)));
}

// Polls the FP64 values [b, e) of src (value j in words 2j, 2j + 1) until both words of each carry
// `tag`, and hands each to sink(j, value); thread `tid` of `nth` takes every nth value, B values in
// flight. False if a word stayed stale for kSpinLimit rounds.
template <int B, class Sink>
__device__ __forceinline__ bool pollValues(const unsigned long long* src, int b, int e, unsigned tag, int tid,
                                           int nth, Sink&& sink) {
  for (int j0 = b + tid; j0 < e; j0 += B * nth) {
    unsigned pending = 0;  // bit 2u: low word of value u, bit 2u + 1: its high word
#pragma unroll
    for (int u = 0; u < B; ++u)
      if (j0 + u * nth < e) pending |= 3u << (2 * u);
    unsigned lo[B], hi[B];
#pragma unroll
    for (int u = 0; u < B; ++u) lo[u] = hi[u] = 0u;
    long long spins = 0;
    unsigned nap = 32;  // back off while words are stale, so waiting CTAs do not flood L2
    while (pending) {
      unsigned long long w[2 * B];
#pragma unroll
      for (int u = 0; u < 2 * B; ++u) {
        const int j = j0 + (u >> 1) * nth;
        w[u] = ((pending >> u) & 1u) ? loadRelaxed(src + 2 * static_cast<size_t>(j) + (u & 1)) : 0ull;
      }
#pragma unroll
      for (int u = 0; u < 2 * B; ++u) {
        if (((pending >> u) & 1u) && static_cast<unsigned>(w[u] >> 32) == tag) {
          if (u & 1) hi[u >> 1] = static_cast<unsigned>(w[u]);
          else lo[u >> 1] = static_cast<unsigned>(w[u]);
          pending &= ~(1u << u);
        }
      }
      if (pending) {
        if (++spins > kSpinLimit) return false;
        __nanosleep(nap);
        nap = min(2 * nap, 256u);
      }
    }
#pragma unroll
    for (int u = 0; u < B; ++u)
      if (j0 + u * nth < e) sink(j0 + u * nth, __hiloint2double(static_cast<int>(hi[u]), static_cast<int>(lo[u])));
  }
  return true;
}

__device__ __forceinline__ double warpMaxD(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ double warpSumD(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Warp 0: maximum of the FP64 partials tagged `tag` of the team's ranks into *out (words 0 and 1 of
// each rank's line); other warps return true.
__device__ __forceinline__ bool pollPartials(const unsigned long long* ptag, int team, unsigned tag, double* out) {
  if (threadIdx.x >= 32) return true;
  const int lane = threadIdx.x;
  unsigned pending = 0;
#pragma unroll
  for (int i = 0; i < kMaxTeam / 32; ++i)
    if (lane + 32 * i < team) pending |= 3u << (2 * i);
  unsigned lo[kMaxTeam / 32], hi[kMaxTeam / 32];
#pragma unroll
  for (int i = 0; i < kMaxTeam / 32; ++i) lo[i] = hi[i] = 0u;
  long long spins = 0;
  unsigned nap = 32;
  bool good = true;
  while (true) {
    unsigned long long w[2 * (kMaxTeam / 32)];
#pragma unroll
    for (int u = 0; u < 2 * (kMaxTeam / 32); ++u)
      w[u] = ((pending >> u) & 1u) ? loadRelaxed(ptag + kPartStride * (lane + 32 * (u >> 1)) + (u & 1)) : 0ull;
#pragma unroll
    for (int u = 0; u < 2 * (kMaxTeam / 32); ++u) {
      if (((pending >> u) & 1u) && static_cast<unsigned>(w[u] >> 32) == tag) {
        if (u & 1) hi[u >> 1] = static_cast<unsigned>(w[u]);
        else lo[u >> 1] = static_cast<unsigned>(w[u]);
        pending &= ~(1u << u);
      }
    }
    if (__all_sync(0xffffffffu, pending == 0)) break;
    if (++spins > kSpinLimit) {
      good = false;
      break;
    }
    __nanosleep(nap);
    nap = min(2 * nap, 256u);
  }
  double mx = 0.0;
#pragma unroll
  for (int i = 0; i < kMaxTeam / 32; ++i)
    if (lane + 32 * i < team) mx = fmax(mx, __hiloint2double(static_cast<int>(hi[i]), static_cast<int>(lo[i])));
  mx = warpMaxD(mx);
  if (lane == 0) *out = mx;
  return good;
}

// FP64 value as an FP32 pair with hi + lo = v to ~2⁻⁴⁸ relative.
__device__ __forceinline__ void splitF(double v, float& hi, float& lo) {
  hi = __double2float_rn(v);
  lo = __double2float_rn(v - static_cast<double>(hi));
}

// (s, c) += (ah + al)·(rh + rl) as double-float: ah·rh = p + e exactly (FMA), s + p = t + err exactly
// (Knuth's two-sum), err + e and the cross terms ah·rl + al·rh into the error word c; al·rl (≈2⁻⁴⁸
// of the term) is dropped. The _rn intrinsics keep the compiler from contracting any of it.
__device__ __forceinline__ void dfTerm(float& s, float& c, float ah, float al, float rh, float rl) {
  const float p = __fmul_rn(ah, rh);
  const float e = __fmaf_rn(ah, rh, -p);
  const float x = __fmaf_rn(ah, rl, __fmul_rn(al, rh));
  const float t = __fadd_rn(s, p);
  const float bb = __fsub_rn(t, s);
  const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(p, bb));
  s = t;
  c = __fadd_rn(c, __fadd_rn(err, __fadd_rn(e, x)));
}

// Up to NR rows of Ã⁻¹ (hi rows from Ah0, lo rows from Al0, nr of them) times the three components
// of r (hi in Rh, lo in Rl, component-major with row length ld) over the float4 columns [jb, je),
// one warp; each r load serves NR rows. Sums (FP64) land in dl[3·(li + r) + c].
template <int NR, bool SMEM>
__device__ __forceinline__ void rowGroup(const float* Ah0, const float* Al0, int nr, const float* Rh,
                                         const float* Rl, int ld, int li, int jb, int je, double* dl) {
  const int lane = threadIdx.x & 31;
  const float4* ah4 = reinterpret_cast<const float4*>(Ah0);
  const float4* al4 = reinterpret_cast<const float4*>(Al0);
  const int ld4 = ld / 4;
  float s[NR][3], cc[NR][3];
#pragma unroll
  for (int r = 0; r < NR; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) s[r][c] = cc[r][c] = 0.f;
  for (int j = jb + lane; j < je; j += 32) {
    float4 rh[3], rl[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      rh[c] = reinterpret_cast<const float4*>(Rh + c * ld)[j];
      rl[c] = reinterpret_cast<const float4*>(Rl + c * ld)[j];
    }
#pragma unroll
    for (int r = 0; r < NR; ++r) {
      if (r < nr) {
        const float4 uh = SMEM ? ah4[r * ld4 + j] : __ldg(ah4 + r * ld4 + j);
        const float4 ul = SMEM ? al4[r * ld4 + j] : __ldg(al4 + r * ld4 + j);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          dfTerm(s[r][c], cc[r][c], uh.x, ul.x, rh[c].x, rl[c].x);
          dfTerm(s[r][c], cc[r][c], uh.y, ul.y, rh[c].y, rl[c].y);
          dfTerm(s[r][c], cc[r][c], uh.z, ul.z, rh[c].z, rl[c].z);
          dfTerm(s[r][c], cc[r][c], uh.w, ul.w, rh[c].w, rl[c].w);
        }
      }
    }
  }
#pragma unroll
  for (int r = 0; r < NR; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double v = warpSumD(static_cast<double>(s[r][c]) + static_cast<double>(cc[r][c]));
      if (lane == 0 && r < nr) dl[3 * (li + r) + c] = v;
    }
}

// Incidence sums of one vertex in FP64, accumulated by the lanes of a group and then reduced (the
// FP64 form of correction.cuh's CorrectionSums).
struct CorrectionSums64 {
  double a[3] = {0.0, 0.0, 0.0};  // mass + edge terms of t
  double f[3] = {0.0, 0.0, 0.0};  // bend terms of t
  double p[3] = {0.0, 0.0, 0.0};  // what the matrix adds to f − a by seeing pinned vertices at q

  // Edge incidences [e0, e1) (other vertex | pinned << 31, ℓ, κ) and bend incidences [s0, s1)
  // (a, b, c each | pinned << 31, (−k)·w_v); lane gl of G takes every G-th. Xw holds the window's
  // positions (vertex u at 3·(u − wlo)).
  __device__ __forceinline__ void accumulate(const InstanceDev& I, const int* eo, const double* erest,
                                             const double* ekap, int e0, int e1, const int* bv, const double* bf,
                                             int s0, int s1, const double* Xw, int wlo, const double* xv, int gl,
                                             int G) {
    for (int q = e0 + gl; q < e1; q += G) {
      const int oo = eo[q];
      const int o = oo & 0x7fffffff;
      const double* xo = Xw + 3 * (o - wlo);
      const double rx = xv[0] - xo[0], ry = xv[1] - xo[1], rz = xv[2] - xo[2];  // x_v − x_o
      const double len = sqrt(rx * rx + ry * ry + rz * rz);
      double dx = 0.0, dy = 0.0, dz = 0.0;
      if (!(len <= 1e-12)) {
        const double sc = erest[q] / len;
        dx = rx * sc;
        dy = ry * sc;
        dz = rz * sc;
      }
      const double kap = ekap[q];
      a[0] = fma(kap, rx - dx, a[0]);
      a[1] = fma(kap, ry - dy, a[1]);
      a[2] = fma(kap, rz - dz, a[2]);
      if (oo < 0) {  // pinned neighbour: the matrix sees it at q
        const double qx = __ldg(I.q + 3 * o), qy = __ldg(I.q + 3 * o + 1), qz = __ldg(I.q + 3 * o + 2);
        p[0] = fma(kap, (xv[0] - qx) - rx, p[0]);
        p[1] = fma(kap, (xv[1] - qy) - ry, p[1]);
        p[2] = fma(kap, (xv[2] - qz) - rz, p[2]);
      }
    }
    for (int q = s0 + gl; q < s1; q += G) {
      const int ma = bv[3 * q], mb = bv[3 * q + 1], mc = bv[3 * q + 2];
      const int ia = ma & 0x7fffffff, ib = mb & 0x7fffffff, ic = mc & 0x7fffffff;
      const double fac = bf[q];
      const double* xa = Xw + 3 * (ia - wlo);
      const double* xb = Xw + 3 * (ib - wlo);
      const double* xc = Xw + 3 * (ic - wlo);
      double s3[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        s3[c] = (xa[c] - xb[c]) + (xc[c] - xb[c]);
        f[c] = fma(fac, s3[c], f[c]);
      }
      if ((ma | mb | mc) < 0) {  // pinned members: the matrix part sees them at q
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const double ya = ma < 0 ? __ldg(I.q + 3 * ia + c) : xa[c];
          const double yb = mb < 0 ? __ldg(I.q + 3 * ib + c) : xb[c];
          const double yc = mc < 0 ? __ldg(I.q + 3 * ic + c) : xc[c];
          p[c] = fma(fac, s3[c] - ((ya - yb) + (yc - yb)), p[c]);
        }
      }
    }
  }
  // mass term (x − x̂)·m/h², added by one lane
  __device__ __forceinline__ void addMass(const double* xv, const double* xh, double mh2) {
#pragma unroll
    for (int c = 0; c < 3; ++c) a[c] = fma(xv[c] - xh[c], mh2, a[c]);
  }
  template <int G>
  __device__ __forceinline__ void reduce() {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) {
        a[c] += __shfl_xor_sync(0xffffffffu, a[c], o);
        f[c] += __shfl_xor_sync(0xffffffffu, f[c], o);
        p[c] += __shfl_xor_sync(0xffffffffu, p[c], o);
      }
    }
  }
  // ‖t‖ / m (Integrator.cpp:230-263)
  __device__ __forceinline__ double residual(double mass) const {
    const double t0 = a[0] + f[0], t1 = a[1] + f[1], t2 = a[2] + f[2];
    return sqrt(t0 * t0 + t1 * t1 + t2 * t2) / mass;
  }
  // r = −(mass + edge terms) + bend terms, pinned neighbours at q
  __device__ __forceinline__ void correction(double* r) const {
#pragma unroll
    for (int c = 0; c < 3; ++c) r[c] = (f[c] - a[c]) - p[c];
  }
};

template <bool TIMED>
__global__ void __launch_bounds__(kDeltaThreads, 1) substepDelta64Kernel(const InstanceDev* __restrict__ insts,
                                                                        int team, int substeps) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double red[kWarps];
  __shared__ double gate;
  __shared__ int failed;
  const int rank = static_cast<int>(blockIdx.x) % team;
  const InstanceDev& I = insts[blockIdx.x / team];
  const int n = I.n, ld = I.denseLd;
  const int chunk = (n + team - 1) / team;
  const int rb = min(n, rank * chunk), re = min(n, rb + chunk), m = re - rb;
  const int resRows = min(m, I.denseResRows);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const Delta64Carve cv(n, ld, I.denseResRows, I.teamWCap, I.teamECap, I.teamBCap, chunk);
  float* Rh = reinterpret_cast<float*>(smem + cv.rh);
  float* Rl = reinterpret_cast<float*>(smem + cv.rl);
  float* Ah = reinterpret_cast<float*>(smem + cv.ah);
  float* Al = reinterpret_cast<float*>(smem + cv.al);
  double* Xw = reinterpret_cast<double*>(smem + cv.xw);
  double* erest = reinterpret_cast<double*>(smem + cv.erest);
  double* ekap = reinterpret_cast<double*>(smem + cv.ekap);
  double* bfac = reinterpret_cast<double*>(smem + cv.bfac);
  double* mh2 = reinterpret_cast<double*>(smem + cv.mh2);
  double* mass = reinterpret_cast<double*>(smem + cv.mass);
  double* xh64 = reinterpret_cast<double*>(smem + cv.xh);
  double* xn64 = reinterpret_cast<double*>(smem + cv.xn);
  double* v64 = reinterpret_cast<double*>(smem + cv.v);
  double* dl = reinterpret_cast<double*>(smem + cv.dl);  // kSegments × 3·chunk
  int* eo = reinterpret_cast<int*>(smem + cv.eo);
  int* bv = reinterpret_cast<int*>(smem + cv.bv);
  int* pinnedOwn = reinterpret_cast<int*>(smem + cv.pin);
  int* sEb = reinterpret_cast<int*>(smem + cv.eb);
  int* sBb = reinterpret_cast<int*>(smem + cv.bb);
  const int wlo = I.window[2 * rank], whi = I.window[2 * rank + 1];

  if (threadIdx.x == 0) failed = 0;
  const int e0 = (m > 0) ? I.rstart[rb] : 0, b0 = (m > 0) ? I.bstart[rb] : 0;
  const int eN = (m > 0) ? I.rstart[re] - e0 : 0, bN = (m > 0) ? I.bstart[re] - b0 : 0;
  auto flagged = [&](int u) { return I.pinned[u] ? static_cast<int>(0x80000000u | static_cast<unsigned>(u)) : u; };
  for (int t = threadIdx.x; t < eN; t += blockDim.x) {
    const int pq = I.rinc[e0 + t], e = pq >> 1;
    const int o = I.eab[2 * e + ((pq & 1) ? 0 : 1)];  // bit 0 set: v is the edge's b, the other end a
    eo[t] = flagged(o);
    erest[t] = I.erest[e];
    ekap[t] = I.ek[e];
  }
  for (int t = threadIdx.x; t < bN; t += blockDim.x) {
    const int st = I.binc[b0 + t];
    bv[3 * t] = flagged(I.babc[3 * st]);
    bv[3 * t + 1] = flagged(I.babc[3 * st + 1]);
    bv[3 * t + 2] = flagged(I.babc[3 * st + 2]);
    bfac[t] = I.bfac[b0 + t];
  }
  for (int t = threadIdx.x; t < m; t += blockDim.x) {
    mh2[t] = I.m[rb + t] * I.invH2;
    mass[t] = I.m[rb + t];
    pinnedOwn[t] = I.pinned[rb + t];
  }
  for (int t = threadIdx.x; t <= m; t += blockDim.x) {
    sEb[t] = (m > 0) ? I.rstart[rb + t] - e0 : 0;
    sBb[t] = (m > 0) ? I.bstart[rb + t] - b0 : 0;
  }
  for (int t = threadIdx.x; t < 3 * m; t += blockDim.x) v64[t] = I.v[3 * rb + t];
  for (int t = threadIdx.x; t < 3 * (whi - wlo); t += blockDim.x) Xw[t] = I.x[3 * wlo + t];
  for (int j = n + threadIdx.x; j < ld; j += blockDim.x)
    for (int c = 0; c < 3; ++c) Rh[c * ld + j] = Rl[c * ld + j] = 0.f;
  {
    const float4* srcH = reinterpret_cast<const float4*>(I.Ainv + static_cast<size_t>(rb) * ld);
    const float4* srcL = reinterpret_cast<const float4*>(I.AinvLo + static_cast<size_t>(rb) * ld);
    float4* dstH = reinterpret_cast<float4*>(Ah);
    float4* dstL = reinterpret_cast<float4*>(Al);
    const int total = resRows * (ld / 4);
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      dstH[t] = __ldg(srcH + t);
      dstL[t] = __ldg(srcL + t);
    }
  }
  unsigned epoch = *I.epoch;  // exchanges of this launch continue the previous launch's epochs
  unsigned long long* ptagB = I.ptag + 2 * kPartStride * team;
  const int groups = (m + kGroupRows - 1) / kGroupRows;
  const int segs = groups > 0 ? max(1, min(kSegments, kWarps / groups)) : 1;
  const int q4 = ld / 4;
  const int gl = threadIdx.x & (kGroup - 1), group = threadIdx.x / kGroup, ngroups = blockDim.x / kGroup;
  __syncthreads();

  const StageClock<TIMED> clk(I, rank == 0 && threadIdx.x == 0);
  for (int step = 0; step < substeps; ++step) {
    // predict own rows (Integrator.cpp:447-472)
    double sc = 0.0;
    for (int t = threadIdx.x; t < 3 * m; t += blockDim.x) {
      const int li = t / 3, c = t - 3 * li, v = rb + li;
      const double p = Xw[3 * (v - wlo) + c];
      const double xh = (p + v64[t] * I.h) + I.gh2[c];
      xn64[t] = p;
      xh64[t] = xh;
      sc = fmax(sc, fabs(xh - p));
    }
    const double scW = warpMaxD(sc);
    __syncthreads();  // x̂ of own rows is read by other threads below
    clk.lap(I, rank == 0 && threadIdx.x == 0, kStagePredict);
    double scale = 0.0;
    int used = 0;
    bool conv = false;
    double lastRes = I.useResidual ? 0.0 : -1.0;
    for (int k = 0;; ++k) {
      const unsigned tagA = ++epoch;  // odd: epochs are consumed in (A, B) pairs
      const unsigned buf = (tagA >> 1) & 1u;
      unsigned long long* rtag = I.rtag + static_cast<size_t>(buf) * 6 * n;
      unsigned long long* ptagA = I.ptag + buf * kPartStride * team;
      // correction r and residual of x^k for own vertices, kGroup lanes per vertex (FP64)
      double resLocal = 0.0;
      for (int base = 0; base < m; base += ngroups) {
        const int li = base + group;
        const bool active = li < m;
        const bool isFree = active && pinnedOwn[li] == 0;
        const int v = rb + li;
        CorrectionSums64 cs;
        if (isFree) {
          const double* xv = Xw + 3 * (v - wlo);
          cs.accumulate(I, eo, erest, ekap, sEb[li], sEb[li + 1], bv, bfac, sBb[li], sBb[li + 1], Xw, wlo, xv, gl,
                        kGroup);
          if (gl == 0) cs.addMass(xv, xh64 + 3 * li, mh2[li]);
        }
        cs.reduce<kGroup>();
        if (active && gl == 0) {
          double r[3] = {0.0, 0.0, 0.0};
          if (isFree) {
            if (mass[li] > 0.0) resLocal = fmax(resLocal, cs.residual(mass[li]));
            cs.correction(r);
          }
          for (int c = 0; c < 3; ++c) publish(rtag + 2 * (3 * static_cast<size_t>(v) + c), tagA, r[c]);
        }
      }
      // exchange A, a full barrier of the team: the whole correction (warps 1..) and the maximum
      // of the residuals — at k = 0 of the scale — (warp 0)
      resLocal = warpMaxD(resLocal);
      if (lane == 0) red[warp] = (k == 0) ? scW : resLocal;
      __syncthreads();
      clk.lap(I, rank == 0 && threadIdx.x == 0, kStageLocal);  // the correction pass: projection, scatter and residual in one
      bool ok = true;
      if (warp == 0) {
        if (lane == 0) {
          double pm = 0.0;
          for (int w = 0; w < kWarps; ++w) pm = fmax(pm, red[w]);
          if (!(I.withholdRank == rank && step == 0 && k == 0)) publish(ptagA + kPartStride * rank, tagA, pm);
        }
        __syncwarp();
        ok = pollPartials(ptagA, team, tagA, &gate);
      } else {
        ok = pollValues<5>(rtag, 0, 3 * n, tagA, threadIdx.x - 32, blockDim.x - 32, [&](int j, double val) {
          const int v = j / 3, c = j - 3 * v;
          float hi, lo;
          splitF(val, hi, lo);
          Rh[c * ld + v] = hi;
          Rl[c * ld + v] = lo;
        });
      }
      if (!ok) failed = 1;
      __syncthreads();
      if (failed) break;
      const double gateA = gate;
      if (k == 0) scale = (gateA < I.gScaleHH) ? I.gScaleHH : gateA;
      bool stop = k == I.maxIter;
      if (I.useResidual && k >= 1) {
        lastRes = gateA;
        used = k;
        if (I.resTrace && rank == 0 && threadIdx.x == 0) I.resTrace[(size_t)step * I.maxIter + k - 1] = gateA;
        conv = gateA <= I.resThreshold;
        stop = stop || conv;
      }
      if (stop) {
        ++epoch;  // the unused B epoch: the next A epoch stays odd
        break;
      }

      // this CTA's rows of Ã⁻¹·r: groups of kGroupRows rows × column segments over the warps
      for (int task = warp; task < groups * segs; task += kWarps) {
        const int li = kGroupRows * (task / segs), sg = task - (task / segs) * segs;
        const int jb = q4 * sg / segs, je = q4 * (sg + 1) / segs;
        const int nr = min(kGroupRows, m - li);
        double* out = dl + sg * 3 * chunk;
        if (li < resRows) {  // resRows is a multiple of 4 unless it covers every row
          rowGroup<kGroupRows, true>(Ah + static_cast<size_t>(li) * ld, Al + static_cast<size_t>(li) * ld, nr, Rh,
                                     Rl, ld, li, jb, je, out);
        } else {
          rowGroup<kGroupRows, false>(I.Ainv + static_cast<size_t>(rb + li) * ld,
                                      I.AinvLo + static_cast<size_t>(rb + li) * ld, nr, Rh, Rl, ld, li, jb, je, out);
        }
      }
      __syncthreads();
      clk.lap(I, rank == 0 && threadIdx.x == 0, kStageSolve);  // exchange A and this CTA's rows of Ã⁻¹·r
      // x^{k+1} = x^k + Δ (pinned rows: q), published for the team
      const unsigned tagB = ++epoch;
      double dmax = 0.0;
      for (int t = threadIdx.x; t < 3 * m; t += blockDim.x) {
        const int li = t / 3, c = t - 3 * li, v = rb + li;
        double* xp = Xw + 3 * (v - wlo) + c;
        double x = *xp;
        if (pinnedOwn[li]) {
          const double qv = I.q[3 * v + c];
          dmax = fmax(dmax, fabs(qv - x));
          x = qv;
        } else {
          double d = dl[t];
          for (int sgi = 1; sgi < segs; ++sgi) d += dl[sgi * 3 * chunk + t];
          dmax = fmax(dmax, fabs(d));
          x += d;
        }
        *xp = x;
        publish(I.xtag + 2 * (3 * static_cast<size_t>(v) + c), tagB, x);
      }
      // exchange B: the positions this CTA reads; with the displacement gate also the maximum of
      // the displacements (warp 0), which makes it a full barrier — with the residual gate a CTA
      // waits only for the CTAs owning its window
      __syncthreads();  // own positions are read back by other threads below
      auto sinkX = [&](int j, double val) { Xw[j - 3 * wlo] = val; };
      if (!I.useResidual) {
        dmax = warpMaxD(dmax);
        if (lane == 0) red[warp] = dmax;
        __syncthreads();
        if (warp == 0) {
          if (lane == 0) {
            double pm = 0.0;
            for (int w = 0; w < kWarps; ++w) pm = fmax(pm, red[w]);
            publish(ptagB + kPartStride * rank, tagB, pm);
          }
          __syncwarp();
          ok = pollPartials(ptagB, team, tagB, &gate);
        } else {
          ok = pollValues<3>(I.xtag, 3 * wlo, 3 * whi, tagB, threadIdx.x - 32, blockDim.x - 32, sinkX);
        }
      } else {
        ok = pollValues<3>(I.xtag, 3 * wlo, 3 * whi, tagB, threadIdx.x, blockDim.x, sinkX);
      }
      if (!ok) failed = 1;
      __syncthreads();
      if (failed) break;
      clk.lap(I, rank == 0 && threadIdx.x == 0, kStageUnpack);  // the update and exchange B (the window's positions)
      if (!I.useResidual) {
        const double diff = gate;
        const double rel = (scale > 0.0) ? diff / scale : diff;
        const bool absHit = (I.absTol > 0.0) && (diff <= I.absTol);
        const bool relHit = (I.relTol > 0.0) && (rel <= I.relTol);
        used = k + 1;
        conv = absHit || relHit;
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
      v64[t] = pinnedOwn[li] ? 0.0 : (Xw[3 * (v - wlo) + c] - xn64[t]) * I.dampInvH;
    }
    if (used == 0) {  // no update ran: pinned vertices are resnapped to q over the whole window
      for (int t = threadIdx.x; t < 3 * (whi - wlo); t += blockDim.x) {
        const int u = wlo + t / 3;
        if (I.pinned[u]) Xw[t] = I.q[3 * wlo + t];
      }
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
    I.x[3 * rb + t] = pinnedOwn[li] ? I.q[3 * v + c] : Xw[3 * (v - wlo) + c];
    I.v[3 * rb + t] = v64[t];
    I.xn[3 * rb + t] = xn64[t];
  }
}

}  // namespace

int delta64ResidentCtas(int smemBytes) {
  constexpr int kMaxDynamic = 224 * 1024;  // leaves room for the kernel's static shared memory
  if (smemBytes > kMaxDynamic) return 0;
  int least = 1 << 30;
  for (auto kernel : {substepDelta64Kernel<false>, substepDelta64Kernel<true>}) {  // both must fit
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

int launchSubstepDelta64(const InstanceDev* d, int count, int team, int smemBytes, int substeps, void* stream,
                         bool timed) {
  if (count <= 0 || substeps <= 0) return 0;
  if (team > kMaxTeam || delta64ResidentCtas(smemBytes) < count * team)
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
  const cudaError_t e = timed ? cudaLaunchKernelEx(&cfg, substepDelta64Kernel<true>, d, team, substeps)
                              : cudaLaunchKernelEx(&cfg, substepDelta64Kernel<false>, d, team, substeps);
  return static_cast<int>(e != cudaSuccess ? e : cudaGetLastError());
}

}  // namespace pdg
