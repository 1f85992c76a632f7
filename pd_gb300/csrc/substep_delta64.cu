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
// neighbours and bend partners). An exchange word carries the epoch it was written in and its data,
// written and polled with relaxed gpu-scope accesses: a position or a partial maximum travels as two
// words (epoch << 32 | low or high 32 bits of the FP64), an r value as one packed word (packR). r and
// the A partials alternate between two buffers. Polls do not sleep between rounds (a store is
// visible to another SM ~250 ns later on the same die, ~370 ns on the other; each round waits for its
// own loads). Every poll gives up after a bounded number of rounds, sets the instance's error flag and
// ends the CTA. Chebyshev-weighted iterates are not taken here (the planner keeps the supernodal kernel then).
// The same kernel serves PD_PRECISION_FP32_PROJECTION on small cloths: the projection d_e in FP32,
// the correction, the solve and the residual as above.
#include <cstdint>

#include <algorithm>

#include "device.cuh"

namespace pdg {
namespace {

constexpr int kWarps = kDeltaThreads / 32;
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

// Polls the values [b, e) of src (value j in words 2j, 2j + 1) until both words of each carry `tag`,
// and hands each to sink(j, low 32 bits of word 2j, of word 2j + 1); thread `tid` of `nth` takes every
// nth value, B values in flight. False if a word stayed stale for kSpinLimit rounds.
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
      if (pending && ++spins > kSpinLimit) return false;
    }
#pragma unroll
    for (int u = 0; u < B; ++u)
      if (j0 + u * nth < e) sink(j0 + u * nth, lo[u], hi[u]);
  }
  return true;
}

// Non-negative doubles order like their bit patterns read as signed 64-bit integers, so their maxima
// are taken with integer operations: on this part an FP64 warp instruction occupies its sub-core's
// FP64 pipe for ~80 cycles whatever its active lanes, and these reductions would otherwise be a
// large share of an iteration. A NaN counts as 0 (it is skipped, as the reference's `>` skips it).
// r travels as one word: an 8-bit epoch tag, the FP32 hi part and the top 24 bits of the FP32 lo
// part rounded to nearest (sign, exponent, 15 mantissa bits): hi + lo keeps r to ~2⁻³⁹ relative, and
// Δ = Ã⁻¹·r, a correction, to far below the FP64 rounding of the positions. A word is rewritten every
// fourth epoch, so its tag is never more than 4 behind the current one and 8 bits tell them apart.
__device__ __forceinline__ unsigned long long packR(unsigned tag, float hi, float lo) {
  const unsigned lo24 = (__float_as_uint(lo) + 0x80u) >> 8;
  return (static_cast<unsigned long long>(tag & 0xffu) << 56) |
         (static_cast<unsigned long long>(__float_as_uint(hi)) << 24) | lo24;
}

// Polls the packed words [b, e) of src until each carries the current 8-bit tag and hands
// sink(j, hi, lo) the pair; B words in flight per thread. False after kSpinLimit stale rounds.
template <int B, class Sink>
__device__ __forceinline__ bool pollPacked(const unsigned long long* src, int b, int e, unsigned tag, int tid,
                                           int nth, Sink&& sink) {
  const unsigned t8 = tag & 0xffu;
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
        if (((pending >> u) & 1u) && static_cast<unsigned>(w[u] >> 56) == t8) {
          sink(j0 + u * nth, __uint_as_float(static_cast<unsigned>(w[u] >> 24)),
               __uint_as_float(static_cast<unsigned>(w[u] & 0xffffffull) << 8));
          pending &= ~(1u << u);
        }
      }
      if (pending && ++spins > kSpinLimit) return false;
    }
  }
  return true;
}

__device__ __forceinline__ long long maxKey(double v) {
  const long long b = __double_as_longlong(v);
  return (b & 0x7fffffffffffffffll) > 0x7ff0000000000000ll ? 0ll : b;
}

__device__ __forceinline__ double warpMaxNonNeg(double v) {
  long long b = maxKey(v);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
  return __longlong_as_double(b);
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
  }
  long long mx = 0;
#pragma unroll
  for (int i = 0; i < kMaxTeam / 32; ++i)
    if (lane + 32 * i < team)
      mx = max(mx, maxKey(__hiloint2double(static_cast<int>(hi[i]), static_cast<int>(lo[i]))));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) *out = __longlong_as_double(mx);
  return good;
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

// (s, c) + (s2, c2) for double-float pairs: the two-sum of s and s2, the rest into c.
__device__ __forceinline__ void dfAdd(float& s, float& c, float s2, float c2) {
  const float t = __fadd_rn(s, s2);
  const float bb = __fsub_rn(t, s);
  const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(s2, bb));
  s = t;
  c = __fadd_rn(c, __fadd_rn(c2, err));
}

// Up to NR rows of Ã⁻¹ (hi rows from Ah0, lo rows from Al0, nr of them) times the three components
// of r (hi in Rh, lo in Rl, component-major with row length ld) over the float4 columns [jb, je),
// one warp; each r load serves NR rows. The lanes' double-float sums are reduced over the warp in
// FP32 and land as a pair, dh[3·(li + r) + c] + dlo[3·(li + r) + c].
template <int NR, bool SMEM>
__device__ __forceinline__ void rowGroup(const float* Ah0, const float* Al0, int nr, const float* Rh,
                                         const float* Rl, int ld, int li, int jb, int je, float* dh, float* dlo) {
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
      float hs = s[r][c], hc = cc[r][c];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
        dfAdd(hs, hc, __shfl_xor_sync(0xffffffffu, hs, o), __shfl_xor_sync(0xffffffffu, hc, o));
      if (lane == 0 && r < nr) {
        dh[3 * (li + r) + c] = hs;
        dlo[3 * (li + r) + c] = hc;
      }
    }
}

// ℓ/‖rel‖ for dot = rel·rel > 0: the FP32 reciprocal square root refined by two Newton steps in FP64
// (2⁻²² → 2⁻⁴⁴ → FP64 rounding), fewer FP64 instructions than a square root and a division.
__device__ __forceinline__ double restOverLength(double dot, double rest) {
  double y = static_cast<double>(rsqrtf(static_cast<float>(dot)));
  const double nh = -0.5 * dot;
  y = y * fma(nh * y, y, 1.5);
  y = y * fma(nh * y, y, 1.5);
  return rest * y;
}

// The terms of one edge incidence of own vertex v (other vertex o, FP64): κ·((x_v − x_o) − d_e) into
// t[0..2] and, when o is pinned, what the matrix adds by seeing o at q, κ·((x_v − q_o) − (x_v − x_o)),
// into t[3..5] (zeros otherwise). d_e = ℓ·rel/‖rel‖, zero when ‖rel‖ ≤ 1e-12 (DistanceTerm.cpp:94-102).
// With I.proj32 (PD_PRECISION_FP32_PROJECTION) d_e itself is FP32, from the FP64 difference, as in
// the supernodal kernels' projectEdge; everything else stays FP64.
__device__ __forceinline__ void edgeIncidence(const InstanceDev& I, const double* xv, const double* xo, int oo,
                                              double rest, double kap, double* t) {
  const double rx = xv[0] - xo[0], ry = xv[1] - xo[1], rz = xv[2] - xo[2];
  if (I.proj32) {
    const float fx = static_cast<float>(rx), fy = static_cast<float>(ry), fz = static_cast<float>(rz);
    const float len = sqrtf(fx * fx + fy * fy + fz * fz);
    float dx = 0.f, dy = 0.f, dz = 0.f;
    if (!(len <= 1e-12f)) {
      const float s = static_cast<float>(rest) / len;
      dx = fx * s;
      dy = fy * s;
      dz = fz * s;
    }
    t[0] = kap * (rx - static_cast<double>(dx));
    t[1] = kap * (ry - static_cast<double>(dy));
    t[2] = kap * (rz - static_cast<double>(dz));
  } else {
    const double dot = fma(rx, rx, fma(ry, ry, rz * rz));
    double sc = 0.0;
    if (!(dot <= 1e-24)) sc = restOverLength(dot, rest);
    t[0] = kap * (rx - rx * sc);
    t[1] = kap * (ry - ry * sc);
    t[2] = kap * (rz - rz * sc);
  }
  if (oo < 0) {
    const int o = oo & 0x7fffffff;
    t[3] = kap * ((xv[0] - __ldg(I.q + 3 * o)) - rx);
    t[4] = kap * ((xv[1] - __ldg(I.q + 3 * o + 1)) - ry);
    t[5] = kap * ((xv[2] - __ldg(I.q + 3 * o + 2)) - rz);
  } else {
    t[3] = t[4] = t[5] = 0.0;
  }
}

// The terms of one bend incidence (members a, b, c with pinned flags, fac = (−k)·w_v): fac·(w·x)
// into t[0..2] and, with pinned members, fac·(w·x − w·x̃) with x̃ = q on pinned members into t[3..5].
__device__ __forceinline__ void bendIncidence(const InstanceDev& I, const double* Xw, int wlo, const int* mb,
                                              double fac, double* t) {
  const int ia = mb[0] & 0x7fffffff, ib = mb[1] & 0x7fffffff, ic = mb[2] & 0x7fffffff;
  const double* xa = Xw + 3 * (ia - wlo);
  const double* xb = Xw + 3 * (ib - wlo);
  const double* xc = Xw + 3 * (ic - wlo);
  const bool pinnedAny = (mb[0] | mb[1] | mb[2]) < 0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double s3 = (xa[c] - xb[c]) + (xc[c] - xb[c]);
    t[c] = fac * s3;
    double pc = 0.0;
    if (pinnedAny) {
      const double ya = mb[0] < 0 ? __ldg(I.q + 3 * ia + c) : xa[c];
      const double yb = mb[1] < 0 ? __ldg(I.q + 3 * ib + c) : xb[c];
      const double yc = mb[2] < 0 ? __ldg(I.q + 3 * ic + c) : xc[c];
      pc = fac * (s3 - ((ya - yb) + (yc - yb)));
    }
    t[3 + c] = pc;
  }
}

template <bool TIMED>
__global__ void __launch_bounds__(kDeltaThreads, 1) substepDelta64Kernel(const InstanceDev* __restrict__ insts,
                                                                        int team, int substeps) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double red[kWarps];
  __shared__ double gate;
  __shared__ int gateHit;  // the gate's decision, taken once by thread 0 and read by every thread
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
  float* dh = reinterpret_cast<float*>(smem + cv.dl);  // kSegments × 3·chunk: Δ per segment, hi
  float* dlo = dh + kSegments * 3 * chunk;              // and lo
  double* econ = reinterpret_cast<double*>(smem + cv.econ);  // 6 per edge incidence
  double* bcon = reinterpret_cast<double*>(smem + cv.bcon);  // 6 per bend incidence
  double* tres = reinterpret_cast<double*>(smem + cv.tres);  // t of own vertices (3 per vertex)
  int* eOwn = reinterpret_cast<int*>(smem + cv.eown);        // own vertex (local index) of each incidence
  int* bOwn = reinterpret_cast<int*>(smem + cv.bown);
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
  for (int li = threadIdx.x; li < m; li += blockDim.x) {
    for (int q = I.rstart[rb + li] - e0; q < I.rstart[rb + li + 1] - e0; ++q) eOwn[q] = li;
    for (int q = I.bstart[rb + li] - b0; q < I.bstart[rb + li + 1] - b0; ++q) bOwn[q] = li;
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
  const int ePad = (eN + 31) & ~31;  // edge incidences in the first warps, bend incidences after them
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
    const double scW = warpMaxNonNeg(sc);
    __syncthreads();  // x̂ of own rows is read by other threads below
    clk.lap(I, rank == 0 && threadIdx.x == 0, kStagePredict);
    double scale = 0.0;
    int used = 0;
    bool conv = false;
    double lastRes = I.useResidual ? 0.0 : -1.0;
    for (int k = 0;; ++k) {
      const unsigned tagA = ++epoch;  // odd: epochs are consumed in (A, B) pairs
      const unsigned buf = (tagA >> 1) & 1u;
      unsigned long long* rtag = I.rtag + static_cast<size_t>(buf) * 3 * n;
      unsigned long long* ptagA = I.ptag + buf * kPartStride * team;
      // correction r and residual of x^k for own vertices (FP64; Integrator.cpp:230-263 for the
      // residual): one lane per incidence computes its terms, then three lanes per vertex sum them in
      // incidence order, then one lane per vertex takes the residual's norm. r is published as FP32
      // hi/lo words, the pair the product needs.
      for (int t = threadIdx.x; t < ePad + bN; t += blockDim.x) {
        if (t < eN) {
          const int li = eOwn[t];
          const double* xv = Xw + 3 * (rb + li - wlo);
          const double* xo = Xw + 3 * ((eo[t] & 0x7fffffff) - wlo);
          edgeIncidence(I, xv, xo, eo[t], erest[t], ekap[t], econ + 6 * t);
        } else if (t >= ePad) {
          const int q = t - ePad;
          bendIncidence(I, Xw, wlo, bv + 3 * q, bfac[q], bcon + 6 * q);
        }
      }
      __syncthreads();
      for (int t = threadIdx.x; t < 3 * m; t += blockDim.x) {
        const int li = t / 3, c = t - 3 * li, v = rb + li;
        double r = 0.0, tv = 0.0;
        if (!pinnedOwn[li]) {
          double a = 0.0, f = 0.0, pc = 0.0;
          for (int q = sEb[li]; q < sEb[li + 1]; ++q) {
            a += econ[6 * q + c];
            pc += econ[6 * q + 3 + c];
          }
          for (int q = sBb[li]; q < sBb[li + 1]; ++q) {
            f += bcon[6 * q + c];
            pc += bcon[6 * q + 3 + c];
          }
          a = fma(Xw[3 * (v - wlo) + c] - xh64[t], mh2[li], a);  // mass term (x − x̂)·m/h²
          tv = a + f;
          r = (f - a) - pc;
        }
        tres[t] = tv;
        const float hi = __double2float_rn(r);
        const float lo = __double2float_rn(r - static_cast<double>(hi));
        storeRelaxed(rtag + 3 * static_cast<size_t>(v) + c, packR(tagA, hi, lo));
      }
      __syncthreads();
      double resLocal = 0.0;
      for (int li = threadIdx.x; li < m; li += blockDim.x) {
        if (pinnedOwn[li] || !(mass[li] > 0.0)) continue;
        const double t0 = tres[3 * li], t1 = tres[3 * li + 1], t2 = tres[3 * li + 2];
        resLocal = fmax(resLocal, sqrt(fma(t0, t0, fma(t1, t1, t2 * t2))) / mass[li]);
      }
      // exchange A, a full barrier of the team: the whole correction (warps 1..) and the maximum
      // of the residuals — at k = 0 of the scale — (warp 0)
      resLocal = warpMaxNonNeg(resLocal);
      if (lane == 0) red[warp] = (k == 0) ? scW : resLocal;
      __syncthreads();
      clk.lap(I, rank == 0 && threadIdx.x == 0, kStageLocal);  // the correction pass: projection, scatter and residual in one
      bool ok = true;
      if (warp == 0) {
        if (lane == 0) {
          long long pm = 0;
          for (int w = 0; w < kWarps; ++w) pm = max(pm, maxKey(red[w]));
          if (!(I.withholdRank == rank && step == 0 && k == 0))
            publish(ptagA + kPartStride * rank, tagA, __longlong_as_double(pm));
        }
        __syncwarp();
        ok = pollPartials(ptagA, team, tagA, &gate);
        if (lane == 0) gateHit = (k >= 1 && gate <= I.resThreshold) ? 1 : 0;  // one FP64 compare, not one a warp
      } else {
        ok = pollPacked<10>(rtag, 0, 3 * n, tagA, threadIdx.x - 32, blockDim.x - 32,
                            [&](int j, float hi, float lo) {  // r as its FP32 pair
                              const int v = j / 3, c = j - 3 * v;
                              Rh[c * ld + v] = hi;
                              Rl[c * ld + v] = lo;
                            });
      }
      if (!ok) failed = 1;
      __syncthreads();
      if (failed) break;
      if (k == 0) scale = (gate < I.gScaleHH) ? I.gScaleHH : gate;
      bool stop = k == I.maxIter;
      if (I.useResidual && k >= 1) {
        used = k;
        if (threadIdx.x == 0) {  // the only thread that reports them
          lastRes = gate;
          if (I.resTrace && rank == 0) I.resTrace[(size_t)step * I.maxIter + k - 1] = gate;
        }
        conv = gateHit != 0;
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
        float* oh = dh + sg * 3 * chunk;
        float* ol = dlo + sg * 3 * chunk;
        if (li < resRows) {  // resRows is a multiple of 4 unless it covers every row
          rowGroup<kGroupRows, true>(Ah + static_cast<size_t>(li) * ld, Al + static_cast<size_t>(li) * ld, nr, Rh,
                                     Rl, ld, li, jb, je, oh, ol);
        } else {
          rowGroup<kGroupRows, false>(I.Ainv + static_cast<size_t>(rb + li) * ld,
                                      I.AinvLo + static_cast<size_t>(rb + li) * ld, nr, Rh, Rl, ld, li, jb, je, oh,
                                      ol);
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
          float hs = dh[t], hc = dlo[t];  // the segments' pairs summed in FP32, then one FP64 sum
          for (int sgi = 1; sgi < segs; ++sgi) dfAdd(hs, hc, dh[sgi * 3 * chunk + t], dlo[sgi * 3 * chunk + t]);
          const double d = static_cast<double>(hs) + static_cast<double>(hc);
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
      auto sinkX = [&](int j, unsigned wl, unsigned wh) {  // a position: low and high words of the FP64
        Xw[j - 3 * wlo] = __hiloint2double(static_cast<int>(wh), static_cast<int>(wl));
      };
      if (!I.useResidual) {
        dmax = warpMaxNonNeg(dmax);
        if (lane == 0) red[warp] = dmax;
        __syncthreads();
        if (warp == 0) {
          if (lane == 0) {
            long long pm = 0;
            for (int w = 0; w < kWarps; ++w) pm = max(pm, maxKey(red[w]));
            publish(ptagB + kPartStride * rank, tagB, __longlong_as_double(pm));
          }
          __syncwarp();
          ok = pollPartials(ptagB, team, tagB, &gate);
          if (lane == 0) {  // the displacement gate's decision, once
            const double diff = gate;
            const double rel = (scale > 0.0) ? diff / scale : diff;
            gateHit = ((I.absTol > 0.0) && (diff <= I.absTol)) || ((I.relTol > 0.0) && (rel <= I.relTol)) ? 1 : 0;
          }
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
