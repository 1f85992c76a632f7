// substep_team.cuh — the substep run by a "team": one CTA, or a thread-block cluster of CTAs
// working on one cloth.
//
// A single small cloth cannot fill a GB300 and one SM's FP64 pipe (≈1.6 ops/clk) caps a one-CTA
// substep, so a cluster of up to 16 CTAs shares one cloth: every vertex / edge / row loop is
// strided over all threads of the cluster, phases are separated by cluster barriers (release /
// acquire at cluster scope, ≈0.26 µs), reductions go through distributed shared memory, and the
// cloth's working arrays live in L2 (loads that may see other CTAs' writes bypass L1 with
// ld.global.cg). With one CTA the same code uses __syncthreads and ordinary loads.
#pragma once

#include <cooperative_groups.h>

#include "substep_common.cuh"

namespace pdg {

template <bool CLUSTER>
struct Team {
  int rank;  // CTA rank in the cluster
  int size;  // CTAs in the cluster
  // A grid team (one cloth on a cooperative launch of many CTAs, CLUSTER = true): 2 × size doubles
  // of global memory for the team maximum; null for a cluster. Barriers are then grid barriers.
  double* gslots = nullptr;
  __device__ __forceinline__ int tid() const { return rank * (int)blockDim.x + (int)threadIdx.x; }
  __device__ __forceinline__ int count() const { return size * (int)blockDim.x; }
  __device__ __forceinline__ void sync() const {
    if (CLUSTER) {
      if (gslots) cooperative_groups::this_grid().sync();
      else cooperative_groups::this_cluster().sync();
    } else {
      __syncthreads();
    }
  }
  // loads of data another CTA of the cluster may have written since the last barrier
  template <class T>
  __device__ __forceinline__ T ld(const T* p) const {
    if (CLUSTER) return __ldcg(p);
    return *p;
  }
};

// Max over the team of non-negative values (NaN-skipping). `slots` is a 2-entry shared array
// whose alternating use keeps a reduction's writes from racing with remote reads of the last one.
template <bool CLUSTER>
__device__ __forceinline__ double teamMax(const Team<CLUSTER>& tm, double v, double* red, double* slots, int& parity) {
  v = blockMax(v, red);
  if (!CLUSTER) return v;
  if (tm.gslots) {  // grid team: one slot per CTA in global memory, two buffers by parity
    double* g = tm.gslots + parity * tm.size;
    parity ^= 1;
    if (threadIdx.x == 0) g[tm.rank] = v;
    cooperative_groups::this_grid().sync();
    double m = 0.0;
    for (int r = threadIdx.x; r < tm.size; r += blockDim.x) m = fmax(m, __ldcg(g + r));
    return blockMax(m, red);
  }
  double* slot = slots + parity;
  parity ^= 1;
  if (threadIdx.x == 0) *slot = v;
  cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
  cl.sync();
  double m = 0.0;
  for (int r = 0; r < tm.size; ++r) m = fmax(m, *cl.map_shared_rank(slot, r));
  return m;
}

// d_e = ℓ·rel/‖rel‖ (0 when degenerate), in FP64 or — with proj32 — in FP32 from the FP64
// difference (the projection is where FP32 is safe: it only normalises a short vector).
__device__ __forceinline__ void projectEdge(const InstanceDev& I, int e, double rx, double ry, double rz, double& dx,
                                            double& dy, double& dz) {
  if (I.proj32) {
    const float fx = static_cast<float>(rx), fy = static_cast<float>(ry), fz = static_cast<float>(rz);
    const float len = sqrtf(fx * fx + fy * fy + fz * fz);
    if (!(len <= 1e-12f)) {
      const float s = static_cast<float>(I.erest[e]) / len;
      dx = fx * s;
      dy = fy * s;
      dz = fz * s;
    }
    return;
  }
  const double len = sqrt(rx * rx + ry * ry + rz * rz);
  if (!(len <= 1e-12)) {
    const double s = I.erest[e] / len;
    dx = rx * s;
    dy = ry * s;
    dz = rz * s;
  }
}

// Edge e at positions X (I.x, or I.xsol for the residual of an over-relaxed iteration): κ·d_e and
// κ·rel − κ·d_e (DistanceTerm.cpp:94-152, Integrator.cpp:246-248).
template <bool CLUSTER>
__device__ __forceinline__ void edgeTerms(const InstanceDev& I, const Team<CLUSTER>& tm, const double* X, int e,
                                          bool wantRc) {
  const int a = I.eab[2 * e], b = I.eab[2 * e + 1];
  const double rx = tm.ld(X + 3 * a) - tm.ld(X + 3 * b);
  const double ry = tm.ld(X + 3 * a + 1) - tm.ld(X + 3 * b + 1);
  const double rz = tm.ld(X + 3 * a + 2) - tm.ld(X + 3 * b + 2);
  double dx = 0.0, dy = 0.0, dz = 0.0;
  projectEdge(I, e, rx, ry, rz, dx, dy, dz);
  const double k = I.ek[e];
  const double cx = dx * k, cy = dy * k, cz = dz * k;
  I.kd[3 * e] = cx;
  I.kd[3 * e + 1] = cy;
  I.kd[3 * e + 2] = cz;
  if (wantRc) {
    I.rc[3 * e] = fma(rx, k, -cx);
    I.rc[3 * e + 1] = fma(ry, k, -cy);
    I.rc[3 * e + 2] = fma(rz, k, -cz);
  }
}

// b_v in colour order with pin elimination, pinned rows = q, stored at v's elimination position.
template <bool CLUSTER>
__device__ __forceinline__ void gatherRow(const InstanceDev& I, const Team<CLUSTER>& tm, int v, double* w) {
  double b0, b1, b2;
  if (I.pinned[v]) {
    b0 = I.q[3 * v];
    b1 = I.q[3 * v + 1];
    b2 = I.q[3 * v + 2];
  } else {
    b0 = tm.ld(I.bbase + 3 * v);
    b1 = tm.ld(I.bbase + 3 * v + 1);
    b2 = tm.ld(I.bbase + 3 * v + 2);
    if (I.hasBendRhs) {
      b0 += I.bendRhs[3 * v];
      b1 += I.bendRhs[3 * v + 1];
      b2 += I.bendRhs[3 * v + 2];
    }
    for (int k = I.sstart[v]; k < I.sstart[v + 1]; ++k) {
      const int p = I.sinc[k];
      const int e = p >> 1;
      const double sgn = (p & 1) ? -1.0 : 1.0;
      b0 = fma(sgn, tm.ld(I.kd + 3 * e), b0);
      b1 = fma(sgn, tm.ld(I.kd + 3 * e + 1), b1);
      b2 = fma(sgn, tm.ld(I.kd + 3 * e + 2), b2);
      const int other = I.eab[2 * e + ((p & 1) ^ 1)];
      if (I.pinned[other]) {
        const double k = I.ek[e];
        b0 = fma(k, I.q[3 * other], b0);
        b1 = fma(k, I.q[3 * other + 1], b1);
        b2 = fma(k, I.q[3 * other + 2], b2);
      }
    }
  }
  const int r = I.iperm[v];
  w[3 * r] = b0;
  w[3 * r + 1] = b1;
  w[3 * r + 2] = b2;
}

// Nonlinear residual of vertex v at positions X (Integrator.cpp:230-263).
template <bool CLUSTER>
__device__ __forceinline__ double residualAt(const InstanceDev& I, const Team<CLUSTER>& tm, const double* X, int v) {
  double f0 = 0.0, f1 = 0.0, f2 = 0.0;
  for (int k = I.rstart[v]; k < I.rstart[v + 1]; ++k) {
    const int p = I.rinc[k];
    const int e = p >> 1;
    const double sgn = (p & 1) ? -1.0 : 1.0;
    f0 = fma(sgn, tm.ld(I.rc + 3 * e), f0);
    f1 = fma(sgn, tm.ld(I.rc + 3 * e + 1), f1);
    f2 = fma(sgn, tm.ld(I.rc + 3 * e + 2), f2);
  }
  for (int k = I.bstart[v]; k < I.bstart[v + 1]; ++k) {
    const int s = I.binc[k];
    const int a = I.babc[3 * s], b = I.babc[3 * s + 1], c = I.babc[3 * s + 2];
    const double fac = I.bfac[k];
    f0 = fma(tm.ld(X + 3 * a) - 2.0 * tm.ld(X + 3 * b) + tm.ld(X + 3 * c), fac, f0);
    f1 = fma(tm.ld(X + 3 * a + 1) - 2.0 * tm.ld(X + 3 * b + 1) + tm.ld(X + 3 * c + 1), fac, f1);
    f2 = fma(tm.ld(X + 3 * a + 2) - 2.0 * tm.ld(X + 3 * b + 2) + tm.ld(X + 3 * c + 2), fac, f2);
  }
  const double mass = I.m[v];
  const double mh2 = mass * I.invH2;
  const double t0 = fma(tm.ld(X + 3 * v) - tm.ld(I.xhat + 3 * v), mh2, f0);
  const double t1 = fma(tm.ld(X + 3 * v + 1) - tm.ld(I.xhat + 3 * v + 1), mh2, f1);
  const double t2 = fma(tm.ld(X + 3 * v + 2) - tm.ld(I.xhat + 3 * v + 2), mh2, f2);
  return sqrt(t0 * t0 + t1 * t1 + t2 * t2) / mass;
}

template <int G>
__device__ __forceinline__ double groupSum(double v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, G);
  return v;
}

// Supernodal solve over the nested-dissection tree (see substep_fast.cu): per level, an
// off-block gather then a dense-inverse mat-vec, both as G-lane group reductions, in forward
// and then backward order. G is chosen per level from the rows' lengths (gF / gB tables).
template <bool CLUSTER>
struct TeamSolve {
  template <int G, class Body>
  static __device__ __forceinline__ void rows(const Team<CLUSTER>& tm, int cnt, Body&& body) {
    const int lane = threadIdx.x & (G - 1);
    const int groups = (int)blockDim.x / G;
    const int gid = tm.rank * groups + (int)threadIdx.x / G;
    const int stride = tm.size * groups;
    for (int base = 0; base < cnt; base += stride) {  // uniform trip count keeps shuffles converged
      const int idx = base + gid;
      double a0 = 0.0, a1 = 0.0, a2 = 0.0;
      body.accumulate(idx, lane, G, a0, a1, a2);
      if (G > 1) {
        a0 = groupSum<G>(a0);
        a1 = groupSum<G>(a1);
        a2 = groupSum<G>(a2);
      }
      if (lane == 0) body.finish(idx, a0, a1, a2);
    }
  }
  template <class Body>
  static __device__ __forceinline__ void dispatch(const Team<CLUSTER>& tm, int g, int cnt, Body&& body) {
    switch (g) {
      case 1: rows<1>(tm, cnt, body); break;
      case 2: rows<2>(tm, cnt, body); break;
      case 4: rows<4>(tm, cnt, body); break;
      case 8: rows<8>(tm, cnt, body); break;
      case 16: rows<16>(tm, cnt, body); break;
      default: rows<32>(tm, cnt, body); break;
    }
  }

  struct FwdGather {  // t_i = w_i − Σ_{j < s0} L_ij·y_j
    const InstanceDev& I; const Team<CLUSTER>& tm; const double* w; double* t; int beg, cnt;
    __device__ void accumulate(int idx, int lane, int G, double& a0, double& a1, double& a2) const {
      if (idx >= cnt) return;
      const int i = I.lvlRows[beg + idx];
#pragma unroll 4
      for (int p = I.Lrp[i] + lane; p < I.offEnd[i]; p += G) {
        const int j = I.Lci[p];
        const double lv = I.Lrv[p];
        a0 = fma(lv, tm.ld(w + 3 * j), a0);
        a1 = fma(lv, tm.ld(w + 3 * j + 1), a1);
        a2 = fma(lv, tm.ld(w + 3 * j + 2), a2);
      }
    }
    __device__ void finish(int idx, double a0, double a1, double a2) const {
      if (idx >= cnt) return;
      const int i = I.lvlRows[beg + idx];
      t[3 * i] = tm.ld(w + 3 * i) - a0;
      t[3 * i + 1] = tm.ld(w + 3 * i + 1) - a1;
      t[3 * i + 2] = tm.ld(w + 3 * i + 2) - a2;
    }
  };
  struct FwdDense {  // y_i = Σ_{c ≤ r} (L_SS⁻¹)_{rc}·t_{s0+c}
    const InstanceDev& I; const Team<CLUSTER>& tm; double* w; const double* t; int beg, cnt;
    __device__ void accumulate(int idx, int lane, int G, double& a0, double& a1, double& a2) const {
      if (idx >= cnt) return;
      const int i = I.lvlRows[beg + idx];
      const int s = I.rowSn[i];
      const int s0 = I.snStart[s];
      const int r = i - s0;
      const double* X = I.invL + I.snInvOff[s] + (int64_t)r * (r + 1) / 2;
#pragma unroll 4
      for (int c = lane; c <= r; c += G) {
        const double xv = X[c];
        const int j = s0 + c;
        a0 = fma(xv, tm.ld(t + 3 * j), a0);
        a1 = fma(xv, tm.ld(t + 3 * j + 1), a1);
        a2 = fma(xv, tm.ld(t + 3 * j + 2), a2);
      }
    }
    __device__ void finish(int idx, double a0, double a1, double a2) const {
      if (idx >= cnt) return;
      const int i = I.lvlRows[beg + idx];
      w[3 * i] = a0;
      w[3 * i + 1] = a1;
      w[3 * i + 2] = a2;
    }
  };
  struct BwdGather {  // t_k = D⁻¹_k·y_k − Σ_{i ≥ s1} L_ik·x_i
    const InstanceDev& I; const Team<CLUSTER>& tm; const double* w; double* t; int beg, cnt;
    __device__ void accumulate(int idx, int lane, int G, double& a0, double& a1, double& a2) const {
      if (idx >= cnt) return;
      const int k = I.lvlRows[beg + idx];
#pragma unroll 4
      for (int p = I.offBeg[k] + lane; p < I.Lcp[k + 1]; p += G) {
        const int i = I.Lri[p];
        const double lv = I.Lcv[p];
        a0 = fma(lv, tm.ld(w + 3 * i), a0);
        a1 = fma(lv, tm.ld(w + 3 * i + 1), a1);
        a2 = fma(lv, tm.ld(w + 3 * i + 2), a2);
      }
    }
    __device__ void finish(int idx, double a0, double a1, double a2) const {
      if (idx >= cnt) return;
      const int k = I.lvlRows[beg + idx];
      const double di = I.dinv[k];
      t[3 * k] = fma(tm.ld(w + 3 * k), di, -a0);
      t[3 * k + 1] = fma(tm.ld(w + 3 * k + 1), di, -a1);
      t[3 * k + 2] = fma(tm.ld(w + 3 * k + 2), di, -a2);
    }
  };
  struct BwdDense {  // x_k = Σ_{c ≥ r} (L_SS⁻¹)_{cr}·t_{s0+c}
    const InstanceDev& I; const Team<CLUSTER>& tm; double* w; const double* t; int beg, cnt;
    __device__ void accumulate(int idx, int lane, int G, double& a0, double& a1, double& a2) const {
      if (idx >= cnt) return;
      const int k = I.lvlRows[beg + idx];
      const int s = I.rowSn[k];
      const int s0 = I.snStart[s];
      const int sz = I.snStart[s + 1] - s0;
      const int r = k - s0;
      const double* XT = I.invLT + I.snInvOff[s] + (int64_t)r * sz - (int64_t)r * (r - 1) / 2;
#pragma unroll 4
      for (int c = lane; c < sz - r; c += G) {
        const double xv = XT[c];
        const int j = k + c;
        a0 = fma(xv, tm.ld(t + 3 * j), a0);
        a1 = fma(xv, tm.ld(t + 3 * j + 1), a1);
        a2 = fma(xv, tm.ld(t + 3 * j + 2), a2);
      }
    }
    __device__ void finish(int idx, double a0, double a1, double a2) const {
      if (idx >= cnt) return;
      const int k = I.lvlRows[beg + idx];
      w[3 * k] = a0;
      w[3 * k + 1] = a1;
      w[3 * k + 2] = a2;
    }
  };

  static __device__ void run(const InstanceDev& I, const Team<CLUSTER>& tm, double* w, double* t) {
    for (int l = 0; l < I.nlevS; ++l) {
      const int beg = I.lvlRowPtr[l], cnt = I.lvlRowPtr[l + 1] - beg;
      dispatch(tm, I.lvlG[4 * l + 0], cnt, FwdGather{I, tm, w, t, beg, cnt});
      tm.sync();
      dispatch(tm, I.lvlG[4 * l + 1], cnt, FwdDense{I, tm, w, t, beg, cnt});
      tm.sync();
    }
    for (int l = I.nlevS - 1; l >= 0; --l) {
      const int beg = I.lvlRowPtr[l], cnt = I.lvlRowPtr[l + 1] - beg;
      dispatch(tm, I.lvlG[4 * l + 2], cnt, BwdGather{I, tm, w, t, beg, cnt});
      tm.sync();
      dispatch(tm, I.lvlG[4 * l + 3], cnt, BwdDense{I, tm, w, t, beg, cnt});
      tm.sync();
    }
  }
};

// Whole substeps of one instance by a team (same steps and formulas as runSubsteps in
// substep_common.cuh, with FMA contraction allowed). Solve::run(I, tm, w, t) turns the gathered
// right-hand side in w (elimination order) into the solution, with t a second 3n workspace: the
// FP64 supernodal solve, or the FP32 solve with one FP64 refinement step (substep_mixed_grid.cu).
template <bool CLUSTER, bool TIMED = false, class Solve = TeamSolve<CLUSTER>>
__device__ void runSubstepsTeam(const InstanceDev& I, const Team<CLUSTER>& tm, int substeps, double* w, double* t,
                                double* red, double* slots) {
  int parity = 0;
  const int T = tm.tid(), NT = tm.count();
  const StageClock<TIMED> clk(I, tm.rank == 0 && threadIdx.x == 0);
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
    clk.lap(I, tm.rank == 0 && threadIdx.x == 0, kStagePredict);
    scale = (scale < I.gScaleHH) ? I.gScaleHH : scale;
    for (int e = T; e < I.ne; e += NT) edgeTerms(I, tm, I.x, e, false);  // projection of x_n
    tm.sync();
    clk.lap(I, tm.rank == 0 && threadIdx.x == 0, kStageLocal);
    int used = 0;
    bool conv = false;
    double lastRes = I.useResidual ? 0.0 : -1.0;
    for (int k = 0; k < I.maxIter; ++k) {
      for (int v = T; v < I.n; v += NT) gatherRow(I, tm, v, w);
      tm.sync();
      clk.lap(I, tm.rank == 0 && threadIdx.x == 0, kStageScatter);
      Solve::run(I, tm, w, t);
      clk.lap(I, tm.rank == 0 && threadIdx.x == 0, kStageSolve);
      // unpack + displacement scan; an over-relaxed iteration puts x_prev + (x_solve − x_prev)·ω
      // and keeps x_solve for the residual (Integrator.cpp:631-641)
      const bool blend = k >= I.chebFrom;
      const bool split = blend && I.useResidual;
      const double om = blend ? I.omega[k] : 1.0;
      double diff = 0.0;
      for (int v = T; v < I.n; v += NT) {
        const int r = I.iperm[v];
        for (int c = 0; c < 3; ++c) {
          const double xs = tm.ld(w + 3 * r + c), p = tm.ld(I.x + 3 * v + c);
          double put = xs;
          if (blend) {
            put = p + (xs - p) * om;
            if (split) I.xsol[3 * v + c] = xs;
          }
          diff = fmax(diff, fabs(put - p));
          I.x[3 * v + c] = put;
        }
      }
      tm.sync();
      clk.lap(I, tm.rank == 0 && threadIdx.x == 0, kStageUnpack);
      const double* X = split ? I.xsol : I.x;
      for (int e = T; e < I.ne; e += NT) edgeTerms(I, tm, X, e, I.useResidual != 0);
      tm.sync();
      clk.lap(I, tm.rank == 0 && threadIdx.x == 0, kStageLocal);
      double res = 0.0;
      if (I.useResidual) {
        for (int v = T; v < I.n; v += NT) {
          if (I.pinned[v] || !(I.m[v] > 0.0)) continue;
          const double r = residualAt(I, tm, X, v);
          if (r > res) res = r;
        }
        res = teamMax(tm, res, red, slots, parity);
      }
      if (split) {  // the next scatter projects the over-relaxed positions
        for (int e = T; e < I.ne; e += NT) edgeTerms(I, tm, I.x, e, false);
        tm.sync();
      }
      diff = teamMax(tm, diff, red, slots, parity);
      clk.lap(I, tm.rank == 0 && threadIdx.x == 0, kStageUnpack);
      // gate (Integrator.cpp:676-747): every thread holds the reduced values and decides alike
      const double rel = (scale > 0.0) ? diff / scale : diff;
      const bool absHit = (I.absTol > 0.0) && (diff <= I.absTol);
      const bool relHit = (I.relTol > 0.0) && (rel <= I.relTol);
      conv = I.useResidual ? (res <= I.resThreshold) : (absHit || relHit);
      used = k + 1;
      lastRes = I.useResidual ? res : -1.0;
      if (I.resTrace && I.useResidual && T == 0) I.resTrace[(size_t)step * I.maxIter + k] = res;
      if (conv) break;
    }
    for (int v = T; v < I.n; v += NT) {  // velocity, damping, pin resnap
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
    clk.lap(I, tm.rank == 0 && threadIdx.x == 0, kStageVelocity);
    clk.finish(I, tm.rank == 0 && threadIdx.x == 0);
  }
}

}  // namespace pdg
