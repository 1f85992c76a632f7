// device.cuh — per-instance device descriptor shared by the substep kernels.
//
// One cloth instance = one entry of a work table. Each kernel block takes one instance and runs
// whole substeps on it, so a batch of cloths is one launch with one block per cloth.
#pragma once

#include <cstdint>

namespace pdg {

struct InstanceDev {
  // sizes
  int32_t n, ne, nb;
  int32_t nlevF, nlevB;
  int32_t maxIter;
  int32_t useResidual;   // residual_tolerance > 0: the residual alone decides convergence
  int32_t hasBendRhs;
  // host-computed scalars (bitwise the same expressions as the reference)
  double h;              // dt
  double invH2;          // 1/(h·h)
  double dampInvH;       // (1 − k_d)·(1/h)
  double gh2[3];         // g·(h·h)
  double gScaleHH;       // |g|·h·h
  double resThreshold;   // residual_tolerance · max(|g|, 1e−12)
  double relTol, absTol;
  // over-relaxed iterates (Integrator.cpp:476-645): iteration k ≥ chebFrom puts
  // x_prev + ω_k·(x_solve − x_prev) and gates on the residual of x_solve
  int32_t chebFrom;      // INT32_MAX: plain PD
  const double* omega;   // maxIter weights ω_k
  // vertex state (3n interleaved unless noted)
  double* x;
  double* v;
  double* xn;            // positions at the start of the substep
  double* xhat;          // predicted positions
  double* xsol;          // the solve's result before over-relaxation (residual point)
  double* bbase;         // (M/h²)·x̂
  const double* m;       // n
  const uint8_t* pinned; // n
  const double* q;       // pin positions
  const double* bendRhs; // 3n or null
  // edges
  const int32_t* eab;    // 2E
  const double* erest;
  const double* ek;
  double* kd;            // 3E  κ·d_e (scatter contribution of the current iterate)
  double* rc;            // 3E  κ·(x_a − x_b) − κ·d_e (residual contribution)
  const int32_t* sstart; // n+1, colour-ordered incidence (edge << 1 | vertex is b)
  const int32_t* sinc;
  const int32_t* rstart; // n+1, edge-ordered incidence
  const int32_t* rinc;
  const int32_t* bstart; // n+1, bend incidence in stencil order
  const int32_t* binc;
  const double* bfac;    // (−k)·w_v per incidence
  const int32_t* babc;   // 3B
  // factor of P·Ã·Pᵀ
  const int32_t* iperm;  // vertex → elimination position
  const int32_t* Lrp;    // forward CSR (row r: columns ascending)
  const int32_t* Lci;
  const double* Lrv;
  const int32_t* Lcp;    // backward CSC (column k: rows ascending)
  const int32_t* Lri;
  const double* Lcv;
  const double* dinv;
  const int32_t* fwdPtr;
  const int32_t* fwdRows;
  const int32_t* bwdPtr;
  const int32_t* bwdRows;
  double* w;             // 3n solve workspace in elimination order (global fallback)
  // supernodal form (nested-dissection tree levels)
  int32_t nlevS;
  const int32_t* lvlRowPtr;
  const int32_t* lvlRows;
  const int32_t* rowSn;
  const int32_t* snStart;
  const int32_t* offEnd;
  const int32_t* offBeg;
  const int64_t* snInvOff;
  const double* invL;
  const double* invLT;
  double* tbuf;          // second 3n workspace (global fallback)
  const int32_t* lvlG;   // lanes per row for [level][fwd gather, fwd dense, bwd gather, bwd dense]
  // mixed precision
  int32_t proj32;        // projection (d_e) computed in FP32, accumulated in FP64
  const int32_t* lvlG32; // lanes per row for the one-CTA FP32 solve
  const float* Lrv32;
  const float* Lcv32;
  const float* invL32;
  const float* invLT32;
  const float* dinv32;
  const int32_t* Aptr;   // Ã in elimination order (FP64 refinement residual)
  const int32_t* Acol;
  const double* Aval;
  double* x0;            // 3n global fallback workspaces of the one-CTA mixed kernel
  float* y32;
  float* t32;
  // dense-inverse solve for small cloths: Ã⁻¹ in vertex order (FP32, rows padded to denseLd) and
  // Ã in vertex order (FP64) for the refinement residual
  int32_t denseLd;
  const float* Ainv;
  const float* AinvLo;         // FP64 team kernel: Ã⁻¹ − Ainv as FP32 (Ainv + AinvLo = the FP64 inverse
                               // to ≈2⁻⁴⁸ relative), rows padded to denseLd; null otherwise
  const int32_t* Vptr;
  const int32_t* Vcol;
  const double* Vval;
  // correction-form dense solve by a team of CTAs (MIXED). Exchange words carry
  // (epoch << 32 | FP32 bits): a reader knows a word is current from its epoch alone.
  int32_t denseResRows;        // rows of Ã⁻¹ a CTA keeps in shared memory (multiple of 4 unless all)
  int32_t teamECap, teamBCap;  // most edge / bend incidences of one CTA's vertices
  int32_t teamWCap;            // most window vertices of one CTA
  const int4* tEdge;           // per edge incidence (rstart order): other | pinned << 31, rest, κ (FP32 bits), 0
  const int4* tBend;           // per bend incidence (bstart order): a, b, c (| pinned << 31), (−k)·w_v bits
  const float4* tVtx;          // per vertex: m/h², 1/m (0 when m ≤ 0), pinned, 0
  const float4* qhl;           // per vertex: pin position as hi (x, y, z, 0), lo (x, y, z, 0)
  float* xhl;                  // 8n: positions as pairs (one-CTA correction kernel)
  float* xhathl;               // 8n: x̂ as pairs (one-CTA correction kernel)
  unsigned long long* rtag;    // 2 × 3n words: correction b − Ã·x, component-major, two buffers
  unsigned long long* xtag;    // 6n words: positions as hi x, y, z, lo x, y, z (x = hi + lo)
  unsigned long long* ptag;    // 3 × team × 16 words: per-CTA partial maxima (A in two buffers, B)
  uint32_t* epoch;             // last exchange epoch of the previous launch
  const int32_t* window;       // 2 × team: vertex range [lo, hi) whose positions a CTA reads
  int32_t* err;                // set when an exchange gave up waiting
  int32_t withholdRank;        // failure-path test hook, −1 otherwise: this CTA of the team withholds
                               // its exchange-A partial in the first iteration of a launch, so the
                               // team's bounded waits run out and report through err
  // statistics
  double* stageNs;       // null, or the stage-time accumulators (ns) of StageTimes, rank 0's view:
                         // predict, localStep, scatter, solve, unpackScan, velocity, total
  double* resTrace;      // null, or per substep of the current launch maxIter values: the gate's
                         // residual after each iteration (NaN for iterations not run)
  int32_t* iterLog;      // per substep of the current launch
  uint8_t* convLog;
  double* lastResidual;  // scalar
  int32_t* earlyExits;   // scalar, accumulates
  int32_t* iterationsUsed;
  int32_t* converged;
};

// Stages of StageTimes (core/sim/Scene.h:140-149) timed on the device.
enum StageIndex { kStagePredict = 0, kStageLocal, kStageScatter, kStageSolve, kStageUnpack, kStageVelocity, kStageTotal,
                  kStageCount };

// %globaltimer laps of one thread (rank 0's thread 0) into I.stageNs; nothing when stageNs is null.
// A lap is taken right after a barrier, so the stage it closes is finished in the whole CTA. The
// two timestamps live in shared memory (one pair per CTA of the kernel), so a kernel carries only
// the `on` predicate in registers.
static __shared__ unsigned long long stageStamp[2];  // start of the substep, last lap
static __shared__ int stageOn;                        // this CTA times stages (rank 0, stageNs set)

// TIMED = false (every launch unless stage timing is on): no code at all, so the untimed kernels
// are compiled exactly as without timing; the timed instantiations are launched only while it is on.
template <bool TIMED>
struct StageClock {
  __device__ __forceinline__ StageClock(const InstanceDev&, bool) {}
  __device__ __forceinline__ void lap(const InstanceDev&, bool, int) const {}
  __device__ __forceinline__ void finish(const InstanceDev&, bool) const {}
};

template <>
struct StageClock<true> {
  __device__ __forceinline__ StageClock(const InstanceDev& I, bool thread0) {
    if (thread0) {
      stageOn = I.stageNs != nullptr;
      if (stageOn) stageStamp[0] = stageStamp[1] = now();
    }
  }
  static __device__ __forceinline__ unsigned long long now() {
    unsigned long long v;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(v));
    return v;
  }
  // called by every thread; only the timing thread (the one that set stageOn) acts
  __device__ __forceinline__ void lap(const InstanceDev& I, bool thread0, int stage) const {
    if (!thread0 || !stageOn) return;
    const unsigned long long n = now();
    I.stageNs[stage] += static_cast<double>(n - stageStamp[1]);
    stageStamp[1] = n;
  }
  // closes the substep at the last lap's stamp, so that the stages partition the total exactly
  __device__ __forceinline__ void finish(const InstanceDev& I, bool thread0) const {
    if (!thread0 || !stageOn) return;
    I.stageNs[kStageTotal] += static_cast<double>(stageStamp[1] - stageStamp[0]);
    stageStamp[0] = stageStamp[1];
  }
};

// Launch the reference-order FP64 substep kernel over `count` instances.
int launchSubstepExact(const InstanceDev* dInstances, int count, int substeps, int smemBytes,
                       void* stream, bool timed = false);
// Reference-order FP64 3-column solve for one instance: b (3n, vertex order) → x.
int launchSolveExact(const InstanceDev* dInstance, const double* b, double* x, int smemBytes,
                     void* stream);
// One column of that solve: b, x of n doubles in vertex order; w an n-double workspace used when
// 8n bytes exceed smemBytes. Bit-identical to the matching column of launchSolveExact.
int launchSolveColumnExact(const InstanceDev* dInstance, const double* b, double* x, double* w, int smemBytes,
                           void* stream);
// FP64 substep with the supernodal solve (smem: 6n doubles when they fit).
int launchSubstepFast(const InstanceDev* dInstances, int count, int substeps, int smemBytes, void* stream,
                      bool timed = false);
int launchSolveFast(const InstanceDev* dInstance, const double* b, double* x, int smemBytes, void* stream);
// FP64 supernodal substep with `clusterSize` CTAs (a thread-block cluster) per instance.
int launchSubstepCluster(const InstanceDev* dInstances, int count, int clusterSize, int substeps, void* stream,
                         bool timed = false);
// `want` if a cluster of that many 256-thread CTAs can run on this device, else 0.
int clusterSizeSupported(int want);
// One cloth (dInstances[0]) of the FP64 supernodal substep by `ctas` co-resident CTAs on a
// cooperative launch (the cluster code with grid barriers); gridCapacity: the most CTAs it holds.
int launchSubstepGrid(const InstanceDev* dInstances, int ctas, int substeps, void* stream, bool timed = false);
int gridCapacity();
// FP32-solve substep (FP32 supernodal solve + one FP64 refinement step) of one large cloth on a
// cooperative grid of `ctas` 256-thread CTAs (substep_mixed_grid.cu); mixedGridCapacity() is the
// most CTAs co-resident on the device.
int launchSubstepMixedGrid(const InstanceDev* dInstances, int ctas, int substeps, void* stream, bool timed = false);
int mixedGridCapacity();
// Mixed-precision substep (FP32 solve + one FP64 refinement step): one CTA per instance with
// smemBytes of workspace (72·n when it fits, else 0 = global), or a cluster of clusterSize CTAs
// per instance, each CTA solving the whole system in its own shared memory (72·max n bytes).
int launchSubstepMixed(const InstanceDev* dInstances, int count, int substeps, int smemBytes, void* stream);
int launchSubstepMixedCluster(const InstanceDev* dInstances, int count, int clusterSize, int smemBytes, int substeps,
                              void* stream);
int mixedClusterSupported(int clusterSize, int smemBytes);
// Mixed-precision substep for small cloths with the explicit FP32 inverse: the cluster splits
// the rows of Ã⁻¹ (smemBytes = 48·n + 12·denseLd).
int launchSubstepDenseCluster(const InstanceDev* dInstances, int count, int clusterSize, int smemBytes, int substeps,
                              void* stream);
int denseClusterSupported(int clusterSize, int smemBytes);
// MIXED substep for small cloths by `team` co-resident CTAs per instance (cooperative launch):
// x ← x + Ã⁻¹·(b − Ã·x) with the rows of the explicit FP32 inverse split over the team.
int launchSubstepDelta(const InstanceDev* dInstances, int count, int team, int smemBytes, int substeps, void* stream,
                       bool timed = false);
// CTAs of kDeltaThreads threads with smemBytes each that can be co-resident on the device.
int deltaResidentCtas(int smemBytes);
// MIXED substep for cloths above the explicit-inverse limit, one CTA per instance: x ← x +
// L⁻¹·(b − Ã·x) with the FP32 supernodal solve (smemBytes: 24·n when the solve vectors fit).
int launchSubstepCorr(const InstanceDev* dInstances, int count, int substeps, int smemBytes, void* stream,
                      bool timed = false);
// The same by a thread-block cluster of `cs` 256-thread CTAs per instance (vectors in L2).
int launchSubstepCorrCluster(const InstanceDev* dInstances, int count, int cs, int substeps, void* stream,
                             bool timed = false);
// `cs` if a cluster of that many correction-kernel CTAs can run on this device, else 0.
int corrClusterSupported(int cs);
// One cloth (dInstances[0]) by `ctas` co-resident CTAs on a cooperative launch: the cluster code
// with grid barriers. corrGridCapacity: the most CTAs such a launch can hold on this device.
int launchSubstepCorrGrid(const InstanceDev* dInstances, int ctas, int substeps, void* stream, bool timed = false);
// A MIXED batch above the explicit-inverse limit as a work table (substep_corr.cu): resident CTAs of
// `threads` (512 or 1024) threads take cloths in descriptor order from *counter (reset here, on the
// stream, before the launch) until none is left; dynamic shared memory smemBytes per CTA.
int launchSubstepCorrWork(const InstanceDev* dInstances, int count, int* counter, int threads, int substeps,
                          int smemBytes, void* stream, bool timed = false);
int corrGridCapacity();
constexpr int kDeltaThreads = 512;
// warps of the MIXED team kernel that apply the CTA's rows of Ã⁻¹, each leaving a partial sum per row
// and component in shared memory
constexpr int kDeltaProductWarps = 8;

// FP64 team kernel (substep_delta64.cu) on `team` CTAs of kDeltaThreads threads per cloth, the
// correction form with Ã⁻¹·r in double-float arithmetic; delta64ResidentCtas as deltaResidentCtas.
int launchSubstepDelta64(const InstanceDev* dInstances, int count, int team, int smemBytes, int substeps,
                         void* stream, bool timed = false);
int delta64ResidentCtas(int smemBytes);

// Column segments a row group of Ã⁻¹ is split into by the FP64 team kernel (its partial sums of Δ).
constexpr int kDelta64Segments = 2;

// Byte offsets of the FP64 team kernel's dynamic shared memory, computed alike on the host (to size
// the launch and the rows of Ã⁻¹ that fit) and in the kernel. FP32 arrays first (16-byte aligned
// float4 rows: ld is a multiple of 32), then FP64, then int32:
//   r as hi and lo (3·ld floats each), resident rows of Ã⁻¹ as hi and lo (resRows·ld each),
//   window positions (3·wCap), per own edge incidence ℓ, κ and per bend incidence (−k)·w_v,
//   per own vertex m/h², m, x̂, x_n, v and t (the residual force), per edge and per bend incidence
//   its six FP64 terms, the segments' partial sums of Δ as FP32 pairs,
//   per edge incidence the other vertex, per bend incidence its three vertices, per own vertex
//   the pinned flag, the incidence offsets of own vertices, and each incidence's own vertex.
struct Delta64Carve {
  size_t rh, rl, ah, al, xw, erest, ekap, bfac, mh2, mass, xh, xn, v, tres, econ, bcon, dl, eo, bv, pin, eb, bb,
      eown, bown, total;
  __host__ __device__ Delta64Carve(int n, int ld, int resRows, int wCap, int eCap, int bCap, int chunk) {
    (void)n;
    size_t o = 0;
    auto take = [&](size_t bytes) {
      const size_t at = o;
      o += bytes;
      return at;
    };
    rh = take(12ull * ld);
    rl = take(12ull * ld);
    ah = take(4ull * resRows * ld);
    al = take(4ull * resRows * ld);
    xw = take(24ull * wCap);
    erest = take(8ull * eCap);
    ekap = take(8ull * eCap);
    bfac = take(8ull * bCap);
    mh2 = take(8ull * chunk);
    mass = take(8ull * chunk);
    xh = take(24ull * chunk);
    xn = take(24ull * chunk);
    v = take(24ull * chunk);
    tres = take(24ull * chunk);
    econ = take(48ull * eCap);
    bcon = take(48ull * bCap);
    dl = take(24ull * kDelta64Segments * chunk);  // 2 floats for each of 3·chunk entries per segment
    eo = take(4ull * eCap);
    bv = take(12ull * bCap);
    pin = take(4ull * chunk);
    eb = take(4ull * (chunk + 1));
    bb = take(4ull * (chunk + 1));
    eown = take(4ull * eCap);
    bown = take(4ull * bCap);
    total = o;
  }
};

// Work arrays of one gradient problem (adjoint.cu): the loss is the mean over free vertices of
// |x_S − target|² after S substeps with the iteration count fixed.
struct GradDev {
  const double* target;  // 3n
  const double* force;   // 3n or null
  double* ckX;           // S × 3n checkpoints of x
  double* ckV;           // S × 3n checkpoints of v
  double* it;            // (K + 1) × 3n iterates of the substep being reversed (recompute mode)
  double* itAll;         // S × (K + 1) × 3n iterates of every substep, or null: recompute from
                         // the checkpoints
  double* xs;            // working state
  double* vs;
  double* xb;            // adjoints
  double* vb;
  double* xkb;
  double* xnb;
  double* xhb;
  double* ge;            // 3E: κ_e·J_e·(λ_a − λ_b)
  double* kb;            // E
  double* fb;            // 3n
  double* loss;          // 1
  int32_t wantGrad;
};
// Loss (and, where wantGrad, gradients) of `count` problems, one CTA each (smemBytes: 48·n when
// the solve vectors fit) or a thread-block cluster of clusterSize CTAs each (vectors in the
// instances' L2 workspaces). gradClusterSupported: clusterSize if the device runs it, else 0.
int launchGradient(const InstanceDev* dInstances, const GradDev* dGrads, int count, int clusterSize, int substeps,
                   int smemBytes, void* stream);
int gradClusterSupported(int clusterSize);
// Fills the instance's Ã⁻¹ (FP32, rows denseLd apart) from its FP64 supernodal factor: three
// columns per CTA, one in each component of the solve.
int launchDenseInverse(const InstanceDev* dInstance, int n, void* stream);

// Power iteration on the linearised PD map of one instance at its positions (spectrum.cu):
// out[0..3] = ρ(T), its previous estimate, λ_max(B), its previous estimate. Work arrays of 3n
// (x0, p, y) and 3E (nE) doubles; a cluster of clusterSize CTAs when the device runs it, else one.
int launchSpectrum(const InstanceDev* dInstance, const double* x0, double* p, double* y, double* nE, double* out,
                   int iters, int clusterSize, void* stream);

// Device arrays of one instance's factor for the numeric refactorization (refactor.cu).
struct RefactorDev {
  int32_t n;
  int32_t maxRowLen;       // longest CSR row of L
  int64_t nnz;             // strictly lower entries
  int64_t nInv;            // entries of the packed block inverses
  const int32_t* colptr;
  const int32_t* rowidx;
  double* colval;
  const int32_t* rowptr;
  const int32_t* colidx;
  double* rowval;
  double* d;
  double* dinv;
  const int32_t* cscToCsr;
  const int32_t* aPosCsc;
  const int32_t* aPosDiag;
  const double* Aval;      // Ã in elimination order (CSR)
  const int32_t* snStart;
  const int32_t* rowSn;
  const int32_t* offEnd;
  const int64_t* snInvOff;
  double* invL;
  double* invLT;
  float* rowval32;
  float* colval32;
  float* invL32;
  float* invLT32;
  float* dinv32;
  int* status;             // set to j + 1 for a zero or non-finite pivot d_j
};
// Shared memory of one level launch for rows of up to maxRowLen entries.
int refactorSmemBytes(int maxRowLen);
// LDLᵀ values level by level — the columns dLvlRows[lvlRowPtr[l] .. lvlRowPtr[l+1]) and the
// supernodes dSnByLevel[snLevelPtr[l] .. snLevelPtr[l+1]) of level l (the pointers into them are
// host arrays) — then the block inverses of the ns supernodes (maxSn: the largest) and the FP32
// copies.
int launchRefactor(const RefactorDev& r, const int32_t* dSnByLevel, const int32_t* snLevelPtr, const int32_t* dLvlRows,
                   const int32_t* lvlRowPtr, int levels, int ns, int maxSn, void* stream);

// One instance's state in the caller's page-locked host arrays (device-visible addresses) and in
// the arena (state_copy.cu).
struct HostStateDev {
  double* hx;
  double* hv;
  double* dx;
  double* dv;
  const int32_t* err;  // the instance's team-exchange error flag, or null
  int32_t n;
};
// Host → arena for every instance (grid: chunks × instances, count ≤ 65535); sets status[0] when
// a position is not finite. maxN: the largest instance's vertex count. status: two ints in mapped
// host memory (device-visible address).
int launchGatherState(const HostStateDev* dTable, int count, int maxN, int* status, void* stream);
// Arena → host for every instance; sets status[1] when an instance's error flag is set.
int launchScatterState(const HostStateDev* dTable, int count, int maxN, int* status, void* stream);

constexpr int kBlockThreads = 256;   // one CTA per cloth (several CTAs share an SM in a batch), and
                                      // the CTAs of the FP64 cluster kernel (fewer threads per
                                      // barrier beat more threads per level there)
constexpr int kClusterThreads = 1024; // mixed cluster kernels: one CTA fills its SM to hide L2 latency

}  // namespace pdg
