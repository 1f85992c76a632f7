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
  // vertex state (3n interleaved unless noted)
  double* x;
  double* v;
  double* xn;            // positions at the start of the substep
  double* xhat;          // predicted positions
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
  // statistics
  int32_t* iterLog;      // per substep of the current launch
  uint8_t* convLog;
  double* lastResidual;  // scalar
  int32_t* earlyExits;   // scalar, accumulates
  int32_t* iterationsUsed;
  int32_t* converged;
};

// Launch the reference-order FP64 substep kernel over `count` instances.
int launchSubstepExact(const InstanceDev* dInstances, int count, int substeps, int smemBytes,
                       void* stream);
// Reference-order FP64 3-column solve for one instance: b (3n, vertex order) → x.
int launchSolveExact(const InstanceDev* dInstance, const double* b, double* x, int smemBytes,
                     void* stream);
// FP64 substep with the supernodal solve (smem: 6n doubles when they fit).
int launchSubstepFast(const InstanceDev* dInstances, int count, int substeps, int smemBytes, void* stream);
int launchSolveFast(const InstanceDev* dInstance, const double* b, double* x, int smemBytes, void* stream);
// FP64 supernodal substep with `clusterSize` CTAs (a thread-block cluster) per instance.
int launchSubstepCluster(const InstanceDev* dInstances, int count, int clusterSize, int substeps, void* stream);
// `want` if a cluster of that many 256-thread CTAs can run on this device, else 0.
int clusterSizeSupported(int want);

constexpr int kBlockThreads = 256;

}  // namespace pdg
