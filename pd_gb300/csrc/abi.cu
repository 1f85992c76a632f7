// abi.cu — the C ABI of include/pd_gb300.h: instance build, device arena, sim and solver handles.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <iterator>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <type_traits>
#include <random>
#include <string>
#include <vector>

#include "../../include/pd_gb300.h"
#include "device.cuh"
#include "host.hpp"

namespace {

thread_local std::string g_lastError;

int fail(int code, const std::string& msg) {
  g_lastError = msg;
  return code;
}
}  // namespace

namespace pdg {
void setLastError(const std::string& msg) { g_lastError = msg; }
}  // namespace pdg

namespace {
int cudaFail(cudaError_t e, const char* what) {
  return fail(PD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define PD_CUDA(call)                                   \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cudaFail(e_, #call);  \
  } while (0)

using Clock = std::chrono::steady_clock;
double secondsSince(Clock::time_point t0) {
  return std::chrono::duration<double>(Clock::now() - t0).count();
}

pdg::GridSpec gridSpecOf(const pd_scene_config& c) {
  pdg::GridSpec g;
  g.nx = c.grid_nx;
  g.ny = c.grid_ny;
  g.spacing = c.grid_spacing;
  g.stiffness = c.stiffness;
  g.density = c.density;
  g.shearStiffness = c.shear_stiffness;
  g.bendStiffness = c.bend_stiffness;
  g.bendSampling = c.bend_sampling;
  g.bendStride = c.bend_stride;
  g.massMode = c.mass_mode;
  g.totalMass = c.total_mass;
  g.pinMode = c.pin_mode;
  return g;
}

// ------------------------------------------------------------------------------ device arena
// All arrays of all instances of a handle live in one device allocation, uploaded with one copy.
struct Arena {
  std::vector<uint8_t> host;
  size_t add(const void* src, size_t bytes) {
    const size_t off = (host.size() + 255) & ~size_t(255);
    host.resize(off + (bytes ? bytes : 1), 0);
    if (src && bytes) std::memcpy(host.data() + off, src, bytes);
    return off;
  }
  template <class T>
  size_t add(const std::vector<T>& v) {
    return add(v.data(), v.size() * sizeof(T));
  }
  size_t zeros(size_t bytes) { return add(nullptr, bytes); }
};

// One cloth: host preparation plus the offsets of its device arrays.
struct Instance {
  pdg::Scene scene;
  pd_scene_config cfg{};
  pdg::Topology topo;
  pdg::ScalarMatrix L;
  pdg::Factor F;
  pdg::SupernodeTree tree;
  pdg::Stamp stamp;
  std::vector<double> bendRhs;
  int factorizeCount = 0, analyzeCount = 0;
  // arena offsets
  size_t oX, oV, oXn, oXhat, oXsol, oBbase, oM, oPin, oQ, oBend, oEab, oRest, oK, oKd, oRc, oSs, oSi, oRs, oRi, oBs,
      oBi, oBf, oBabc, oIperm, oLrp, oLci, oLrv, oLcp, oLri, oLcv, oDinv, oFp, oFr, oBp, oBr, oW, oLastRes,
      oEarly, oIters, oConv, oLvlPtr, oLvlRows, oRowSn, oSnStart, oOffEnd, oOffBeg, oSnInv, oInvL, oInvLT, oT,
      oLvlG, oLvlG32, oLrv32, oLcv32, oInvL32, oInvLT32, oDinv32, oAptr, oAcol, oAval, oX0, oY32, oT32, oAinv, oAinvLo,
      oVptr, oVcol, oVval, oRtag, oXtag, oPtag, oEpoch, oWindow, oErr, oTEdge, oTBend, oTVtx, oQhl, oXhl,
      oXhatHl, oD, oCscToCsr, oAPosCsc, oAPosDiag, oSnByLevel;
  bool gpuRefactor = false;   // the next upload computes the factor's values on the device
  double assembleSeconds = 0.0;  // StageTimes::assemble: (re)factorizations, host and device
  int deviceRefactorCount = 0;
  std::vector<int32_t> patRowptr, patCol;  // pattern of Ã the current symbolic factor was built for
  int denseLd = 0;      // > 0: Ã⁻¹ is in the arena
  int corrTeam = 1;     // correction kernel: CTAs (a cluster when > 1) running this instance
  int corrThreads = pdg::kBlockThreads;  // correction kernel: threads of the CTA(s) running it
  int denseResRows = 0; // team kernel: rows of Ã⁻¹ each CTA keeps in shared memory
  int teamECap = 0, teamBCap = 0;
  int teamWCap = 0;     // most window vertices of one CTA
  size_t bytes = 0;
};

bool validPrecision(int p) { return p >= PD_PRECISION_FP64_EXACT && p <= PD_PRECISION_MIXED; }
// FP64 supernodal solve (with FP64 or FP32 projection)
bool supernodalFp64(int p) { return p == PD_PRECISION_FP64 || p == PD_PRECISION_FP32_PROJECTION; }
// FP32 solve + FP64 refinement
bool mixedSolve(int p) { return p == PD_PRECISION_FP32_SOLVE || p == PD_PRECISION_MIXED; }
bool projection32(int p) { return p == PD_PRECISION_FP32_PROJECTION || p == PD_PRECISION_MIXED; }
// bytes of per-CTA workspace: reference order w; supernodal w, t; mixed B, X0 (FP64) and Y, T (FP32)
int workspaceBytesPerVertex(int p) { return mixedSolve(p) ? 72 : (p == PD_PRECISION_FP64_EXACT ? 24 : 48); }

// The reference-order mode keeps the host factorization: its bits are part of the parity bar.
// PD_GB300_HOST_REFACTOR=1 forces the host path for every mode (to compare the two).
bool deviceRefactorAllowed(int precision) {
  if (precision == PD_PRECISION_FP64_EXACT) return false;
  const char* env = std::getenv("PD_GB300_HOST_REFACTOR");
  return !(env && env[0] == '1');
}

std::string prepare(Instance& I, bool reanalyze) {
  const auto& c = I.cfg;
  if (!(c.dt > 0.0)) return "dt must be positive";
  if (c.max_iterations < 0) return "max_iterations must be >= 0";
  if (!validPrecision(c.precision)) return "unsupported precision mode";
  if (c.cheb_mode < PD_CHEB_OFF || c.cheb_mode > PD_CHEB_INTERVAL) return "cheb_mode must be 0, 1 or 2";
  std::string err = pdg::validateScene(I.scene);
  if (!err.empty()) return err;
  pdg::assembleMatrix(I.scene, c.dt, I.L);
  std::vector<int32_t> perm;
  if (reanalyze || I.F.perm.empty()) {
    perm = pdg::nestedDissection(I.scene, I.L, 24, &I.tree);
    I.analyzeCount += 1;
  } else {
    perm = I.F.perm;
  }
  if (!reanalyze && !perm.empty() && deviceRefactorAllowed(c.precision) && I.F.maxRowLen > 0 &&
      I.L.rowptr == I.patRowptr && I.L.col == I.patCol &&
      pdg::refactorSmemBytes(I.F.maxRowLen) <= 200 * 1024) {
    // same pattern, new values: the numeric LDLᵀ runs on the device at the next upload
    pdg::refreshAval(I.F, I.L);
    I.gpuRefactor = true;
  } else {
    pdg::Factor fresh;  // a failed factorization leaves the previous factor whole
    if (!pdg::factorize(I.L, perm, fresh, &err)) {
      I.stamp = pdg::Stamp{};  // L holds the failed values: the next edit rebuilds from the scene
      return err;
    }
    I.F = std::move(fresh);
    pdg::buildSupernodal(I.F, I.tree);
    pdg::buildMixed(I.F, I.L);
    if (c.precision != PD_PRECISION_FP64_EXACT) pdg::buildRefactorMaps(I.F);
    else I.F.maxRowLen = 0;
    I.patRowptr = I.L.rowptr;
    I.patCol = I.L.col;
    I.gpuRefactor = false;
  }
  I.factorizeCount += 1;
  pdg::assembleBendingRhs(I.scene, I.bendRhs);
  I.stamp = pdg::computeStamp(I.scene, c.dt);
  return {};
}

// Shared memory of the team kernel for one instance: positions as hi/lo pairs (32 B a vertex),
// the padded correction (12 B a row), `resRows` rows of Ã⁻¹, and per owned vertex x, x_n, x̂, v
// (FP64) and Δ (FP32). Fills *resRows with as many rows as fit in kDeltaSmem (a multiple of four
// unless all).
constexpr int kDeltaSmem = 220 * 1024;
// Pin positions as FP32 pairs per vertex: hi (x, y, z, 0), lo (x, y, z, 0) with hi = fl32(q) and
// lo = fl32(q − hi), the split the team kernel applies to positions.
std::vector<float> pinPairs(const pdg::Scene& s) {
  std::vector<float> out(8 * static_cast<size_t>(s.n), 0.0f);
  for (size_t v = 0; v < static_cast<size_t>(s.n); ++v) {
    for (int c = 0; c < 3; ++c) {
      const double q = s.q[3 * v + c];
      const float hi = static_cast<float>(q);
      out[8 * v + c] = hi;
      out[8 * v + 4 + c] = static_cast<float>(q - static_cast<double>(hi));
    }
  }
  return out;
}

// Most edge / bend incidences of one CTA's vertex range.
void teamCaps(const Instance& I, int team, int* eCap, int* bCap) {
  const int n = I.scene.n, chunk = (n + team - 1) / team;
  *eCap = *bCap = 0;
  for (int r = 0; r < team; ++r) {
    const int rb = std::min(n, r * chunk), re = std::min(n, rb + chunk);
    *eCap = std::max(*eCap, I.topo.rstart[re] - I.topo.rstart[rb]);
    *bCap = std::max(*bCap, I.topo.bstart[re] - I.topo.bstart[rb]);
  }
}

// Team kernel: the vertex range [lo, hi) whose positions CTA r reads — its vertices, their edge
// neighbours and bend-stencil partners — as (lo, hi) per CTA.
std::vector<int32_t> teamWindows(const Instance& I, int team) {
  const auto& s = I.scene;
  std::vector<int32_t> window(2 * static_cast<size_t>(team), 0);
  const int chunk = (s.n + team - 1) / team;
  for (int r = 0; r < team; ++r) {
    const int rb = std::min(s.n, r * chunk), re = std::min(s.n, rb + chunk);
    if (rb >= re) continue;
    int lo = rb, hi = re;
    for (int v = rb; v < re; ++v) {
      for (int q = I.topo.rstart[v]; q < I.topo.rstart[v + 1]; ++q) {
        const pdg::Edge& e = s.edges[I.topo.rinc[q] >> 1];
        lo = std::min({lo, e.a, e.b});
        hi = std::max({hi, e.a + 1, e.b + 1});
      }
      for (int q = I.topo.bstart[v]; q < I.topo.bstart[v + 1]; ++q) {
        const pdg::Bend& b = s.bends[I.topo.binc[q]];
        lo = std::min({lo, b.a, b.b, b.c});
        hi = std::max({hi, b.a + 1, b.b + 1, b.c + 1});
      }
    }
    window[2 * r] = lo;
    window[2 * r + 1] = hi;
  }
  return window;
}

int teamWindowCap(const Instance& I, int team) {
  const std::vector<int32_t> w = teamWindows(I, team);
  int cap = 0;
  for (int r = 0; r < team; ++r) cap = std::max(cap, w[2 * r + 1] - w[2 * r]);
  return cap;
}

int deltaSmem(const Instance& I, int team, int* resRows) {
  const int n = I.scene.n, ld = (n + 31) / 32 * 32, chunk = (n + team - 1) / team;
  int eCap = 0, bCap = 0;
  teamCaps(I, team, &eCap, &bCap);
  const int wCap = teamWindowCap(I, team);
  // positions, correction, incidences, vertex constants, FP64 state, Δ, incidence offsets
  // (16·chunk vertex constants, 32·chunk x̂, 48·chunk x_n and v, 12·chunk partial sums of Δ per
  // product warp), and the window's previous positions (over-relaxed iterations)
  const long fixed = 32L * n + 12L * ld + 16L * (eCap + bCap) + (96L + 12L * pdg::kDeltaProductWarps) * chunk +
                     8L * (chunk + 1) + 32L * wCap;
  long rows = fixed < kDeltaSmem ? (kDeltaSmem - fixed) / (4L * ld) : 0;
  if (rows >= chunk) {
    rows = chunk;
  } else {
    rows &= ~3L;  // whole groups of four rows
  }
  *resRows = static_cast<int>(rows);
  return static_cast<int>(fixed + 4L * rows * ld);
}

// Shared memory of the FP64 team kernel for one instance (pdg::Delta64Carve), with as many resident
// rows of Ã⁻¹ (hi and lo, 8 bytes an entry) as fit in kDeltaSmem: all of the CTA's rows, else a
// multiple of four.
int delta64Smem(const Instance& I, int team, int* resRows) {
  const int n = I.scene.n, ld = (n + 31) / 32 * 32, chunk = (n + team - 1) / team;
  int eCap = 0, bCap = 0;
  teamCaps(I, team, &eCap, &bCap);
  const int wCap = teamWindowCap(I, team);
  const long fixed = static_cast<long>(pdg::Delta64Carve(n, ld, 0, wCap, eCap, bCap, chunk).total);
  long rows = fixed < kDeltaSmem ? (kDeltaSmem - fixed) / (8L * ld) : 0;
  if (rows >= chunk) {
    rows = chunk;
  } else {
    rows &= ~3L;  // whole groups of four rows
  }
  *resRows = static_cast<int>(rows);
  return static_cast<int>(pdg::Delta64Carve(n, ld, static_cast<int>(rows), wCap, eCap, bCap, chunk).total);
}

// kind: 0 none, 1 dense inverse (cluster kernel), 2 dense inverse + team kernel buffers,
// 3 FP32 tables + position pairs of the one-CTA correction kernel, 4 dense inverse as hi/lo pairs +
// FP64 team kernel buffers
void layout(Instance& I, Arena& A, int teamCtas, int denseKind, double latencyScale = 1.0) {
  const auto& s = I.scene;
  const size_t n = s.n, ne = s.edges.size(), nb = s.bends.size();
  I.oLvlG = A.add(pdg::chooseGroupWidths(I.F, teamCtas, latencyScale));
  const size_t before = A.host.size();
  I.denseLd = 0;
  I.denseResRows = 0;
  I.oAinv = I.oAinvLo = I.oVptr = I.oVcol = I.oVval = 0;
  I.oRtag = I.oXtag = I.oPtag = I.oEpoch = I.oWindow = I.oErr = I.oTEdge = I.oTBend = I.oTVtx = I.oQhl = 0;
  I.oXhl = I.oXhatHl = 0;
  I.teamECap = I.teamBCap = I.teamWCap = 0;
  if (denseKind == 1 || denseKind == 2 || denseKind == 4) {
    // Ã⁻¹ (FP32, rows padded to 32) is filled on the GPU after the upload (launchDenseInverse)
    I.denseLd = static_cast<int>((n + 31) / 32 * 32);
    I.oAinv = A.zeros(4 * n * static_cast<size_t>(I.denseLd));
    if (denseKind == 4) I.oAinvLo = A.zeros(4 * n * static_cast<size_t>(I.denseLd));
    I.oVptr = A.add(I.L.rowptr);
    I.oVcol = A.add(I.L.col);
    I.oVval = A.add(I.L.val);
  }
  if (denseKind == 2 || denseKind == 4) {
    if (denseKind == 2) deltaSmem(I, teamCtas, &I.denseResRows);
    else delta64Smem(I, teamCtas, &I.denseResRows);
    teamCaps(I, teamCtas, &I.teamECap, &I.teamBCap);
    I.teamWCap = teamWindowCap(I, teamCtas);
    // two buffers of 3n values: one word each (FP32), two words each (FP64)
    I.oRtag = A.zeros(8 * 2 * 3 * n * (denseKind == 4 ? 2 : 1));
    I.oXtag = A.zeros(8 * 6 * n);  // 3n positions: hi and lo (FP32), or low and high words (FP64)
    I.oPtag = A.zeros(8 * 3 * 16 * static_cast<size_t>(teamCtas));  // A (two buffers), B; a line each
    I.oEpoch = A.zeros(4);
    I.oErr = A.zeros(4);
    I.oWindow = A.add(teamWindows(I, teamCtas));
  }
  if (denseKind == 2 || denseKind == 3) {
    // incidences in the kernels' FP32 form (pinned endpoints flagged in bit 31)
    auto bitsOf = [](float f) {
      int32_t i;
      std::memcpy(&i, &f, 4);
      return i;
    };
    auto flag = [&](int v) { return s.pinned[v] ? static_cast<int32_t>(0x80000000u | static_cast<uint32_t>(v)) : v; };
    std::vector<int32_t> te(4 * I.topo.rinc.size()), tb(4 * I.topo.binc.size());
    for (int v = 0; v < s.n; ++v) {
      for (int q = I.topo.rstart[v]; q < I.topo.rstart[v + 1]; ++q) {
        const pdg::Edge& e = s.edges[I.topo.rinc[q] >> 1];
        const int o = (I.topo.rinc[q] & 1) ? e.a : e.b;
        te[4 * q] = flag(o);
        te[4 * q + 1] = bitsOf(static_cast<float>(e.rest));
        te[4 * q + 2] = bitsOf(static_cast<float>(e.k));
      }
      for (int q = I.topo.bstart[v]; q < I.topo.bstart[v + 1]; ++q) {
        const pdg::Bend& b = s.bends[I.topo.binc[q]];
        tb[4 * q] = flag(b.a);
        tb[4 * q + 1] = flag(b.b);
        tb[4 * q + 2] = flag(b.c);
        tb[4 * q + 3] = bitsOf(static_cast<float>(I.topo.bfac[q]));
      }
    }
    std::vector<float> tv(4 * n, 0.0f);
    const double invH2 = 1.0 / (I.cfg.dt * I.cfg.dt);
    for (size_t v = 0; v < n; ++v) {
      const double mv = s.m[v];
      tv[4 * v] = static_cast<float>(mv * invH2);
      tv[4 * v + 1] = mv > 0.0 ? static_cast<float>(1.0 / mv) : 0.0f;
      tv[4 * v + 2] = s.pinned[v] ? 1.0f : 0.0f;
    }
    I.oTEdge = A.add(te);
    I.oTBend = A.add(tb);
    I.oTVtx = A.add(tv);
    I.oQhl = A.add(pinPairs(s));
    if (denseKind == 3) {
      I.oXhl = A.zeros(32 * n);
      I.oXhatHl = A.zeros(32 * n);
    }
  }
  I.oX = A.add(s.x);
  I.oV = A.add(s.v);
  I.oXn = A.zeros(24 * n);
  I.oXhat = A.zeros(24 * n);
  I.oXsol = A.zeros(24 * n);
  I.oBbase = A.zeros(24 * n);
  I.oM = A.add(s.m);
  I.oPin = A.add(s.pinned);
  I.oQ = A.add(s.q);
  I.oBend = A.add(I.bendRhs);
  std::vector<int32_t> eab(2 * ne);
  std::vector<double> rest(ne), k(ne);
  for (size_t e = 0; e < ne; ++e) {
    eab[2 * e] = s.edges[e].a;
    eab[2 * e + 1] = s.edges[e].b;
    rest[e] = s.edges[e].rest;
    k[e] = s.edges[e].k;
  }
  I.oEab = A.add(eab);
  I.oRest = A.add(rest);
  I.oK = A.add(k);
  I.oKd = A.zeros(24 * ne);
  I.oRc = A.zeros(24 * ne);
  I.oSs = A.add(I.topo.sstart);
  I.oSi = A.add(I.topo.sinc);
  I.oRs = A.add(I.topo.rstart);
  I.oRi = A.add(I.topo.rinc);
  I.oBs = A.add(I.topo.bstart);
  I.oBi = A.add(I.topo.binc);
  I.oBf = A.add(I.topo.bfac);
  std::vector<int32_t> babc(3 * nb);
  for (size_t b = 0; b < nb; ++b) {
    babc[3 * b] = s.bends[b].a;
    babc[3 * b + 1] = s.bends[b].b;
    babc[3 * b + 2] = s.bends[b].c;
  }
  I.oBabc = A.add(babc);
  I.oIperm = A.add(I.F.iperm);
  I.oLrp = A.add(I.F.rowptr);
  I.oLci = A.add(I.F.colidx);
  I.oLrv = A.add(I.F.rowval);
  I.oLcp = A.add(I.F.colptr);
  I.oLri = A.add(I.F.rowidx);
  I.oLcv = A.add(I.F.colval);
  I.oDinv = A.add(I.F.dinv);
  I.oFp = A.add(I.F.fwdLevelPtr);
  I.oFr = A.add(I.F.fwdRows);
  I.oBp = A.add(I.F.bwdLevelPtr);
  I.oBr = A.add(I.F.bwdRows);
  I.oW = A.zeros(24 * n);
  const double minusOne = -1.0;
  I.oLastRes = A.add(&minusOne, sizeof(double));
  I.oEarly = A.zeros(4);
  I.oIters = A.zeros(4);
  I.oConv = A.zeros(4);
  I.oLvlPtr = A.add(I.F.lvlRowPtr);
  I.oLvlRows = A.add(I.F.lvlRows);
  I.oRowSn = A.add(I.F.rowSn);
  I.oSnStart = A.add(I.F.snStart);
  I.oOffEnd = A.add(I.F.offEnd);
  I.oOffBeg = A.add(I.F.offBeg);
  I.oSnInv = A.add(I.F.snInvOff);
  I.oInvL = A.add(I.F.invL);
  I.oInvLT = A.add(I.F.invLT);
  I.oT = A.zeros(24 * n);
  // FP32 solve: the correction kernel's teams are 256-thread CTAs, the other mixed kernels' 1024
  // (a grid team, teamCtas > 16: rows strided over all of its 256-thread CTAs)
  I.oLvlG32 = A.add(denseKind == 3  ? pdg::chooseGroupWidths32(I.F, I.corrThreads, I.corrTeam, latencyScale)
                    : teamCtas > 16 ? pdg::chooseGroupWidths32(I.F, pdg::kBlockThreads, teamCtas, latencyScale)
                                    : pdg::chooseGroupWidths32(I.F, teamCtas > 1 ? pdg::kClusterThreads
                                                                                 : pdg::kBlockThreads,
                                                               1, latencyScale));
  I.oLrv32 = A.add(I.F.rowval32);
  I.oLcv32 = A.add(I.F.colval32);
  I.oInvL32 = A.add(I.F.invL32);
  I.oInvLT32 = A.add(I.F.invLT32);
  I.oDinv32 = A.add(I.F.dinv32);
  I.oAptr = A.add(I.F.Aptr);
  I.oAcol = A.add(I.F.Acol);
  I.oAval = A.add(I.F.Aval);
  I.oX0 = A.zeros(24 * n);
  I.oY32 = A.zeros(12 * n);
  I.oT32 = A.zeros(12 * n);
  I.oD = A.add(I.F.d);
  I.oCscToCsr = A.add(I.F.cscToCsr);
  I.oAPosCsc = A.add(I.F.aPosCsc);
  I.oAPosDiag = A.add(I.F.aPosDiag);
  I.oSnByLevel = A.add(I.F.snByLevel);
  I.bytes = A.host.size() - before;
}

// Over-relaxation weights of one substep's iterations (Integrator.cpp:529,590-617): mode ρ blends
// from k = cheb_start + 1 with ω = 2/(2 − ρ²), then ω ← 4/(4 − ρ²·ω); the interval mode blends
// from k = 0 with ω_k = 1/(m + δ·cos(π(2j − 1)/(2T))), j = k + 1, T = the iteration budget. The
// weights depend on the configuration only, so they are a table computed here.
int32_t chebFrom(const pd_scene_config& c) {
  if (c.cheb_mode == PD_CHEB_INTERVAL) return 0;
  if (c.cheb_mode == PD_CHEB_RHO) return c.cheb_start < 0 ? 0 : c.cheb_start + 1;
  return INT32_MAX;
}

std::vector<double> chebWeights(const pd_scene_config& c) {
  std::vector<double> w(std::max(0, c.max_iterations), 1.0);
  const int from = chebFrom(c);
  double omega = 1.0;
  for (int k = from; k < c.max_iterations; ++k) {
    if (c.cheb_mode == PD_CHEB_RHO) {
      omega = (k == c.cheb_start + 1) ? 2.0 / (2.0 - c.cheb_rho * c.cheb_rho)
                                      : 4.0 / (4.0 - c.cheb_rho * c.cheb_rho * omega);
    } else {
      const double pi = 3.14159265358979323846;
      const double T = static_cast<double>(c.max_iterations);
      const double j = static_cast<double>(k + 1);
      const double theta = pi * (2.0 * j - 1.0) / (2.0 * T);
      omega = 1.0 / (c.cheb_m + c.cheb_d * std::cos(theta));
    }
    w[k] = omega;
  }
  return w;
}

// Failure-path test hook of the team kernel: PD_GB300_TEST_WITHHOLD_RANK=r makes CTA r withhold
// its first exchange-A partial, so the team's bounded waits run out (the launch then fails with
// PD_ERR_CUDA and the exchange words are reset). Read when the descriptors are written; unset: −1.
int32_t withholdRankForTests() {
  const char* env = std::getenv("PD_GB300_TEST_WITHHOLD_RANK");
  if (!env || !env[0]) return -1;
  char* end = nullptr;
  const long r = std::strtol(env, &end, 10);
  return (end && *end == 0 && r >= 0 && r < 1024) ? static_cast<int32_t>(r) : -1;
}

pdg::InstanceDev describe(const Instance& I, uint8_t* base, int32_t* iterLog, uint8_t* convLog,
                          const double* omega, double* resTrace, double* stageNs) {
  auto P = [&](size_t off) { return base + off; };
  const auto& c = I.cfg;
  const auto& s = I.scene;
  pdg::InstanceDev d{};
  d.withholdRank = withholdRankForTests();
  d.stageNs = stageNs;
  d.n = s.n;
  d.ne = static_cast<int32_t>(s.edges.size());
  d.nb = static_cast<int32_t>(s.bends.size());
  d.nlevF = static_cast<int32_t>(I.F.fwdLevelPtr.size()) - 1;
  d.nlevB = static_cast<int32_t>(I.F.bwdLevelPtr.size()) - 1;
  d.maxIter = c.max_iterations;
  d.useResidual = c.residual_tolerance > 0.0 ? 1 : 0;
  d.hasBendRhs = s.bends.empty() ? 0 : 1;
  const double h = c.dt;
  d.h = h;
  d.invH2 = 1.0 / (h * h);
  d.dampInvH = (1.0 - c.velocity_damping) * (1.0 / h);
  for (int k = 0; k < 3; ++k) d.gh2[k] = c.gravity[k] * (h * h);
  const double gl = std::sqrt(c.gravity[0] * c.gravity[0] + c.gravity[1] * c.gravity[1] + c.gravity[2] * c.gravity[2]);
  d.gScaleHH = gl * h * h;
  d.resThreshold = c.residual_tolerance * ((gl < 1.0e-12) ? 1.0e-12 : gl);
  d.relTol = c.rel_tolerance;
  d.absTol = c.abs_tolerance;
  d.x = reinterpret_cast<double*>(P(I.oX));
  d.v = reinterpret_cast<double*>(P(I.oV));
  d.xn = reinterpret_cast<double*>(P(I.oXn));
  d.xhat = reinterpret_cast<double*>(P(I.oXhat));
  d.xsol = reinterpret_cast<double*>(P(I.oXsol));
  d.chebFrom = chebFrom(c);
  d.omega = omega;
  d.resTrace = resTrace;
  d.bbase = reinterpret_cast<double*>(P(I.oBbase));
  d.m = reinterpret_cast<const double*>(P(I.oM));
  d.pinned = reinterpret_cast<const uint8_t*>(P(I.oPin));
  d.q = reinterpret_cast<const double*>(P(I.oQ));
  d.bendRhs = reinterpret_cast<const double*>(P(I.oBend));
  d.eab = reinterpret_cast<const int32_t*>(P(I.oEab));
  d.erest = reinterpret_cast<const double*>(P(I.oRest));
  d.ek = reinterpret_cast<const double*>(P(I.oK));
  d.kd = reinterpret_cast<double*>(P(I.oKd));
  d.rc = reinterpret_cast<double*>(P(I.oRc));
  d.sstart = reinterpret_cast<const int32_t*>(P(I.oSs));
  d.sinc = reinterpret_cast<const int32_t*>(P(I.oSi));
  d.rstart = reinterpret_cast<const int32_t*>(P(I.oRs));
  d.rinc = reinterpret_cast<const int32_t*>(P(I.oRi));
  d.bstart = reinterpret_cast<const int32_t*>(P(I.oBs));
  d.binc = reinterpret_cast<const int32_t*>(P(I.oBi));
  d.bfac = reinterpret_cast<const double*>(P(I.oBf));
  d.babc = reinterpret_cast<const int32_t*>(P(I.oBabc));
  d.iperm = reinterpret_cast<const int32_t*>(P(I.oIperm));
  d.Lrp = reinterpret_cast<const int32_t*>(P(I.oLrp));
  d.Lci = reinterpret_cast<const int32_t*>(P(I.oLci));
  d.Lrv = reinterpret_cast<const double*>(P(I.oLrv));
  d.Lcp = reinterpret_cast<const int32_t*>(P(I.oLcp));
  d.Lri = reinterpret_cast<const int32_t*>(P(I.oLri));
  d.Lcv = reinterpret_cast<const double*>(P(I.oLcv));
  d.dinv = reinterpret_cast<const double*>(P(I.oDinv));
  d.fwdPtr = reinterpret_cast<const int32_t*>(P(I.oFp));
  d.fwdRows = reinterpret_cast<const int32_t*>(P(I.oFr));
  d.bwdPtr = reinterpret_cast<const int32_t*>(P(I.oBp));
  d.bwdRows = reinterpret_cast<const int32_t*>(P(I.oBr));
  d.w = reinterpret_cast<double*>(P(I.oW));
  d.nlevS = static_cast<int32_t>(I.F.lvlRowPtr.size()) - 1;
  d.lvlRowPtr = reinterpret_cast<const int32_t*>(P(I.oLvlPtr));
  d.lvlRows = reinterpret_cast<const int32_t*>(P(I.oLvlRows));
  d.rowSn = reinterpret_cast<const int32_t*>(P(I.oRowSn));
  d.snStart = reinterpret_cast<const int32_t*>(P(I.oSnStart));
  d.offEnd = reinterpret_cast<const int32_t*>(P(I.oOffEnd));
  d.offBeg = reinterpret_cast<const int32_t*>(P(I.oOffBeg));
  d.snInvOff = reinterpret_cast<const int64_t*>(P(I.oSnInv));
  d.invL = reinterpret_cast<const double*>(P(I.oInvL));
  d.invLT = reinterpret_cast<const double*>(P(I.oInvLT));
  d.tbuf = reinterpret_cast<double*>(P(I.oT));
  d.lvlG = reinterpret_cast<const int32_t*>(P(I.oLvlG));
  d.proj32 = projection32(c.precision) ? 1 : 0;
  d.lvlG32 = reinterpret_cast<const int32_t*>(P(I.oLvlG32));
  d.Lrv32 = reinterpret_cast<const float*>(P(I.oLrv32));
  d.Lcv32 = reinterpret_cast<const float*>(P(I.oLcv32));
  d.invL32 = reinterpret_cast<const float*>(P(I.oInvL32));
  d.invLT32 = reinterpret_cast<const float*>(P(I.oInvLT32));
  d.dinv32 = reinterpret_cast<const float*>(P(I.oDinv32));
  d.Aptr = reinterpret_cast<const int32_t*>(P(I.oAptr));
  d.Acol = reinterpret_cast<const int32_t*>(P(I.oAcol));
  d.Aval = reinterpret_cast<const double*>(P(I.oAval));
  d.x0 = reinterpret_cast<double*>(P(I.oX0));
  d.y32 = reinterpret_cast<float*>(P(I.oY32));
  d.t32 = reinterpret_cast<float*>(P(I.oT32));
  d.denseLd = I.denseLd;
  if (I.denseLd > 0) {
    d.Ainv = reinterpret_cast<const float*>(P(I.oAinv));
    d.AinvLo = I.oAinvLo ? reinterpret_cast<const float*>(P(I.oAinvLo)) : nullptr;
    d.Vptr = reinterpret_cast<const int32_t*>(P(I.oVptr));
    d.Vcol = reinterpret_cast<const int32_t*>(P(I.oVcol));
    d.Vval = reinterpret_cast<const double*>(P(I.oVval));
  }
  d.denseResRows = I.denseResRows;
  if (I.oTEdge) {
    d.tEdge = reinterpret_cast<const int4*>(P(I.oTEdge));
    d.tBend = reinterpret_cast<const int4*>(P(I.oTBend));
    d.tVtx = reinterpret_cast<const float4*>(P(I.oTVtx));
    d.qhl = reinterpret_cast<const float4*>(P(I.oQhl));
  }
  if (I.oXhl) {
    d.xhl = reinterpret_cast<float*>(P(I.oXhl));
    d.xhathl = reinterpret_cast<float*>(P(I.oXhatHl));
  }
  if (I.oRtag) {
    d.teamECap = I.teamECap;
    d.teamWCap = I.teamWCap;
    d.teamBCap = I.teamBCap;
    d.rtag = reinterpret_cast<unsigned long long*>(P(I.oRtag));
    d.xtag = reinterpret_cast<unsigned long long*>(P(I.oXtag));
    d.ptag = reinterpret_cast<unsigned long long*>(P(I.oPtag));
    d.epoch = reinterpret_cast<uint32_t*>(P(I.oEpoch));
    d.window = reinterpret_cast<const int32_t*>(P(I.oWindow));
    d.err = reinterpret_cast<int32_t*>(P(I.oErr));
  }
  d.iterLog = iterLog;
  d.convLog = convLog;
  d.lastResidual = reinterpret_cast<double*>(P(I.oLastRes));
  d.earlyExits = reinterpret_cast<int32_t*>(P(I.oEarly));
  d.iterationsUsed = reinterpret_cast<int32_t*>(P(I.oIters));
  d.converged = reinterpret_cast<int32_t*>(P(I.oConv));
  return d;
}

constexpr int kMaxSmem = 200 * 1024;
constexpr int kBatchCluster = 4;                // CTAs per large cloth of a MIXED batch
constexpr int kBatchClusterMinVertices = 8192;  // "large"

// Status code of a preparation failure message.
int prepareCode(const std::string& err) {
  if (err.find("pivot") != std::string::npos) return PD_ERR_FACTORIZATION;
  if (err.find("precision") != std::string::npos) return PD_ERR_UNSUPPORTED;
  return PD_ERR_INVALID_ARGUMENT;
}

}  // namespace

// ------------------------------------------------------------------------------ sim handle
struct pd_sim {
  std::vector<Instance> inst;
  cudaStream_t stream = nullptr;
  uint8_t* dArena = nullptr;
  size_t arenaBytes = 0;
  pdg::InstanceDev* dDesc = nullptr;
  pdg::InstanceDev* dDescOrder = nullptr;  // batch descriptors by decreasing cost (correction kernel)
  double* dOmega = nullptr;                // over-relaxation weights of every instance
  size_t omegaCap = 0;
  bool traceOn = false;                    // record each iteration's gate residual
  double* dTrace = nullptr;                // per instance logCapacity × max_iterations
  size_t traceCap = 0, traceLen = 0;
  std::vector<size_t> traceOff;
  int32_t* dIterLog = nullptr;
  uint8_t* dConvLog = nullptr;
  int logCapacity = 0;
  int lastSubsteps = 0;
  int smemBytes = 0;
  int teamCtas = 1;  // CTAs per instance (a thread-block cluster when > 1)
  bool dense = false;  // mixed modes: the cluster applies the explicit FP32 inverse
  bool delta = false;  // MIXED: a team of co-resident CTAs per cloth, correction-form dense solve
  bool delta64 = false;  // FP64: the same team form, FP64 correction and double-float Ã⁻¹ product
  bool corr = false;   // MIXED above the dense limit: one CTA per cloth, correction-form FP32 solve
  int corrBig = 0;     // batch: instances (first in dDescOrder) run by clusters of kBatchCluster CTAs
  int workThreads = 0; // batch: > 0 runs it as a work table on resident CTAs of this many threads
  int* dCounter = nullptr;  // the work table's next-cloth counter
  cudaStream_t aux = nullptr;   // second stream: the batch's large cloths beside the small ones
  cudaEvent_t forkEv = nullptr, joinEv = nullptr;
  unsigned generation = 0;      // bumped whenever the arena, the descriptors or the plan change
  bool stageTiming = false;     // the substep kernels time their stages (StageTimes)
  double* dStage = nullptr;     // kStageCount ns accumulators per instance, kept across uploads
  pd_plan plan{};               // overrides of the planner's choices (pd_sim_set_plan / pd_sim_autotune)
  int bigCs = kBatchCluster;    // CTAs per large cloth of a MIXED batch on the second stream
  // host-state stepping (pd_sim_bind_host / pd_sim_step_host)
  std::vector<double*> hostX, hostV;          // the caller's arrays, 3n doubles each
  std::vector<pdg::HostStateDev> hostTable;   // device-visible addresses; empty unless all are page-locked
  pdg::HostStateDev* dHostTable = nullptr;
  unsigned tableGen = ~0u;
  int* hStatus = nullptr;                     // mapped host words: [0] non-finite input, [1] team error
  int* dStatus = nullptr;                     // their device-visible address
  cudaGraphExec_t graphExec = nullptr;        // gather → substeps → scatter, replayed per call
  int graphSubsteps = -1;
  unsigned graphGen = ~0u;
  cudaStream_t ownStream = nullptr;           // capture stream when the handle's stream is the default

  ~pd_sim() {
    release();
    if (aux) cudaStreamDestroy(aux);
    if (forkEv) cudaEventDestroy(forkEv);
    if (joinEv) cudaEventDestroy(joinEv);
    dropGraph();
    if (dHostTable) cudaFree(dHostTable);
    if (hStatus) cudaFreeHost(hStatus);
    if (dStage) cudaFree(dStage);
    if (ownStream) cudaStreamDestroy(ownStream);
    if (dCounter) cudaFree(dCounter);
  }
  void dropGraph() {
    if (graphExec) cudaGraphExecDestroy(graphExec);
    graphExec = nullptr;
    graphSubsteps = -1;
    graphGen = ~0u;
  }
  int precision() const { return inst.empty() ? PD_PRECISION_FP64_EXACT : inst[0].cfg.precision; }
  double latencyScale() const { return plan.latency_scale > 0.0 ? plan.latency_scale : 1.0; }
  // CTAs per cloth the caller asked for: the plan's, else the configuration's (0: the planner's)
  int wantCtas() const { return plan.team_ctas > 0 ? plan.team_ctas : inst[0].cfg.cluster_ctas; }

  // CTAs per cloth for the supernodal FP64 kernel: the requested count, or 16 for up to nine
  // cloths (152 SMs / 16) and fewer for larger batches; reduced until the device accepts it.
  // Mixed modes: every CTA of the cluster solves in its own shared memory, so a cluster needs
  // 72·n bytes of it per CTA.
  // Sets teamCtas and dense. CTAs per cloth: the requested count, or 16 for up to nine cloths
  // (152 SMs / 16) and fewer for larger batches, reduced until the device accepts it. Mixed modes
  // with a cluster apply the explicit FP32 inverse when every cloth is small enough; otherwise
  // every CTA of the cluster solves in its own shared memory (72·n bytes per CTA).
  void planTeam() {
    const int p = precision();
    teamCtas = 1;
    dense = false;
    delta = false;
    delta64 = false;
    corr = false;
    if (p == PD_PRECISION_FP64_EXACT) return;
    if (supernodalFp64(p) && planDelta64()) return;  // FP64, and FP32 projection with the FP64 solve
    for (auto& I : inst) {
      I.corrTeam = 1;
      I.corrThreads = pdg::kBlockThreads;
    }
    corrBig = 0;
    workThreads = 0;
    if (p == PD_PRECISION_MIXED) {
      if (!planDelta()) {
        corr = true;
        teamCtas = planCorr();
        if (teamCtas > 1) {
          for (auto& I : inst) I.corrTeam = teamCtas;
        } else if (inst.size() > 1 && plan.work_threads > pdg::kBlockThreads) {
          // the batch as a work table on resident CTAs of work_threads threads (no clusters)
          workThreads = plan.work_threads;
          for (auto& I : inst) I.corrThreads = workThreads;
        } else if (inst.size() > 1 && plan.big_min_vertices >= 0 &&
                   pdg::corrClusterSupported(bigCs = plan.big_cluster_ctas > 0 ? plan.big_cluster_ctas
                                                                               : kBatchCluster) == bigCs) {
          // a batch: the large cloths, whose one-CTA time would set the launch's makespan, get a
          // small cluster each and run on a second stream beside the others
          const int bigMin = plan.big_min_vertices > 0 ? plan.big_min_vertices : kBatchClusterMinVertices;
          for (auto& I : inst)
            if (I.scene.n >= bigMin) {
              I.corrTeam = bigCs;
              ++corrBig;
            }
          if (corrBig == static_cast<int>(inst.size())) {  // all large: one clustered launch
            teamCtas = bigCs;
            for (auto& I : inst) I.corrTeam = bigCs;
            corrBig = 0;
          }
        }
      }
      return;
    }
    int want = wantCtas();
    if (want <= 0) {
      const int count = static_cast<int>(inst.size());
      want = count <= 9 ? 16 : count <= 19 ? 8 : count <= 38 ? 4 : count <= 76 ? 2 : 1;
    }
    // one large cloth: a grid team, two CTAs an SM (a 256×256 FP64 cloth: 15.6 ms a substep on 304
    // CTAs against 97 ms on a 16-CTA cluster)
    if (!mixedSolve(p) && inst[0].cfg.cluster_ctas <= 0 && plan.team_ctas <= 0 && inst.size() == 1 &&
        inst[0].scene.n >= kBatchClusterMinVertices && pdg::gridCapacity() > 32)
      want = pdg::gridCapacity() / 2;
    if (!mixedSolve(p) && inst.size() == 1 && want > 16 && pdg::gridCapacity() > 16) {  // a grid team
      // its team-maximum slots (2 per CTA) live in the 3n-double workspace x0
      const int ctas = std::min({want, pdg::gridCapacity(), 3 * inst[0].scene.n / 2});
      if (ctas > 16) {
        teamCtas = ctas;
        return;
      }
      want = 16;
    }
    // FP32 solve of one cloth above the explicit-inverse limit: a grid team too (each CTA of a
    // cluster would hold the whole system in its shared memory, which a large cloth does not fit)
    if (p == PD_PRECISION_FP32_SOLVE && inst.size() == 1 && inst[0].scene.n > denseLimit() &&
        pdg::mixedGridCapacity() > 16) {
      if (inst[0].cfg.cluster_ctas <= 0 && plan.team_ctas <= 0 && inst[0].scene.n >= kBatchClusterMinVertices &&
          pdg::mixedGridCapacity() > 32)
        want = pdg::mixedGridCapacity() / 2;
      if (want > 16) {  // its team-maximum slots (2 per CTA) live in the 3n-double workspace x0
        const int ctas = std::min({want, pdg::mixedGridCapacity(), 3 * inst[0].scene.n / 2});
        if (ctas > 16) {
          teamCtas = ctas;
          return;
        }
        want = 16;
      }
    }
    int cs = 1;
    while (cs * 2 <= std::min(want, 16)) cs *= 2;
    if (!mixedSolve(p)) {
      while (cs > 1 && pdg::clusterSizeSupported(cs) != cs) cs /= 2;
      teamCtas = cs;
      return;
    }
    int maxN = 0;
    for (const auto& I : inst) maxN = std::max(maxN, I.scene.n);
    if (cs > 1 && maxN <= denseLimit()) {
      int d = cs;
      while (d > 1 && pdg::denseClusterSupported(d, denseSmem(maxN)) != d) d /= 2;
      if (d > 1) {
        teamCtas = d;
        dense = true;
        return;
      }
    }
    if (72 * maxN > kMaxSmem) return;
    while (cs > 1 && pdg::mixedClusterSupported(cs, 72 * maxN) != cs) cs /= 2;
    teamCtas = cs;
  }
  // MIXED with every cloth small enough for the explicit inverse: `cluster_ctas` CTAs per cloth
  // (0: the SMs shared out over the cloths), all co-resident, at most one per vertex.
  bool planDelta() {
    int maxN = 0, minN = 1 << 30;
    for (const auto& I : inst) {
      maxN = std::max(maxN, I.scene.n);
      minN = std::min(minN, I.scene.n);
    }
    if (maxN > denseLimit()) return false;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    const int count = static_cast<int>(inst.size());
    const int want = wantCtas();
    int team = want > 0 ? want : sms / count;
    team = std::min({team, sms / count, minN, 256});  // 256: partials one polling warp covers
    if (want <= 0 && count == 1) {  // the fewest CTAs with the same rows each: none is left without rows
      const int chunk = (maxN + team - 1) / team;
      team = (maxN + chunk - 1) / chunk;
    }
    if (team < 2) return false;
    int smem = 0, rows = 0;
    for (const auto& I : inst) smem = std::max(smem, deltaSmem(I, team, &rows));
    if (pdg::deltaResidentCtas(smem) < count * team) return false;
    teamCtas = team;
    delta = true;
    return true;
  }
  // FP64 with every cloth small enough for the explicit inverse and no over-relaxation: a team of
  // co-resident CTAs per cloth (the SMs shared out over the cloths, or a requested team of more than
  // 16 CTAs); a requested cluster of 1–16 CTAs keeps the supernodal kernel.
  bool planDelta64() {
    int maxN = 0, minN = 1 << 30;
    for (const auto& I : inst) {
      if (I.cfg.cheb_mode != PD_CHEB_OFF) return false;
      maxN = std::max(maxN, I.scene.n);
      minN = std::min(minN, I.scene.n);
    }
    if (maxN > denseLimit()) return false;
    const int want = wantCtas();
    if (want > 0 && want <= 16) return false;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    const int count = static_cast<int>(inst.size());
    int team = want > 0 ? want : sms / count;
    team = std::min({team, sms / count, minN, 256});  // 256: partials one polling warp covers
    if (want <= 0 && count == 1) {  // the fewest CTAs with the same rows each: none is left without rows
      const int chunk = (maxN + team - 1) / team;
      team = (maxN + chunk - 1) / chunk;
    }
    if (team < 2) return false;
    int smem = 0, rows = 0;
    for (const auto& I : inst) smem = std::max(smem, delta64Smem(I, team, &rows));
    if (pdg::delta64ResidentCtas(smem) < count * team) return false;
    teamCtas = team;
    delta64 = true;
    return true;
  }
  // CTAs per cloth of the correction kernel: a cluster for a few large cloths (as for the FP64
  // supernodal kernel), one CTA per cloth for batches and small cloths.
  int planCorr() const {
    int want = wantCtas();
    // one large cloth: a grid team of every CTA the device holds (a 256×256 cloth: 10.2 ms a
    // substep on 456 CTAs against 65.8 ms on a 16-CTA cluster)
    if (want <= 0 && inst.size() == 1 && inst[0].scene.n >= kBatchClusterMinVertices &&
        pdg::corrGridCapacity() > 16)
      want = pdg::corrGridCapacity();
    if (want > 16 && inst.size() == 1) {  // a grid team; its slots (2 per CTA) live in the 3n-double w
      const int ctas = std::min({want, pdg::corrGridCapacity(), 3 * inst[0].scene.n / 2});
      if (ctas > 16) return ctas;
      want = 16;
    }
    if (want <= 0) {
      int minN = 1 << 30;
      for (const auto& I : inst) minN = std::min(minN, I.scene.n);
      const int count = static_cast<int>(inst.size());
      want = minN < 4096 ? 1 : count <= 9 ? 16 : count <= 19 ? 8 : count <= 38 ? 4 : count <= 76 ? 2 : 1;
    }
    int cs = 1;
    while (cs * 2 <= std::min(want, 16)) cs *= 2;
    while (cs > 1 && pdg::corrClusterSupported(cs) != cs) cs /= 2;
    return cs;
  }
  // Largest cloth solved with the explicit inverse: the configured limit, capped by the
  // kernel's shared memory (denseSmem(n) ≤ kMaxSmem).
  int denseLimit() const {
    const int v = inst[0].cfg.dense_max_vertices;
    const int want = v == 0 ? PD_DENSE_DEFAULT_MAX_VERTICES : v;
    return want > 0 ? std::min(want, kMaxSmem / 60 / 32 * 32) : 0;
  }
  // dense-inverse kernel workspace: b and x₀ in FP64, three padded FP32 vectors
  static int denseSmem(int n) { return 48 * n + 12 * ((n + 31) / 32 * 32); }
  void release() {
    if (dArena) cudaFree(dArena);
    if (dDesc) cudaFree(dDesc);
    if (dDescOrder) cudaFree(dDescOrder);
    if (dOmega) cudaFree(dOmega);
    if (dTrace) cudaFree(dTrace);
    dTrace = nullptr;
    traceCap = traceLen = 0;
    if (dIterLog) cudaFree(dIterLog);
    if (dConvLog) cudaFree(dConvLog);
    dArena = nullptr;
    dDesc = nullptr;
    dDescOrder = nullptr;
    dOmega = nullptr;
    omegaCap = 0;
    dIterLog = nullptr;
    dConvLog = nullptr;
    logCapacity = 0;
  }

  int upload(int capacity) {
    Arena A;
    planTeam();
    for (auto& I : inst) layout(I, A, teamCtas, delta ? 2 : delta64 ? 4 : corr ? 3 : dense ? 1 : 0, latencyScale());
    release();
    if (workThreads > 0 && !dCounter) PD_CUDA(cudaMalloc(&dCounter, sizeof(int)));  // before any capture
    PD_CUDA(cudaMalloc(&dArena, A.host.size()));
    arenaBytes = A.host.size();
    PD_CUDA(cudaMemcpy(dArena, A.host.data(), A.host.size(), cudaMemcpyHostToDevice));
    const int rc = ensureLogs(capacity);
    if (rc != PD_OK) return rc;
    for (auto& I : inst)  // numeric refactorizations on the device, before anything reads the factor
      if (I.gpuRefactor)
        if (const int rc2 = refactorOnDevice(I)) {
          // the device factor is partly overwritten: lay the previous host factor out again, as a
          // failed host factorization leaves it, and let the next stamp change refactorize
          const std::string msg = g_lastError;
          for (auto& J : inst)
            if (J.gpuRefactor) {
              J.gpuRefactor = false;
              J.factorizeCount -= 1;
              J.stamp = pdg::Stamp{};
            }
          upload(capacity);
          g_lastError = msg;
          return rc2;
        }
    for (size_t i = 0; i < inst.size(); ++i) {  // explicit inverses from the uploaded FP64 factors
      if (inst[i].denseLd <= 0) continue;
      const int e = pdg::launchDenseInverse(dDesc + i, inst[i].scene.n, stream);
      if (e != 0) return cudaFail(static_cast<cudaError_t>(e), "explicit inverse launch");
    }
    PD_CUDA(cudaStreamSynchronize(stream));  // complete before a later stream change can race it
    return PD_OK;
  }

  // LDLᵀ values, block inverses and FP32 copies of instance I computed on the device from the
  // uploaded Ã (refactor.cu), then copied back into the host factor, which stays the reference
  // for later uploads and for pd_sim_get_factor.
  int refactorOnDevice(Instance& I) {
    pdg::Factor& F = I.F;
    auto P = [&](size_t off) { return dArena + off; };
    int* dStatus = nullptr;
    PD_CUDA(cudaMalloc(&dStatus, sizeof(int)));
    pdg::RefactorDev r{};
    r.n = F.n;
    r.maxRowLen = F.maxRowLen;
    r.nnz = static_cast<int64_t>(F.colval.size());
    r.nInv = static_cast<int64_t>(F.invL.size());
    r.colptr = reinterpret_cast<const int32_t*>(P(I.oLcp));
    r.rowidx = reinterpret_cast<const int32_t*>(P(I.oLri));
    r.colval = reinterpret_cast<double*>(P(I.oLcv));
    r.rowptr = reinterpret_cast<const int32_t*>(P(I.oLrp));
    r.colidx = reinterpret_cast<const int32_t*>(P(I.oLci));
    r.rowval = reinterpret_cast<double*>(P(I.oLrv));
    r.d = reinterpret_cast<double*>(P(I.oD));
    r.dinv = reinterpret_cast<double*>(P(I.oDinv));
    r.cscToCsr = reinterpret_cast<const int32_t*>(P(I.oCscToCsr));
    r.aPosCsc = reinterpret_cast<const int32_t*>(P(I.oAPosCsc));
    r.aPosDiag = reinterpret_cast<const int32_t*>(P(I.oAPosDiag));
    r.Aval = reinterpret_cast<const double*>(P(I.oAval));
    r.snStart = reinterpret_cast<const int32_t*>(P(I.oSnStart));
    r.rowSn = reinterpret_cast<const int32_t*>(P(I.oRowSn));
    r.offEnd = reinterpret_cast<const int32_t*>(P(I.oOffEnd));
    r.snInvOff = reinterpret_cast<const int64_t*>(P(I.oSnInv));
    r.invL = reinterpret_cast<double*>(P(I.oInvL));
    r.invLT = reinterpret_cast<double*>(P(I.oInvLT));
    r.rowval32 = reinterpret_cast<float*>(P(I.oLrv32));
    r.colval32 = reinterpret_cast<float*>(P(I.oLcv32));
    r.invL32 = reinterpret_cast<float*>(P(I.oInvL32));
    r.invLT32 = reinterpret_cast<float*>(P(I.oInvLT32));
    r.dinv32 = reinterpret_cast<float*>(P(I.oDinv32));
    r.status = dStatus;
    int status = 0;
    cudaError_t e = cudaMemsetAsync(dStatus, 0, sizeof(int), stream);
    const int levels = static_cast<int>(F.snLevelPtr.size()) - 1;
    const int ns = static_cast<int>(F.snStart.size()) - 1;
    int maxSn = 0;
    for (int t = 0; t < ns; ++t) maxSn = std::max(maxSn, F.snStart[t + 1] - F.snStart[t]);
    if (e == cudaSuccess)
      e = static_cast<cudaError_t>(pdg::launchRefactor(r, reinterpret_cast<const int32_t*>(P(I.oSnByLevel)),
                                                       F.snLevelPtr.data(),
                                                       reinterpret_cast<const int32_t*>(P(I.oLvlRows)),
                                                       F.lvlRowPtr.data(), levels, ns, maxSn, stream));
    if (e == cudaSuccess) e = cudaMemcpyAsync(&status, dStatus, sizeof(int), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    cudaFree(dStatus);
    if (e != cudaSuccess) return cudaFail(e, "device refactorization");
    if (status != 0)
      return fail(PD_ERR_FACTORIZATION, "LDL^T pivot " + std::to_string(status - 1) +
                                            " is zero or not finite: L is not positive definite");
    auto back = [&](auto& v, size_t off) {
      using T = typename std::decay_t<decltype(v)>::value_type;
      return cudaMemcpy(v.data(), P(off), v.size() * sizeof(T), cudaMemcpyDeviceToHost);
    };
    for (cudaError_t ee : {back(F.rowval, I.oLrv), back(F.colval, I.oLcv), back(F.d, I.oD), back(F.dinv, I.oDinv),
                           back(F.invL, I.oInvL), back(F.invLT, I.oInvLT), back(F.rowval32, I.oLrv32),
                           back(F.colval32, I.oLcv32), back(F.invL32, I.oInvL32), back(F.invLT32, I.oInvLT32),
                           back(F.dinv32, I.oDinv32)})
      if (ee != cudaSuccess) return cudaFail(ee, "copy of the device factor");
    I.gpuRefactor = false;
    I.deviceRefactorCount += 1;
    return PD_OK;
  }

  int ensureLogs(int capacity) {
    if (capacity <= logCapacity && dDesc) return PD_OK;
    if (dIterLog) cudaFree(dIterLog);
    if (dConvLog) cudaFree(dConvLog);
    dIterLog = nullptr;
    dConvLog = nullptr;
    const size_t count = inst.size();
    PD_CUDA(cudaMalloc(&dIterLog, sizeof(int32_t) * count * capacity));
    PD_CUDA(cudaMalloc(&dConvLog, count * capacity));
    PD_CUDA(cudaMemset(dIterLog, 0, sizeof(int32_t) * count * capacity));
    PD_CUDA(cudaMemset(dConvLog, 0, count * capacity));
    logCapacity = capacity;
    return writeDescriptors();
  }

  int writeDescriptors() {
    ++generation;
    std::vector<pdg::InstanceDev> desc;
    int smem = 0;
    // over-relaxation weights, one table per instance
    std::vector<double> weights;
    std::vector<size_t> wOff(inst.size());
    for (size_t i = 0; i < inst.size(); ++i) {
      wOff[i] = weights.size();
      const std::vector<double> w = chebWeights(inst[i].cfg);
      weights.insert(weights.end(), w.begin(), w.end());
    }
    if (weights.size() > omegaCap) {
      if (dOmega) cudaFree(dOmega);
      dOmega = nullptr;
      omegaCap = 0;
      PD_CUDA(cudaMalloc(&dOmega, sizeof(double) * weights.size()));
      omegaCap = weights.size();
    }
    if (!weights.empty())
      PD_CUDA(cudaMemcpy(dOmega, weights.data(), sizeof(double) * weights.size(), cudaMemcpyHostToDevice));
    // residual trace: logCapacity × max_iterations per instance
    traceOff.assign(inst.size() + 1, 0);
    for (size_t i = 0; i < inst.size(); ++i)
      traceOff[i + 1] = traceOff[i] + static_cast<size_t>(logCapacity) * std::max(1, inst[i].cfg.max_iterations);
    traceLen = traceOn ? traceOff.back() : 0;
    if (traceLen > traceCap) {
      if (dTrace) cudaFree(dTrace);
      dTrace = nullptr;
      traceCap = 0;
      PD_CUDA(cudaMalloc(&dTrace, sizeof(double) * traceLen));
      traceCap = traceLen;
    }
    for (size_t i = 0; i < inst.size(); ++i) {
      desc.push_back(describe(inst[i], dArena, dIterLog + i * logCapacity, dConvLog + i * logCapacity,
                              dOmega ? dOmega + wOff[i] : nullptr, traceOn ? dTrace + traceOff[i] : nullptr,
                              stageTiming ? dStage + pdg::kStageCount * i : nullptr));
      // exact: one 3n workspace; fast: two (RHS / solution and the level temporaries)
      int rows = 0;
      const int need = delta     ? deltaSmem(inst[i], teamCtas, &rows)
                       : delta64 ? delta64Smem(inst[i], teamCtas, &rows)
                       : dense ? denseSmem(inst[i].scene.n)
                       : corr  ? 24 * inst[i].scene.n
                               : workspaceBytesPerVertex(precision()) * inst[i].scene.n;
      // the correction kernel keeps its solve vectors in shared memory up to 48 KB, so that a
      // batch still runs four CTAs per SM
      const int cap = corr ? ((teamCtas > 1 || inst[i].corrTeam > 1) ? 0
                              : workThreads >= 1024       ? kMaxSmem       // one CTA an SM
                              : workThreads > 0           ? 100 * 1024     // two CTAs an SM
                                                          : 48 * 1024)
                           : kMaxSmem;
      if ((delta || delta64 || need <= cap) && need > smem) smem = need;
    }
    smemBytes = smem;
    if (!dDesc) PD_CUDA(cudaMalloc(&dDesc, sizeof(pdg::InstanceDev) * inst.size()));
    PD_CUDA(cudaMemcpy(dDesc, desc.data(), sizeof(pdg::InstanceDev) * desc.size(), cudaMemcpyHostToDevice));
    if (corr && inst.size() > 1) {  // launch order of the one-CTA kernel: most expensive first
      std::vector<size_t> order(inst.size());
      for (size_t i = 0; i < order.size(); ++i) order[i] = i;
      auto cost = [&](size_t i) {
        const Instance& I = inst[i];
        return static_cast<double>(I.F.colval.size()) + 8.0 * I.scene.edges.size() + 4.0 * I.scene.n;
      };
      std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        if (inst[a].corrTeam != inst[b].corrTeam) return inst[a].corrTeam > inst[b].corrTeam;  // clustered first
        return cost(a) > cost(b);
      });
      std::vector<pdg::InstanceDev> sorted;
      for (size_t i : order) sorted.push_back(desc[i]);
      if (!dDescOrder) PD_CUDA(cudaMalloc(&dDescOrder, sizeof(pdg::InstanceDev) * inst.size()));
      PD_CUDA(cudaMemcpy(dDescOrder, sorted.data(), sizeof(pdg::InstanceDev) * sorted.size(),
                         cudaMemcpyHostToDevice));
    } else if (dDescOrder) {
      cudaFree(dDescOrder);
      dDescOrder = nullptr;
    }
    return PD_OK;
  }

  // Copies device positions / velocities of every instance back into the host scenes.
  // Waits for the stream; a team barrier that gave up waiting is reported here (and the
  // barrier counters are reset so that later launches start clean).
  int sync() {
    PD_CUDA(cudaStreamSynchronize(stream));
    if (!delta && !delta64) return PD_OK;
    int bad = 0;
    for (const auto& I : inst) {
      int32_t e = 0;
      PD_CUDA(cudaMemcpy(&e, dArena + I.oErr, 4, cudaMemcpyDeviceToHost));
      bad |= e;
    }
    if (!bad) return PD_OK;
    for (const auto& I : inst) {
      PD_CUDA(cudaMemset(dArena + I.oErr, 0, 4));
      PD_CUDA(cudaMemset(dArena + I.oEpoch, 0, 4));
      PD_CUDA(cudaMemset(dArena + I.oPtag, 0, 8 * 3 * 16 * static_cast<size_t>(teamCtas)));
      PD_CUDA(cudaMemset(dArena + I.oRtag, 0, 8 * 2 * 3 * static_cast<size_t>(I.scene.n) * (delta64 ? 2 : 1)));
      PD_CUDA(cudaMemset(dArena + I.oXtag, 0, 8 * 6 * static_cast<size_t>(I.scene.n)));
    }
    return fail(PD_ERR_CUDA, "a team exchange of the substep kernel gave up waiting; the state is undefined");
  }

  int pullState() {
    if (const int rc_ = sync()) return rc_;
    for (auto& I : inst) {
      PD_CUDA(cudaMemcpy(I.scene.x.data(), dArena + I.oX, 24 * I.scene.n, cudaMemcpyDeviceToHost));
      PD_CUDA(cudaMemcpy(I.scene.v.data(), dArena + I.oV, 24 * I.scene.n, cudaMemcpyDeviceToHost));
    }
    return PD_OK;
  }

  // The second stream and its fork/join events, created before any launch (or capture) needs them.
  int ensureAux() {
    if (corrBig <= 0 || (aux && forkEv && joinEv)) return PD_OK;
    if (!aux) PD_CUDA(cudaStreamCreateWithFlags(&aux, cudaStreamNonBlocking));  // each kept once made
    if (!forkEv) PD_CUDA(cudaEventCreateWithFlags(&forkEv, cudaEventDisableTiming));
    if (!joinEv) PD_CUDA(cudaEventCreateWithFlags(&joinEv, cudaEventDisableTiming));
    return PD_OK;
  }

  // Queues `substeps` substeps of every instance on `st`: the residual-trace reset, then the
  // planned kernel (for a MIXED batch with large cloths: their clusters on the second stream
  // beside the one-CTA launch of the rest). Logs and the second stream must already exist.
  int launchSubsteps(cudaStream_t st, int substeps) {
    const int count = static_cast<int>(inst.size());
    if (traceOn && traceLen) PD_CUDA(cudaMemsetAsync(dTrace, 0xFF, sizeof(double) * traceLen, st));
    int rc;
    const int p = precision();
    if (p == PD_PRECISION_FP64_EXACT) {
      rc = pdg::launchSubstepExact(dDesc, count, substeps, smemBytes, st, stageTiming);
    } else if (delta) {
      rc = pdg::launchSubstepDelta(dDesc, count, teamCtas, smemBytes, substeps, st, stageTiming);
    } else if (delta64) {
      rc = pdg::launchSubstepDelta64(dDesc, count, teamCtas, smemBytes, substeps, st, stageTiming);
    } else if (corr) {
      if (teamCtas > 16) {  // one cloth on a cooperative grid of CTAs
        rc = pdg::launchSubstepCorrGrid(dDesc, teamCtas, substeps, st, stageTiming);
      } else if (teamCtas > 1) {
        rc = pdg::launchSubstepCorrCluster(dDesc, count, teamCtas, substeps, st, stageTiming);
      } else if (workThreads > 0) {
        rc = pdg::launchSubstepCorrWork(dDescOrder ? dDescOrder : dDesc, count, dCounter, workThreads, substeps,
                                        smemBytes, st, stageTiming);
      } else if (corrBig > 0) {
        // the one-CTA launch of the smaller cloths on this stream, submitted first, then the large
        // cloths' clusters on the second stream behind an event wait: the one-CTA cloths take
        // their slots first and finish early while the clusters fill in behind them. With the
        // clusters dispatched first the batch needs more than one wave of them before the rest
        // start (512-cloth batch: 35.0 against 29.4 ms per substep).
        PD_CUDA(cudaEventRecord(forkEv, st));
        rc = pdg::launchSubstepCorr(dDescOrder + corrBig, count - corrBig, substeps, smemBytes, st, stageTiming);
        if (rc == 0) {
          PD_CUDA(cudaStreamWaitEvent(aux, forkEv, 0));
          rc = pdg::launchSubstepCorrCluster(dDescOrder, corrBig, bigCs, substeps, aux, stageTiming);
        }
        if (rc == 0) {
          PD_CUDA(cudaEventRecord(joinEv, aux));
          PD_CUDA(cudaStreamWaitEvent(st, joinEv, 0));
        }
      } else {
        rc = pdg::launchSubstepCorr(dDescOrder ? dDescOrder : dDesc, count, substeps, smemBytes, st, stageTiming);
      }
    } else if (dense) {
      rc = pdg::launchSubstepDenseCluster(dDesc, count, teamCtas, smemBytes, substeps, st);
    } else if (mixedSolve(p)) {
      rc = teamCtas > 16  ? pdg::launchSubstepMixedGrid(dDesc, teamCtas, substeps, st, stageTiming)
           : teamCtas > 1 ? pdg::launchSubstepMixedCluster(dDesc, count, teamCtas, smemBytes, substeps, st)
                          : pdg::launchSubstepMixed(dDesc, count, substeps, smemBytes, st);
    } else {
      rc = teamCtas > 16  ? pdg::launchSubstepGrid(dDesc, teamCtas, substeps, st, stageTiming)
           : teamCtas > 1 ? pdg::launchSubstepCluster(dDesc, count, teamCtas, substeps, st, stageTiming)
                          : pdg::launchSubstepFast(dDesc, count, substeps, smemBytes, st, stageTiming);
    }
    if (rc != 0) return cudaFail(static_cast<cudaError_t>(rc), "substep launch");
    return PD_OK;
  }

  // Records gather → substeps → scatter on `st` as a CUDA graph.
  int captureHostStep(cudaStream_t st, int substeps) {
    dropGraph();
    const int count = static_cast<int>(inst.size());
    int maxN = 1;
    for (const auto& I : inst) maxN = std::max(maxN, I.scene.n);
    PD_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int rc = PD_OK;
    cudaError_t e = static_cast<cudaError_t>(pdg::launchGatherState(dHostTable, count, maxN, dStatus, st));
    if (e == cudaSuccess && substeps > 0) rc = launchSubsteps(st, substeps);
    if (e == cudaSuccess && rc == PD_OK)
      e = static_cast<cudaError_t>(pdg::launchScatterState(dHostTable, count, maxN, dStatus, st));
    cudaGraph_t g = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(st, &g);
    if (rc == PD_OK && (e != cudaSuccess || ee != cudaSuccess))
      rc = cudaFail(e != cudaSuccess ? e : ee, "capture of the host-state step");
    if (rc == PD_OK) {
      e = cudaGraphInstantiate(&graphExec, g, 0);
      if (e != cudaSuccess) {
        graphExec = nullptr;
        rc = cudaFail(e, "cudaGraphInstantiate of the host-state step");
      }
    }
    if (g) cudaGraphDestroy(g);
    if (rc != PD_OK) return rc;
    graphSubsteps = substeps;
    graphGen = generation;
    return PD_OK;
  }
};

// ------------------------------------------------------------------------------ solver handle
struct pd_solver {
  int32_t n3 = 0;           // size of the 3n system
  bool analyzedFlag = false;
  bool ready = false;
  std::vector<int32_t> pattern_cp, pattern_ri;
  pdg::ScalarMatrix A;
  pdg::Factor F;
  std::vector<int32_t> perm;
  uint8_t* dArena = nullptr;
  pdg::InstanceDev* dDesc = nullptr;
  double* dB = nullptr;
  double* dX = nullptr;
  cudaStream_t stream = nullptr;
  pd_solver_stats stats{};
  // per-component slots of solveComponent (IGlobalSolver.h:94-97: the three components may be
  // solved from three threads at once): component c owns dCol[3m·c, 3m·(c+1)) on the device
  // (b, x, workspace), hCol[2m·c, 2m·(c+1)) in page-locked host memory (b, x) and colStream[c]
  double* dCol = nullptr;
  double* hCol = nullptr;
  size_t colM = 0;
  cudaStream_t colStream[3] = {nullptr, nullptr, nullptr};
  void releaseColumns() {
    if (dCol) cudaFree(dCol);
    if (hCol) cudaFreeHost(hCol);
    dCol = nullptr;
    hCol = nullptr;
    colM = 0;
  }
  ~pd_solver() {
    if (dArena) cudaFree(dArena);
    if (dDesc) cudaFree(dDesc);
    if (dB) cudaFree(dB);  // dX points into the same allocation
    releaseColumns();
    for (cudaStream_t& st : colStream)
      if (st) cudaStreamDestroy(st);
  }
};

namespace {

// Extracts the scalar matrix Ã from a 3n × 3n CSC matrix with L = Ã ⊗ I₃; returns "" on success.
std::string scalarFromBlocks(int32_t n3, const int32_t* cp, const int32_t* ri, const double* val,
                             pdg::ScalarMatrix& A) {
  if (n3 <= 0 || n3 % 3 != 0) return "dimension is not a multiple of 3";
  const int n = n3 / 3;
  // collect entries (r, c, v) of component 0 and check the other components mirror them
  std::vector<std::vector<std::pair<int, double>>> rows(n);
  std::vector<std::vector<std::pair<int, double>>> comp[3];
  for (int k = 0; k < 3; ++k) comp[k].assign(n, {});
  for (int c = 0; c < n3; ++c)
    for (int p = cp[c]; p < cp[c + 1]; ++p) {
      const int r = ri[p];
      if (r < 0 || r >= n3) return "row index out of range";
      if (r % 3 != c % 3) return "matrix couples different x/y/z components";
      comp[c % 3][r / 3].push_back({c / 3, val ? val[p] : 0.0});
    }
  for (int k = 0; k < 3; ++k)
    for (auto& row : comp[k]) std::sort(row.begin(), row.end(), [](auto& a, auto& b) { return a.first < b.first; });
  for (int r = 0; r < n; ++r)
    for (int k = 1; k < 3; ++k) {
      if (comp[k][r].size() != comp[0][r].size()) return "components have different sparsity";
      for (size_t t = 0; t < comp[0][r].size(); ++t) {
        if (comp[k][r][t].first != comp[0][r][t].first) return "components have different sparsity";
        if (val && std::memcmp(&comp[k][r][t].second, &comp[0][r][t].second, sizeof(double)) != 0)
          return "components have different values (not a scalar times I3 per block)";
      }
    }
  // symmetrize the pattern from the lower triangle (Eigen's selfadjointView<Lower>)
  std::vector<std::vector<std::pair<int, double>>> sym(n);
  for (int r = 0; r < n; ++r)
    for (auto& e : comp[0][r])
      if (e.first <= r) {
        sym[r].push_back({e.first, e.second});
        if (e.first != r) sym[e.first].push_back({r, e.second});
      }
  A.n = n;
  A.rowptr.assign(n + 1, 0);
  A.col.clear();
  A.val.clear();
  for (int r = 0; r < n; ++r) {
    std::sort(sym[r].begin(), sym[r].end(), [](auto& a, auto& b) { return a.first < b.first; });
    for (auto& e : sym[r]) {
      A.col.push_back(e.first);
      A.val.push_back(e.second);
    }
    A.rowptr[r + 1] = static_cast<int32_t>(A.col.size());
  }
  return {};
}

// Minimum-degree ordering of a scalar pattern (ties → lower index); used when no geometry exists.
std::vector<int32_t> minimumDegreeOrder(const pdg::ScalarMatrix& A) {
  const int n = A.n;
  std::vector<std::vector<int>> adj(n);
  for (int r = 0; r < n; ++r)
    for (int p = A.rowptr[r]; p < A.rowptr[r + 1]; ++p)
      if (A.col[p] != r) adj[r].push_back(A.col[p]);
  for (auto& a : adj) {
    std::sort(a.begin(), a.end());
    a.erase(std::unique(a.begin(), a.end()), a.end());
  }
  std::vector<std::pair<int, int>> heap;
  std::vector<int> deg(n);
  std::vector<uint8_t> done(n, 0);
  for (int v = 0; v < n; ++v) deg[v] = static_cast<int>(adj[v].size());
  std::vector<int32_t> order;
  std::vector<int> merged;
  auto better = [&](int a, int b) { return deg[a] != deg[b] ? deg[a] < deg[b] : a < b; };
  for (int step = 0; step < n; ++step) {
    int best = -1;
    for (int v = 0; v < n; ++v)
      if (!done[v] && (best < 0 || better(v, best))) best = v;
    done[best] = 1;
    order.push_back(best);
    const std::vector<int> nb = adj[best];
    for (int u : nb) {
      merged.clear();
      std::set_union(adj[u].begin(), adj[u].end(), nb.begin(), nb.end(), std::back_inserter(merged));
      adj[u].clear();
      for (int w : merged)
        if (w != u && w != best && !done[w]) adj[u].push_back(w);
      deg[u] = static_cast<int>(adj[u].size());
    }
    adj[best].clear();
  }
  return order;
}

}  // namespace

// ====================================================================================== C API
extern "C" {

const char* pd_last_error(void) { return g_lastError.c_str(); }

void pd_scene_config_default(pd_scene_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->dt = 1.0 / 120.0;
  c->substeps_per_frame = 2;
  c->gravity[1] = -9.81;
  c->stiffness = 2.3e3;
  c->density = 1.0;
  c->velocity_damping = 0.02;
  c->max_iterations = 10;
  c->rel_tolerance = 1.0e-3;
  c->abs_tolerance = 1.0e-12;
  c->residual_tolerance = 1.0e-3;
  c->grid_nx = 40;
  c->grid_ny = 40;
  c->grid_spacing = 0.025;
  c->bend_stride = 1;
  c->total_mass = 1.0;
  c->precision = PD_PRECISION_FP64_EXACT;
  c->cheb_mode = PD_CHEB_OFF;
  c->cheb_rho = 0.98;
  c->cheb_start = 10;
  c->cheb_m = 1.0;
  c->cheb_d = 1.0;
}

int pd_grid_counts(const pd_scene_config* cfg, int32_t* nv, int32_t* ne, int32_t* nb) {
  if (!cfg || !nv || !ne || !nb) return fail(PD_ERR_INVALID_ARGUMENT, "null argument");
  int a, b, c;
  if (!pdg::gridCounts(gridSpecOf(*cfg), &a, &b, &c)) return fail(PD_ERR_INVALID_ARGUMENT, "grid needs nx, ny >= 2");
  *nv = a;
  *ne = b;
  *nb = c;
  return PD_OK;
}

int pd_make_grid(const pd_scene_config* cfg, double* pos, double* mass, uint8_t* pinned, int32_t* edges,
                 double* rest, double* k, int32_t* bends, double* bk) {
  if (!cfg || !pos || !mass || !pinned || !edges || !rest || !k) return fail(PD_ERR_INVALID_ARGUMENT, "null argument");
  pdg::Scene s;
  if (!pdg::makeGrid(gridSpecOf(*cfg), s)) return fail(PD_ERR_INVALID_ARGUMENT, "grid needs nx, ny >= 2");
  if (!s.bends.empty() && (!bends || !bk)) return fail(PD_ERR_INVALID_ARGUMENT, "bend arrays are null");
  std::memcpy(pos, s.x.data(), s.x.size() * sizeof(double));
  std::memcpy(mass, s.m.data(), s.m.size() * sizeof(double));
  std::memcpy(pinned, s.pinned.data(), s.pinned.size());
  for (size_t e = 0; e < s.edges.size(); ++e) {
    edges[2 * e] = s.edges[e].a;
    edges[2 * e + 1] = s.edges[e].b;
    rest[e] = s.edges[e].rest;
    k[e] = s.edges[e].k;
  }
  for (size_t b = 0; b < s.bends.size(); ++b) {
    bends[3 * b] = s.bends[b].a;
    bends[3 * b + 1] = s.bends[b].b;
    bends[3 * b + 2] = s.bends[b].c;
    bk[b] = s.bends[b].k;
  }
  return PD_OK;
}

int pd_obj_counts(const char* obj_text, int32_t* n_vertices, int32_t* n_edges) {
  if (!obj_text || !n_vertices || !n_edges) return fail(PD_ERR_INVALID_ARGUMENT, "null argument");
  pdg::Scene s;
  std::string err;
  if (!pdg::makeObj(obj_text, 1.0, 1.0, s, &err)) return fail(PD_ERR_INVALID_ARGUMENT, "OBJ: " + err);
  *n_vertices = s.n;
  *n_edges = static_cast<int32_t>(s.edges.size());
  return PD_OK;
}

int pd_make_obj(const pd_scene_config* cfg, const char* obj_text, double* pos, double* mass, uint8_t* pinned,
                int32_t* edges, double* rest, double* k) {
  if (!cfg || !obj_text || !pos || !mass || !pinned || !edges || !rest || !k)
    return fail(PD_ERR_INVALID_ARGUMENT, "null argument");
  pdg::Scene s;
  std::string err;
  if (!pdg::makeObj(obj_text, cfg->stiffness, cfg->density, s, &err)) return fail(PD_ERR_INVALID_ARGUMENT, "OBJ: " + err);
  std::memcpy(pos, s.x.data(), s.x.size() * sizeof(double));
  std::memcpy(mass, s.m.data(), s.m.size() * sizeof(double));
  std::memcpy(pinned, s.pinned.data(), s.pinned.size());
  for (size_t e = 0; e < s.edges.size(); ++e) {
    edges[2 * e] = s.edges[e].a;
    edges[2 * e + 1] = s.edges[e].b;
    rest[e] = s.edges[e].rest;
    k[e] = s.edges[e].k;
  }
  return PD_OK;
}

// ---------------------------------------------------------------------------------- sim
static int sceneFromMesh(const pd_mesh& m, pdg::Scene& s) {
  if (m.n_vertices <= 0 || !m.positions || !m.masses || !m.pinned)
    return fail(PD_ERR_INVALID_ARGUMENT, "mesh needs vertices, positions, masses and pin flags");
  if (m.n_edges < 0 || m.n_bends < 0) return fail(PD_ERR_INVALID_ARGUMENT, "negative edge or bend count");
  if (m.n_edges > 0 && (!m.edges || !m.edge_rest || !m.edge_stiffness))
    return fail(PD_ERR_INVALID_ARGUMENT, "edge arrays are null");
  if (m.n_bends > 0 && (!m.bends || !m.bend_stiffness)) return fail(PD_ERR_INVALID_ARGUMENT, "bend arrays are null");
  const size_t n = m.n_vertices;
  s = pdg::Scene{};
  s.n = m.n_vertices;
  s.x.assign(m.positions, m.positions + 3 * n);
  if (m.velocities) s.v.assign(m.velocities, m.velocities + 3 * n);
  else s.v.assign(3 * n, 0.0);
  s.m.assign(m.masses, m.masses + n);
  s.pinned.assign(m.pinned, m.pinned + n);
  for (auto& p : s.pinned) p = p ? 1 : 0;
  if (m.pin_positions) s.q.assign(m.pin_positions, m.pin_positions + 3 * n);
  else s.q = s.x;
  for (int e = 0; e < m.n_edges; ++e)
    s.edges.push_back(pdg::Edge{m.edges[2 * e], m.edges[2 * e + 1], m.edge_rest[e], m.edge_stiffness[e]});
  for (int b = 0; b < m.n_bends; ++b)
    s.bends.push_back(pdg::Bend{m.bends[3 * b], m.bends[3 * b + 1], m.bends[3 * b + 2], m.bend_stiffness[b]});
  return PD_OK;
}

int pd_sim_create_batch(int32_t count, const pd_mesh* meshes, const pd_scene_config* cfgs, pd_sim** out) {
  if (!out) return fail(PD_ERR_INVALID_ARGUMENT, "out is null");
  *out = nullptr;
  if (count <= 0 || !meshes || !cfgs) return fail(PD_ERR_INVALID_ARGUMENT, "empty batch");
  auto sim = std::make_unique<pd_sim>();
  sim->inst.resize(count);
  for (int i = 0; i < count; ++i) {
    Instance& I = sim->inst[i];
    I.cfg = cfgs[i];
    if (cfgs[i].precision != cfgs[0].precision)
      return fail(PD_ERR_INVALID_ARGUMENT, "all instances of a batch must use one precision mode");
    int rc = sceneFromMesh(meshes[i], I.scene);
    if (rc != PD_OK) return rc;
    std::string err = pdg::validateScene(I.scene);
    if (!err.empty()) return fail(PD_ERR_INVALID_ARGUMENT, "instance " + std::to_string(i) + ": " + err);
    pdg::buildTopology(I.scene, I.topo);
    const auto t0 = Clock::now();
    err = prepare(I, true);
    I.assembleSeconds = secondsSince(t0);
    if (!err.empty()) {
      return fail(prepareCode(err), "instance " + std::to_string(i) + ": " + err);
    }
  }
  const int rc = sim->upload(1);
  if (rc != PD_OK) return rc;
  *out = sim.release();
  return PD_OK;
}

int pd_sim_create(const pd_mesh* mesh, const pd_scene_config* cfg, pd_sim** out) {
  if (!mesh || !cfg) return fail(PD_ERR_INVALID_ARGUMENT, "null argument");
  return pd_sim_create_batch(1, mesh, cfg, out);
}

int pd_sim_destroy(pd_sim* s) {
  delete s;
  return PD_OK;
}

int pd_sim_instance_count(const pd_sim* s) { return s ? static_cast<int>(s->inst.size()) : 0; }

int pd_sim_set_stream(pd_sim* s, void* stream) {
  if (!s) return fail(PD_ERR_INVALID_ARGUMENT, "null handle");
  s->stream = static_cast<cudaStream_t>(stream);
  return PD_OK;
}

int pd_sim_step(pd_sim* s, int32_t substeps) {
  if (!s) return fail(PD_ERR_INVALID_ARGUMENT, "null handle");
  if (substeps < 0) return fail(PD_ERR_INVALID_ARGUMENT, "substeps must be >= 0");
  if (substeps == 0) return PD_OK;
  if (substeps > s->logCapacity) {
    if (const int rc_ = s->sync()) return rc_;
    const int rc = s->ensureLogs(substeps);
    if (rc != PD_OK) return rc;
  }
  int rc = s->ensureAux();
  if (rc == PD_OK) rc = s->launchSubsteps(s->stream, substeps);
  if (rc != PD_OK) return rc;
  s->lastSubsteps = substeps;
  return PD_OK;
}

int pd_sim_synchronize(pd_sim* s) {
  if (!s) return fail(PD_ERR_INVALID_ARGUMENT, "null handle");
  if (const int rc_ = s->sync()) return rc_;
  return PD_OK;
}

static int checkInstance(pd_sim* s, int32_t i) {
  if (!s) return fail(PD_ERR_INVALID_ARGUMENT, "null handle");
  if (i < 0 || i >= static_cast<int>(s->inst.size())) return fail(PD_ERR_INVALID_ARGUMENT, "instance index out of range");
  return PD_OK;
}

int pd_sim_get_state(pd_sim* s, int32_t i, double* x, double* v) {
  int rc = checkInstance(s, i);
  if (rc) return rc;
  const Instance& I = s->inst[i];
  const size_t bytes = 24 * static_cast<size_t>(I.scene.n);
  if (x) PD_CUDA(cudaMemcpyAsync(x, s->dArena + I.oX, bytes, cudaMemcpyDeviceToHost, s->stream));
  if (v) PD_CUDA(cudaMemcpyAsync(v, s->dArena + I.oV, bytes, cudaMemcpyDeviceToHost, s->stream));
  if (const int rc_ = s->sync()) return rc_;
  return PD_OK;
}

int pd_sim_set_state(pd_sim* s, int32_t i, const double* x, const double* v) {
  int rc = checkInstance(s, i);
  if (rc) return rc;
  Instance& I = s->inst[i];
  const size_t bytes = 24 * static_cast<size_t>(I.scene.n);
  if (x) {
    for (size_t k = 0; k < 3 * static_cast<size_t>(I.scene.n); ++k)
      if (!std::isfinite(x[k])) return fail(PD_ERR_INVALID_ARGUMENT, "positions contain a non-finite value");
    PD_CUDA(cudaMemcpyAsync(s->dArena + I.oX, x, bytes, cudaMemcpyHostToDevice, s->stream));
  }
  if (v) PD_CUDA(cudaMemcpyAsync(s->dArena + I.oV, v, bytes, cudaMemcpyHostToDevice, s->stream));
  return PD_OK;
}

// Device-visible address of `count` doubles at host address p if the whole range lies in one
// page-locked (cudaHostAlloc / cudaHostRegister) allocation, else null.
static double* mappedHost(double* p, size_t count) {
  cudaPointerAttributes a{}, b{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
  double* last = p + (count - 1);
  if (cudaPointerGetAttributes(&b, last) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  double* d = static_cast<double*>(a.devicePointer);
  if (b.type != cudaMemoryTypeHost || static_cast<double*>(b.devicePointer) != d + (count - 1)) return nullptr;
  return d;
}

int pd_sim_bind_host(pd_sim* s, double* const* x, double* const* v) {
  if (!s) return fail(PD_ERR_INVALID_ARGUMENT, "null handle");
  if (const int rc_ = s->sync()) return rc_;  // no launch in flight still reads the old arrays
  s->dropGraph();
  s->hostX.clear();
  s->hostV.clear();
  s->hostTable.clear();
  s->tableGen = ~0u;
  if (!x && !v) return PD_OK;  // unbind
  if (!x || !v) return fail(PD_ERR_INVALID_ARGUMENT, "positions and velocities must both be given");
  const size_t count = s->inst.size();
  for (size_t i = 0; i < count; ++i)
    if (!x[i] || !v[i]) return fail(PD_ERR_INVALID_ARGUMENT, "instance " + std::to_string(i) + ": null array");
  std::vector<pdg::HostStateDev> table(count);
  bool mapped = count <= 65535;
  for (size_t i = 0; i < count && mapped; ++i) {
    const size_t n3 = 3 * static_cast<size_t>(s->inst[i].scene.n);
    table[i].hx = mappedHost(x[i], n3);
    table[i].hv = mappedHost(v[i], n3);
    table[i].n = s->inst[i].scene.n;
    mapped = table[i].hx && table[i].hv;
  }
  s->hostX.assign(x, x + count);
  s->hostV.assign(v, v + count);
  if (mapped) s->hostTable = std::move(table);
  return PD_OK;
}

int pd_sim_step_host(pd_sim* s, int32_t substeps) {
  if (!s) return fail(PD_ERR_INVALID_ARGUMENT, "null handle");
  if (substeps < 0) return fail(PD_ERR_INVALID_ARGUMENT, "substeps must be >= 0");
  if (s->hostX.empty()) return fail(PD_ERR_STATE, "no host arrays are bound (pd_sim_bind_host)");
  if (substeps > s->logCapacity) {
    if (const int rc_ = s->sync()) return rc_;
    const int rc = s->ensureLogs(substeps);
    if (rc != PD_OK) return rc;
  }
  if (const int rc = s->ensureAux()) return rc;
  const size_t count = s->inst.size();
  if (s->hostTable.empty()) {  // pageable arrays: one copy per array each way
    for (size_t i = 0; i < count; ++i) {
      const size_t n3 = 3 * static_cast<size_t>(s->inst[i].scene.n);
      for (size_t k = 0; k < n3; ++k)
        if (!std::isfinite(s->hostX[i][k])) return fail(PD_ERR_INVALID_ARGUMENT, "positions contain a non-finite value");
    }
    for (size_t i = 0; i < count; ++i) {
      const Instance& I = s->inst[i];
      const size_t bytes = 24 * static_cast<size_t>(I.scene.n);
      PD_CUDA(cudaMemcpyAsync(s->dArena + I.oX, s->hostX[i], bytes, cudaMemcpyHostToDevice, s->stream));
      PD_CUDA(cudaMemcpyAsync(s->dArena + I.oV, s->hostV[i], bytes, cudaMemcpyHostToDevice, s->stream));
    }
    if (substeps > 0) {
      if (const int rc = s->launchSubsteps(s->stream, substeps)) return rc;
      s->lastSubsteps = substeps;
    }
    for (size_t i = 0; i < count; ++i) {
      const Instance& I = s->inst[i];
      const size_t bytes = 24 * static_cast<size_t>(I.scene.n);
      PD_CUDA(cudaMemcpyAsync(s->hostX[i], s->dArena + I.oX, bytes, cudaMemcpyDeviceToHost, s->stream));
      PD_CUDA(cudaMemcpyAsync(s->hostV[i], s->dArena + I.oV, bytes, cudaMemcpyDeviceToHost, s->stream));
    }
    return s->sync();
  }
  // page-locked arrays: gather kernel → substeps → scatter kernel, one CUDA graph replay
  cudaStream_t st = s->stream;
  if (!st) {  // a graph cannot be captured on the legacy default stream
    if (!s->ownStream) PD_CUDA(cudaStreamCreate(&s->ownStream));
    st = s->ownStream;
  }
  if (s->tableGen != s->generation) {
    for (size_t i = 0; i < count; ++i) {
      s->hostTable[i].dx = reinterpret_cast<double*>(s->dArena + s->inst[i].oX);
      s->hostTable[i].dv = reinterpret_cast<double*>(s->dArena + s->inst[i].oV);
      s->hostTable[i].err = (s->delta || s->delta64) ? reinterpret_cast<const int32_t*>(s->dArena + s->inst[i].oErr)
                                                      : nullptr;
    }
    if (!s->dHostTable) PD_CUDA(cudaMalloc(&s->dHostTable, sizeof(pdg::HostStateDev) * count));
    PD_CUDA(cudaMemcpy(s->dHostTable, s->hostTable.data(), sizeof(pdg::HostStateDev) * count,
                       cudaMemcpyHostToDevice));
    s->tableGen = s->generation;
  }
  if (!s->hStatus) {
    PD_CUDA(cudaHostAlloc(&s->hStatus, 2 * sizeof(int), cudaHostAllocMapped));
    PD_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void**>(&s->dStatus), s->hStatus, 0));
  }
  if (!s->graphExec || s->graphSubsteps != substeps || s->graphGen != s->generation)
    if (const int rc = s->captureHostStep(st, substeps)) return rc;
  volatile int* status = s->hStatus;
  status[0] = status[1] = 0;
  PD_CUDA(cudaGraphLaunch(s->graphExec, st));
  if (substeps > 0) s->lastSubsteps = substeps;
  PD_CUDA(cudaStreamSynchronize(st));
  if (status[1])  // a team exchange gave up: report it and reset the exchange words
    if (const int rc_ = s->sync()) return rc_;
  if (status[0])
    return fail(PD_ERR_INVALID_ARGUMENT, "a bound position array holds a non-finite value (the step ran on it)");
  return PD_OK;
}

int pd_sim_device_state(pd_sim* s, int32_t i, double** x, double** v) {
  int rc = checkInstance(s, i);
  if (rc) return rc;
  if (x) *x = reinterpret_cast<double*>(s->dArena + s->inst[i].oX);
  if (v) *v = reinterpret_cast<double*>(s->dArena + s->inst[i].oV);
  return PD_OK;
}

// Rebuilds host preparation of instance i after a change and re-uploads the handle.
static int rebuild(pd_sim* s, int i, bool reanalyze) {
  int rc = s->pullState();
  if (rc) return rc;
  Instance& I = s->inst[i];
  const auto t0 = Clock::now();
  const std::string err = prepare(I, reanalyze);
  if (!err.empty()) return fail(prepareCode(err), err);
  rc = s->upload(s->logCapacity > 0 ? s->logCapacity : 1);
  I.assembleSeconds += secondsSince(t0);
  return rc;
}

int pd_sim_set_pin_positions(pd_sim* s, int32_t i, const double* q) {
  int rc = checkInstance(s, i);
  if (rc) return rc;
  if (!q) return fail(PD_ERR_INVALID_ARGUMENT, "null pin positions");
  Instance& I = s->inst[i];
  I.scene.q.assign(q, q + 3 * static_cast<size_t>(I.scene.n));
  pdg::assembleBendingRhs(I.scene, I.bendRhs);
  PD_CUDA(cudaMemcpyAsync(s->dArena + I.oQ, I.scene.q.data(), 24 * static_cast<size_t>(I.scene.n), cudaMemcpyHostToDevice, s->stream));
  PD_CUDA(cudaMemcpyAsync(s->dArena + I.oBend, I.bendRhs.data(), 24 * static_cast<size_t>(I.scene.n), cudaMemcpyHostToDevice, s->stream));
  std::vector<float> pairs;
  if (I.oQhl) {
    pairs = pinPairs(I.scene);
    PD_CUDA(cudaMemcpyAsync(s->dArena + I.oQhl, pairs.data(), 4 * pairs.size(), cudaMemcpyHostToDevice, s->stream));
  }
  if (const int rc_ = s->sync()) return rc_;
  return PD_OK;
}

int pd_sim_set_edge_stiffness(pd_sim* s, int32_t i, const double* k) {
  int rc = checkInstance(s, i);
  if (rc) return rc;
  if (!k) return fail(PD_ERR_INVALID_ARGUMENT, "null stiffness");
  Instance& I = s->inst[i];
  for (size_t e = 0; e < I.scene.edges.size(); ++e) I.scene.edges[e].k = k[e];
  if (pdg::computeStamp(I.scene, I.cfg.dt).k == I.stamp.k) return PD_OK;  // L unchanged
  return rebuild(s, i, false);
}

int pd_sim_set_pinned(pd_sim* s, int32_t i, const uint8_t* pinned, const double* q) {
  int rc = checkInstance(s, i);
  if (rc) return rc;
  if (!pinned) return fail(PD_ERR_INVALID_ARGUMENT, "null pin mask");
  rc = s->pullState();
  if (rc) return rc;
  Instance& I = s->inst[i];
  for (int v = 0; v < I.scene.n; ++v) I.scene.pinned[v] = pinned[v] ? 1 : 0;
  if (q) I.scene.q.assign(q, q + 3 * static_cast<size_t>(I.scene.n));
  else
    for (int v = 0; v < I.scene.n; ++v)
      if (I.scene.pinned[v])
        for (int c = 0; c < 3; ++c) I.scene.q[3 * v + c] = I.scene.x[3 * v + c];
  const pdg::Stamp now = pdg::computeStamp(I.scene, I.cfg.dt);
  if (now.pin == I.stamp.pin && now.structure == I.stamp.structure) {
    pdg::assembleBendingRhs(I.scene, I.bendRhs);
    return s->upload(s->logCapacity);
  }
  return rebuild(s, i, now.structure != I.stamp.structure);
}

int pd_sim_set_config(pd_sim* s, const pd_scene_config* cfg) {
  if (!s || !cfg) return fail(PD_ERR_INVALID_ARGUMENT, "null argument");
  if (!(cfg->dt > 0.0) || cfg->max_iterations < 0) return fail(PD_ERR_INVALID_ARGUMENT, "invalid dt or iteration count");
  if (!validPrecision(cfg->precision))
    return fail(PD_ERR_UNSUPPORTED, "unsupported precision mode");
  if (cfg->cheb_mode < PD_CHEB_OFF || cfg->cheb_mode > PD_CHEB_INTERVAL)
    return fail(PD_ERR_INVALID_ARGUMENT, "cheb_mode must be 0, 1 or 2");
  bool refactor = false;  // dt is part of L: a new factor
  bool arith = false;     // a new precision mode: a host factorization (FP64_EXACT's bits) and a new plan
  bool replan = false;    // a new CTA count or explicit-inverse limit: a new plan and arena layout
  for (auto& I : s->inst) {
    refactor = refactor || (std::memcmp(&I.cfg.dt, &cfg->dt, sizeof(double)) != 0);
    arith = arith || I.cfg.precision != cfg->precision;
    replan = replan || I.cfg.cluster_ctas != cfg->cluster_ctas || I.cfg.dense_max_vertices != cfg->dense_max_vertices;
  }
  if (refactor || arith || replan) {
    // the planner and the arena layout depend on these fields, so the state comes back to the
    // host before the configuration changes and the handle is laid out again from it
    int rc = s->pullState();
    if (rc) return rc;
    for (auto& I : s->inst) I.cfg = *cfg;
    if (arith) s->plan = pd_plan{};  // a launch plan is tuned for one mode: the planner's choices apply
    for (auto& I : s->inst) {
      if (!refactor && !arith) break;
      const auto t0 = Clock::now();
      // a precision change refactorizes on the host, as a handle created in the new mode does
      if (arith) I.F.maxRowLen = 0;
      const std::string err = prepare(I, false);
      if (!err.empty()) return fail(PD_ERR_FACTORIZATION, err);
      I.assembleSeconds += secondsSince(t0);
    }
    const auto t1 = Clock::now();
    rc = s->upload(s->logCapacity);
    const double share = secondsSince(t1) / static_cast<double>(s->inst.size());
    for (auto& I : s->inst) I.assembleSeconds += share;  // the re-upload (and device refactorization)
    return rc;
  }
  if (const int rc_ = s->sync()) return rc_;
  for (auto& I : s->inst) I.cfg = *cfg;
  return s->writeDescriptors();
}

// ------------------------------------------------------------------------------ stage times
int pd_sim_set_stage_timing(pd_sim* s, int32_t enable) {
  if (!s) return fail(PD_ERR_INVALID_ARGUMENT, "null handle");
  if (const int rc_ = s->sync()) return rc_;
  if (enable && !s->dStage) {
    const size_t bytes = sizeof(double) * pdg::kStageCount * s->inst.size();
    PD_CUDA(cudaMalloc(&s->dStage, bytes));
    PD_CUDA(cudaMemset(s->dStage, 0, bytes));
  }
  s->stageTiming = enable != 0;
  return s->writeDescriptors();
}

int pd_sim_reset_stage_times(pd_sim* s) {
  if (!s) return fail(PD_ERR_INVALID_ARGUMENT, "null handle");
  if (const int rc_ = s->sync()) return rc_;
  if (s->dStage) PD_CUDA(cudaMemset(s->dStage, 0, sizeof(double) * pdg::kStageCount * s->inst.size()));
  for (auto& I : s->inst) I.assembleSeconds = 0.0;
  return PD_OK;
}

int pd_sim_get_stage_times(pd_sim* s, int32_t i, pd_stage_times* out) {
  int rc = checkInstance(s, i);
  if (rc) return rc;
  if (!out) return fail(PD_ERR_INVALID_ARGUMENT, "null output");
  if (const int rc_ = s->sync()) return rc_;
  double ns[pdg::kStageCount] = {0};
  if (s->dStage)
    PD_CUDA(cudaMemcpy(ns, s->dStage + pdg::kStageCount * static_cast<size_t>(i), sizeof(ns), cudaMemcpyDeviceToHost));
  out->predict = ns[pdg::kStagePredict] * 1e-9;
  out->local_step = ns[pdg::kStageLocal] * 1e-9;
  out->scatter = ns[pdg::kStageScatter] * 1e-9;
  out->assemble = s->inst[i].assembleSeconds;
  out->solve = ns[pdg::kStageSolve] * 1e-9;
  out->unpack_scan = ns[pdg::kStageUnpack] * 1e-9;
  out->velocity = ns[pdg::kStageVelocity] * 1e-9;
  out->total = ns[pdg::kStageTotal] * 1e-9;
  return PD_OK;
}

int pd_sim_get_info(pd_sim* s, int32_t i, pd_sim_info* out) {
  int rc = checkInstance(s, i);
  if (rc) return rc;
  if (!out) return fail(PD_ERR_INVALID_ARGUMENT, "null output");
  const Instance& I = s->inst[i];
  out->n_vertices = I.scene.n;
  out->n_edges = static_cast<int32_t>(I.scene.edges.size());
  out->n_bends = static_cast<int32_t>(I.scene.bends.size());
  out->color_count = I.topo.colorCount;
  out->matrix_nnz = static_cast<int64_t>(I.L.val.size());
  out->factor_nnz = static_cast<int64_t>(I.F.colval.size());
  out->forward_levels = static_cast<int32_t>(I.F.fwdLevelPtr.size()) - 1;
  out->backward_levels = static_cast<int32_t>(I.F.bwdLevelPtr.size()) - 1;
  out->factorize_count = I.factorizeCount;
  out->analyze_count = I.analyzeCount;
  out->device_bytes = static_cast<int64_t>(I.bytes);
  out->cluster_ctas = (s->corr && I.corrTeam > 1) ? I.corrTeam : s->teamCtas;
  out->device_factorize_count = I.deviceRefactorCount;
  out->host_state = s->hostX.empty() ? PD_HOST_STATE_NONE : s->hostTable.empty() ? PD_HOST_STATE_COPIES
                                                                                 : PD_HOST_STATE_GRAPH;
  const int p = s->precision();
  out->solve_kind = p == PD_PRECISION_FP64_EXACT ? PD_SOLVE_LEVELS
                    : s->delta64                 ? PD_SOLVE_DENSE64_TEAM
                    : !mixedSolve(p)             ? PD_SOLVE_SUPERNODAL
                    : s->delta                   ? PD_SOLVE_DENSE32_TEAM
                    : s->corr                    ? PD_SOLVE_SUPERNODAL32_CORRECTION
                    : s->dense                   ? PD_SOLVE_DENSE32
                                                 : PD_SOLVE_SUPERNODAL32;
  return PD_OK;
}

int pd_sim_get_stats(pd_sim* s, int32_t i, pd_sim_stats* out) {
  int rc = checkInstance(s, i);
  if (rc) return rc;
  if (!out) return fail(PD_ERR_INVALID_ARGUMENT, "null output");
  const Instance& I = s->inst[i];
  if (const int rc_ = s->sync()) return rc_;
  int32_t ints[3];
  PD_CUDA(cudaMemcpy(&out->last_residual, s->dArena + I.oLastRes, sizeof(double), cudaMemcpyDeviceToHost));
  PD_CUDA(cudaMemcpy(&ints[0], s->dArena + I.oIters, 4, cudaMemcpyDeviceToHost));
  PD_CUDA(cudaMemcpy(&ints[1], s->dArena + I.oConv, 4, cudaMemcpyDeviceToHost));
  PD_CUDA(cudaMemcpy(&ints[2], s->dArena + I.oEarly, 4, cudaMemcpyDeviceToHost));
  out->iterations_used = ints[0];
  out->converged = ints[1];
  out->early_exit_count = ints[2];
  return PD_OK;
}

// ------------------------------------------------------------------------------ spectrum
int pd_sim_spectrum(pd_sim* s, int32_t i, int32_t iters, pd_spectrum* out) {
  int rc = checkInstance(s, i);
  if (rc) return rc;
  if (!out) return fail(PD_ERR_INVALID_ARGUMENT, "null output");
  if (iters < 1 || iters > (1 << 20)) return fail(PD_ERR_INVALID_ARGUMENT, "power_iterations must be in [1, 2^20]");
  if (const int rc_ = s->sync()) return rc_;
  const Instance& I = s->inst[i];
  const size_t n3 = 3 * static_cast<size_t>(I.scene.n), e3 = 3 * std::max<size_t>(1, I.scene.edges.size());
  std::vector<double> x0(n3, 0.0);  // iteration_spectrum.cpp:319-324
  std::mt19937 rng(12345);
  for (int v = 0; v < I.scene.n; ++v) {
    if (I.scene.pinned[v]) continue;
    for (int d = 0; d < 3; ++d) x0[3 * v + d] = static_cast<double>(rng() % 2000) / 1000.0 - 1.0;
  }
  double* work = nullptr;
  PD_CUDA(cudaMalloc(&work, sizeof(double) * (3 * n3 + e3 + 4)));
  double* dx0 = work;
  double* dp = work + n3;
  double* dy = work + 2 * n3;
  double* dnE = work + 3 * n3;
  double* dout = dnE + e3;
  double res[4] = {0, 0, 0, 0};
  cudaError_t e = cudaMemcpyAsync(dx0, x0.data(), sizeof(double) * n3, cudaMemcpyHostToDevice, s->stream);
  const int cs = I.scene.n >= 1024 ? 16 : I.scene.n >= 256 ? 4 : 1;
  if (e == cudaSuccess)
    e = static_cast<cudaError_t>(pdg::launchSpectrum(s->dDesc + i, dx0, dp, dy, dnE, dout, iters, cs, s->stream));
  if (e == cudaSuccess) e = cudaMemcpyAsync(res, dout, sizeof(res), cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  cudaFree(work);
  if (e != cudaSuccess) return cudaFail(e, "spectrum");
  out->rho_plain = res[0];
  out->rho_plain_prev = res[1];
  out->lambda_max = res[2];
  out->lambda_max_prev = res[3];
  out->lambda_min = 1.0 - res[0];
  const double sq = std::sqrt(out->lambda_min / out->lambda_max);
  out->rho_cheb = (1.0 - sq) / (1.0 + sq);
  return PD_OK;
}

// ------------------------------------------------------------------------------ plan / autotuner
// State a re-plan must carry over: positions, velocities and the gate counters of every instance.
struct SavedSim {
  std::vector<std::vector<double>> x, v;
  std::vector<double> lastRes;
  std::vector<int32_t> iters, conv, early;
};

static int saveSim(pd_sim* s, SavedSim& o) {
  if (const int rc = s->pullState()) return rc;
  const size_t count = s->inst.size();
  o.x.resize(count);
  o.v.resize(count);
  o.lastRes.resize(count);
  o.iters.resize(count);
  o.conv.resize(count);
  o.early.resize(count);
  for (size_t i = 0; i < count; ++i) {
    const Instance& I = s->inst[i];
    o.x[i] = I.scene.x;
    o.v[i] = I.scene.v;
    PD_CUDA(cudaMemcpy(&o.lastRes[i], s->dArena + I.oLastRes, sizeof(double), cudaMemcpyDeviceToHost));
    PD_CUDA(cudaMemcpy(&o.iters[i], s->dArena + I.oIters, 4, cudaMemcpyDeviceToHost));
    PD_CUDA(cudaMemcpy(&o.conv[i], s->dArena + I.oConv, 4, cudaMemcpyDeviceToHost));
    PD_CUDA(cudaMemcpy(&o.early[i], s->dArena + I.oEarly, 4, cudaMemcpyDeviceToHost));
  }
  return PD_OK;
}

// Re-plans and re-uploads from the saved state (the arena is seeded from the host scenes).
static int replan(pd_sim* s, const pd_plan& p, const SavedSim& o, int capacity) {
  s->plan = p;
  for (size_t i = 0; i < s->inst.size(); ++i) {
    s->inst[i].scene.x = o.x[i];
    s->inst[i].scene.v = o.v[i];
  }
  if (const int rc = s->upload(capacity)) return rc;
  return s->ensureAux();
}

static int restoreCounters(pd_sim* s, const SavedSim& o) {
  for (size_t i = 0; i < s->inst.size(); ++i) {
    const Instance& I = s->inst[i];
    PD_CUDA(cudaMemcpy(s->dArena + I.oLastRes, &o.lastRes[i], sizeof(double), cudaMemcpyHostToDevice));
    PD_CUDA(cudaMemcpy(s->dArena + I.oIters, &o.iters[i], 4, cudaMemcpyHostToDevice));
    PD_CUDA(cudaMemcpy(s->dArena + I.oConv, &o.conv[i], 4, cudaMemcpyHostToDevice));
    PD_CUDA(cudaMemcpy(s->dArena + I.oEarly, &o.early[i], 4, cudaMemcpyHostToDevice));
  }
  s->lastSubsteps = 0;  // the logs and trace of the tuning launches are not the simulation's
  return PD_OK;
}

static pd_plan effectivePlan(const pd_sim* s) {
  pd_plan p{};
  p.team_ctas = s->teamCtas;
  p.big_min_vertices = s->plan.big_min_vertices != 0 ? s->plan.big_min_vertices : kBatchClusterMinVertices;
  p.big_cluster_ctas = s->bigCs;
  p.work_threads = (s->corr && s->teamCtas == 1 && s->inst.size() > 1)
                       ? (s->workThreads > 0 ? s->workThreads : pdg::kBlockThreads) : 0;
  p.latency_scale = s->latencyScale();
  return p;
}

// Mean time of one substep over `substeps` substeps after one warm-up substep.
static int timeSubsteps(pd_sim* s, int substeps, cudaEvent_t e0, cudaEvent_t e1, double* ms) {
  if (const int rc = s->launchSubsteps(s->stream, 1)) return rc;
  PD_CUDA(cudaEventRecord(e0, s->stream));
  if (const int rc = s->launchSubsteps(s->stream, substeps)) return rc;
  PD_CUDA(cudaEventRecord(e1, s->stream));
  if (const int rc = s->sync()) return rc;
  float t = 0.f;
  PD_CUDA(cudaEventElapsedTime(&t, e0, e1));
  *ms = static_cast<double>(t) / substeps;
  return PD_OK;
}

static bool validPlan(const pd_plan& p) {
  return p.team_ctas >= 0 && p.team_ctas <= 1024 && (p.big_cluster_ctas == 0 || (p.big_cluster_ctas >= 2 &&
         p.big_cluster_ctas <= 16)) && std::isfinite(p.latency_scale) && p.latency_scale >= 0.0 &&
         p.latency_scale <= 1e3 &&
         (p.work_threads == 0 || p.work_threads == 256 || p.work_threads == 512 || p.work_threads == 1024);
}

int pd_sim_set_plan(pd_sim* s, const pd_plan* plan) {
  if (!s || !plan) return fail(PD_ERR_INVALID_ARGUMENT, "null argument");
  if (!validPlan(*plan)) return fail(PD_ERR_INVALID_ARGUMENT, "plan field out of range");
  SavedSim o;
  if (const int rc = saveSim(s, o)) return rc;
  if (const int rc = replan(s, *plan, o, s->logCapacity > 0 ? s->logCapacity : 1)) return rc;
  return restoreCounters(s, o);
}

int pd_sim_get_plan(pd_sim* s, pd_plan* out) {
  if (!s || !out) return fail(PD_ERR_INVALID_ARGUMENT, "null argument");
  *out = effectivePlan(s);
  return PD_OK;
}

int pd_sim_autotune(pd_sim* s, int32_t substeps, pd_plan* tried, double* ms_per_substep, int32_t* n_tried,
                    int32_t* chosen) {
  if (!s) return fail(PD_ERR_INVALID_ARGUMENT, "null handle");
  if (substeps <= 0) return fail(PD_ERR_INVALID_ARGUMENT, "substeps must be > 0");
  SavedSim o;
  if (const int rc = saveSim(s, o)) return rc;
  const int capacity = std::max(s->logCapacity, substeps);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  {
    cudaError_t ce = cudaEventCreate(&e0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
    if (ce != cudaSuccess) {
      if (e0) cudaEventDestroy(e0);
      return cudaFail(ce, "autotune timing events");
    }
  }
  std::vector<pd_plan> plans, effective;
  std::vector<double> times;
  int rc = PD_OK;
  auto run = [&](const pd_plan& p) {
    if (rc != PD_OK || plans.size() >= PD_TUNE_MAX_CANDIDATES) return;
    double ms = 0.0;
    rc = replan(s, p, o, capacity);
    if (rc == PD_OK) rc = timeSubsteps(s, substeps, e0, e1, &ms);
    if (rc != PD_OK) return;
    plans.push_back(p);
    effective.push_back(effectivePlan(s));
    times.push_back(ms);
  };
  auto best = [&]() {
    size_t b = 0;
    for (size_t i = 1; i < times.size(); ++i)
      if (times[i] < times[b]) b = i;
    return b;
  };
  const pd_plan start = s->plan;
  run(start);  // candidate 0: the plan in force
  const int p = s->precision();
  const int count = static_cast<int>(s->inst.size());
  if (rc == PD_OK && p != PD_PRECISION_FP64_EXACT) {
    const int team0 = s->teamCtas;
    const bool delta = s->delta || s->delta64, corr = s->corr, supernodal = !delta && !s->dense;
    if (delta) {  // team sizes below the built-in SMs ÷ cloths
      for (int t : {team0 * 3 / 4, team0 / 2, team0 / 4})
        if (t >= 2 && t != team0 && (!s->delta64 || t > 16)) {
          pd_plan c = start;
          c.team_ctas = t;
          run(c);
        }
      if (s->delta64)  // and the FP64 supernodal kernel on one CTA or a 16-CTA cluster per cloth
        for (int t : {1, 16}) {
          pd_plan c = start;
          c.team_ctas = t;
          run(c);
        }
    } else if (corr && count > 1 && team0 == 1) {  // a batch: which cloths run as clusters, how large
      for (int minN : {-1, 4096, 8192, 12288})
        for (int cs : {2, 4, 8}) {
          if (minN < 0 && cs != 4) continue;
          pd_plan c = start;
          c.big_min_vertices = minN;
          c.big_cluster_ctas = cs;
          if (minN == effective[0].big_min_vertices && cs == effective[0].big_cluster_ctas &&
              effective[0].work_threads == pdg::kBlockThreads)
            continue;
          c.work_threads = pdg::kBlockThreads;
          run(c);
        }
      for (int wt : {512, 1024}) {  // the batch as a work table
        pd_plan c = start;
        c.work_threads = wt;
        if (wt == effective[0].work_threads) continue;
        run(c);
      }
    } else {  // CTAs per cloth of the cluster kernels; one large MIXED cloth also on a grid of CTAs
      std::vector<int> sizes = count <= 9 ? std::vector<int>{1, 2, 4, 8, 16} : std::vector<int>{1, 2, 4};
      const bool mixedGrid = p == PD_PRECISION_FP32_SOLVE && count == 1 && s->inst[0].scene.n > s->denseLimit();
      if ((corr || supernodalFp64(p) || mixedGrid) && count == 1) {
        const int cap = corr ? pdg::corrGridCapacity() : mixedGrid ? pdg::mixedGridCapacity() : pdg::gridCapacity();
        for (int g : {cap / 4, cap / 2, cap})
          if (g > 16) sizes.push_back(g);
      }
      for (int t : sizes)
        if (t != team0) {
          pd_plan c = start;
          c.team_ctas = t;
          run(c);
        }
    }
    if (supernodal) {  // then the lane model's latency weight for the best so far
      const pd_plan b = plans[best()];
      for (double w : {0.5, 2.0}) {
        pd_plan c = b;
        c.latency_scale = w;
        run(c);
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != PD_OK) {  // back to the plan and state the handle had (best effort), then report
    const std::string msg = g_lastError;
    if (replan(s, start, o, s->logCapacity > 0 ? s->logCapacity : 1) == PD_OK) restoreCounters(s, o);
    g_lastError = msg;
    return rc;
  }
  const size_t b = best();
  if (const int rc2 = replan(s, plans[b], o, s->logCapacity > 0 ? s->logCapacity : 1)) return rc2;
  if (const int rc2 = restoreCounters(s, o)) return rc2;
  const size_t k = std::min<size_t>(plans.size(), PD_TUNE_MAX_CANDIDATES);
  for (size_t i = 0; i < k; ++i) {
    if (tried) tried[i] = effective[i];
    if (ms_per_substep) ms_per_substep[i] = times[i];
  }
  if (n_tried) *n_tried = static_cast<int32_t>(k);
  if (chosen) *chosen = static_cast<int32_t>(b);
  return PD_OK;
}

int pd_sim_iteration_log(pd_sim* s, int32_t i, int32_t* iters, uint8_t* conv, int32_t count) {
  int rc = checkInstance(s, i);
  if (rc) return rc;
  if (count < 0 || count > s->lastSubsteps) return fail(PD_ERR_INVALID_ARGUMENT, "count exceeds the last step's substeps");
  if (const int rc_ = s->sync()) return rc_;
  if (iters) PD_CUDA(cudaMemcpy(iters, s->dIterLog + static_cast<size_t>(i) * s->logCapacity, 4 * count, cudaMemcpyDeviceToHost));
  if (conv) PD_CUDA(cudaMemcpy(conv, s->dConvLog + static_cast<size_t>(i) * s->logCapacity, count, cudaMemcpyDeviceToHost));
  return PD_OK;
}

int pd_sim_set_residual_trace(pd_sim* s, int32_t enable) {
  if (!s) return fail(PD_ERR_INVALID_ARGUMENT, "null handle");
  if (const int rc_ = s->sync()) return rc_;
  s->traceOn = enable != 0;
  return s->writeDescriptors();
}

int pd_sim_get_residual_trace(pd_sim* s, int32_t i, double* out, int32_t substeps) {
  int rc = checkInstance(s, i);
  if (rc) return rc;
  if (!out) return fail(PD_ERR_INVALID_ARGUMENT, "null output");
  if (!s->traceOn) return fail(PD_ERR_STATE, "the residual trace is not enabled");
  if (substeps < 0 || substeps > s->lastSubsteps)
    return fail(PD_ERR_INVALID_ARGUMENT, "substeps exceeds the last step's substeps");
  if (const int rc_ = s->sync()) return rc_;
  const size_t k = static_cast<size_t>(std::max(1, s->inst[i].cfg.max_iterations));
  PD_CUDA(cudaMemcpy(out, s->dTrace + s->traceOff[i], sizeof(double) * k * substeps, cudaMemcpyDeviceToHost));
  return PD_OK;
}

int pd_sim_get_factor(pd_sim* s, int32_t i, int32_t* perm, int32_t* colptr, int32_t* rowidx, double* val,
                      double* dinv, int64_t* nnz) {
  int rc = checkInstance(s, i);
  if (rc) return rc;
  const pdg::Factor& F = s->inst[i].F;
  if (nnz) *nnz = static_cast<int64_t>(F.colval.size());
  if (perm) std::memcpy(perm, F.perm.data(), F.perm.size() * 4);
  if (colptr) std::memcpy(colptr, F.colptr.data(), F.colptr.size() * 4);
  if (rowidx) std::memcpy(rowidx, F.rowidx.data(), F.rowidx.size() * 4);
  if (val) std::memcpy(val, F.colval.data(), F.colval.size() * 8);
  if (dinv) std::memcpy(dinv, F.dinv.data(), F.dinv.size() * 8);
  return PD_OK;
}

int pd_sim_solve(pd_sim* s, int32_t i, const double* b, double* x) {
  int rc = checkInstance(s, i);
  if (rc) return rc;
  if (!b || !x) return fail(PD_ERR_INVALID_ARGUMENT, "null vector");
  const Instance& I = s->inst[i];
  const size_t bytes = 24 * static_cast<size_t>(I.scene.n);
  double* dB = nullptr;
  PD_CUDA(cudaMalloc(&dB, 2 * bytes));
  double* dX = dB + 3 * static_cast<size_t>(I.scene.n);
  PD_CUDA(cudaMemcpyAsync(dB, b, bytes, cudaMemcpyHostToDevice, s->stream));
  const bool fast = s->precision() != PD_PRECISION_FP64_EXACT;
  const int need = (fast ? 48 : 24) * I.scene.n;
  const int smem = (need <= kMaxSmem) ? need : 0;
  const int lrc = fast ? pdg::launchSolveFast(s->dDesc + i, dB, dX, smem, s->stream)
                       : pdg::launchSolveExact(s->dDesc + i, dB, dX, smem, s->stream);
  if (lrc != 0) {
    cudaFree(dB);
    return cudaFail(static_cast<cudaError_t>(lrc), "solve launch");
  }
  PD_CUDA(cudaMemcpyAsync(x, dX, bytes, cudaMemcpyDeviceToHost, s->stream));
  if (const int rc_ = s->sync()) return rc_;
  PD_CUDA(cudaFree(dB));
  return PD_OK;
}

int pd_sim_gradient(pd_sim* s, int32_t substeps, const double* const* targets, const double* const* forces,
                    double* loss, double* const* dkappa, double* const* dv0, double* const* dforce) {
  if (!s) return fail(PD_ERR_INVALID_ARGUMENT, "null handle");
  if (substeps < 0) return fail(PD_ERR_INVALID_ARGUMENT, "substeps must be >= 0");
  if (!targets) return fail(PD_ERR_INVALID_ARGUMENT, "null targets");
  const int count = static_cast<int>(s->inst.size());
  for (int i = 0; i < count; ++i)
    if (!targets[i]) return fail(PD_ERR_INVALID_ARGUMENT, "null target of instance " + std::to_string(i));
  for (const auto& I : s->inst)
    if (I.cfg.cheb_mode != PD_CHEB_OFF)
      return fail(PD_ERR_UNSUPPORTED, "gradients of over-relaxed iterations (cheb_mode) are not provided");
  if (const int rc_ = s->sync()) return rc_;
  // device work arrays: per instance [target, force?, every iterate of every substep — or the
  // (x, v) checkpoints and one substep's iterates —, state and adjoints, per-edge terms, loss].
  // Every iterate is kept when the batch's copy fits in half of the free device memory and in
  // PD_GB300_GRADIENT_STORE_BYTES (default 128 GB; 0 always recomputes), which saves the reverse
  // pass re-running each substep.
  bool anyGrad = false;
  for (int i = 0; i < count; ++i)
    anyGrad = anyGrad || (dkappa && dkappa[i]) || (dv0 && dv0[i]) || (dforce && dforce[i]);
  auto doublesOf = [&](int i, bool stored) {
    const Instance& I = s->inst[i];
    const size_t n3 = 3 * static_cast<size_t>(I.scene.n), E = I.scene.edges.size();
    const size_t K = static_cast<size_t>(std::max(0, I.cfg.max_iterations));
    const size_t sub = static_cast<size_t>(std::max(1, substeps));
    const size_t states = stored ? sub * (K + 1) : 2 * sub + (K + 1);
    return n3 * (2 + states + 8) + 4 * E + 4;  // +4 keeps every instance 32-byte aligned
  };
  bool stored = false;
  if (anyGrad) {
    size_t freeB = 0, totalB = 0;
    double want = 0.0;
    for (int i = 0; i < count; ++i) want += 8.0 * doublesOf(i, true);
    double cap = 128.0 * (1ull << 30);
    if (const char* e = std::getenv("PD_GB300_GRADIENT_STORE_BYTES")) cap = std::atof(e);
    if (cudaMemGetInfo(&freeB, &totalB) == cudaSuccess)
      stored = want <= std::min(0.5 * static_cast<double>(freeB), cap);
  }
  std::vector<size_t> off(count + 1, 0);
  for (int i = 0; i < count; ++i) off[i + 1] = off[i] + (doublesOf(i, stored) + 3) / 4 * 4;
  double* dWork = nullptr;
  pdg::GradDev* dG = nullptr;
  PD_CUDA(cudaMalloc(&dWork, sizeof(double) * off[count]));
  if (cudaMalloc(&dG, sizeof(pdg::GradDev) * count) != cudaSuccess) {
    cudaFree(dWork);
    return cudaFail(cudaGetLastError(), "gradient descriptors");
  }
  std::vector<pdg::GradDev> gd(count);
  int smem = 0;
  int rc = PD_OK;
  for (int i = 0; i < count && rc == PD_OK; ++i) {
    const Instance& I = s->inst[i];
    const size_t n3 = 3 * static_cast<size_t>(I.scene.n), E = I.scene.edges.size();
    const size_t K = static_cast<size_t>(std::max(0, I.cfg.max_iterations));
    const size_t sub = static_cast<size_t>(std::max(1, substeps));
    double* p = dWork + off[i];
    pdg::GradDev& g = gd[i];
    g.target = p;
    p += n3;
    g.force = (forces && forces[i]) ? p : nullptr;
    p += n3;
    if (stored) {
      g.ckX = g.ckV = g.it = nullptr;
      g.itAll = p;
      p += sub * (K + 1) * n3;
    } else {
      g.itAll = nullptr;
      g.ckX = p;
      p += sub * n3;
      g.ckV = p;
      p += sub * n3;
      g.it = p;
      p += (K + 1) * n3;
    }
    double** vecs[] = {&g.xs, &g.vs, &g.xb, &g.vb, &g.xkb, &g.xnb, &g.xhb, &g.fb};
    for (double** v : vecs) {
      *v = p;
      p += n3;
    }
    g.ge = p;
    p += 3 * E;
    g.kb = p;
    p += E;
    g.loss = p;
    g.wantGrad = (dkappa && dkappa[i]) || (dv0 && dv0[i]) || (dforce && dforce[i]);
    if (cudaMemcpyAsync(const_cast<double*>(g.target), targets[i], 8 * n3, cudaMemcpyHostToDevice, s->stream) !=
            cudaSuccess ||
        (g.force && cudaMemcpyAsync(const_cast<double*>(g.force), forces[i], 8 * n3, cudaMemcpyHostToDevice,
                                    s->stream) != cudaSuccess))
      rc = cudaFail(cudaGetLastError(), "gradient inputs");
    const int need = 48 * I.scene.n;
    if (need <= kMaxSmem && need > smem) smem = need;
  }
  if (rc == PD_OK && cudaMemcpyAsync(dG, gd.data(), sizeof(pdg::GradDev) * count, cudaMemcpyHostToDevice,
                                     s->stream) != cudaSuccess)
    rc = cudaFail(cudaGetLastError(), "gradient descriptors");
  if (rc == PD_OK) {
    // a cluster per problem where the FP64 path runs clusters (the planner's CTAs per cloth)
    int cs = supernodalFp64(s->precision()) ? std::min(s->teamCtas, 16) : 1;  // a grid team: a 16-CTA cluster
    while (cs > 1 && pdg::gradClusterSupported(cs) != cs) cs /= 2;
    const int lrc = pdg::launchGradient(s->dDesc, dG, count, cs, substeps, smem, s->stream);
    if (lrc != 0) rc = cudaFail(static_cast<cudaError_t>(lrc), "gradient launch");
  }
  for (int i = 0; i < count && rc == PD_OK; ++i) {
    const pdg::GradDev& g = gd[i];
    const Instance& I = s->inst[i];
    const size_t n3 = 3 * static_cast<size_t>(I.scene.n), E = I.scene.edges.size();
    bool ok = !loss || cudaMemcpyAsync(loss + i, g.loss, 8, cudaMemcpyDeviceToHost, s->stream) == cudaSuccess;
    if (g.wantGrad) {
      if (dkappa && dkappa[i]) ok = ok && cudaMemcpyAsync(dkappa[i], g.kb, 8 * E, cudaMemcpyDeviceToHost, s->stream) == cudaSuccess;
      if (dv0 && dv0[i]) ok = ok && cudaMemcpyAsync(dv0[i], g.vb, 8 * n3, cudaMemcpyDeviceToHost, s->stream) == cudaSuccess;
      if (dforce && dforce[i]) ok = ok && cudaMemcpyAsync(dforce[i], g.fb, 8 * n3, cudaMemcpyDeviceToHost, s->stream) == cudaSuccess;
    }
    if (!ok) rc = cudaFail(cudaGetLastError(), "gradient results");
  }
  if (rc == PD_OK && cudaStreamSynchronize(s->stream) != cudaSuccess) rc = cudaFail(cudaGetLastError(), "gradient");
  cudaFree(dG);
  cudaFree(dWork);
  return rc;
}

int pd_scene_factor(const pd_mesh* mesh, const pd_scene_config* cfg, int32_t* perm, int32_t* colptr,
                    int32_t* rowidx, double* val, double* dinv, int64_t* nnz, pd_sim_info* info) {
  if (!mesh || !cfg) return fail(PD_ERR_INVALID_ARGUMENT, "null argument");
  Instance I;
  I.cfg = *cfg;
  int rc = sceneFromMesh(*mesh, I.scene);
  if (rc) return rc;
  std::string err = pdg::validateScene(I.scene);
  if (!err.empty()) return fail(PD_ERR_INVALID_ARGUMENT, err);
  pdg::buildTopology(I.scene, I.topo);
  err = prepare(I, true);
  if (!err.empty()) return fail(prepareCode(err), err);
  const pdg::Factor& F = I.F;
  if (nnz) *nnz = static_cast<int64_t>(F.colval.size());
  if (perm) std::memcpy(perm, F.perm.data(), F.perm.size() * 4);
  if (colptr) std::memcpy(colptr, F.colptr.data(), F.colptr.size() * 4);
  if (rowidx) std::memcpy(rowidx, F.rowidx.data(), F.rowidx.size() * 4);
  if (val) std::memcpy(val, F.colval.data(), F.colval.size() * 8);
  if (dinv) std::memcpy(dinv, F.dinv.data(), F.dinv.size() * 8);
  if (info) {
    Arena A;
    layout(I, A, 1, 0);
    info->cluster_ctas = 1;
    info->host_state = PD_HOST_STATE_NONE;
    info->device_factorize_count = 0;
    info->solve_kind = I.cfg.precision == PD_PRECISION_FP64_EXACT ? PD_SOLVE_LEVELS
                       : mixedSolve(I.cfg.precision)              ? PD_SOLVE_SUPERNODAL32
                                                                  : PD_SOLVE_SUPERNODAL;
    info->n_vertices = I.scene.n;
    info->n_edges = static_cast<int32_t>(I.scene.edges.size());
    info->n_bends = static_cast<int32_t>(I.scene.bends.size());
    info->color_count = I.topo.colorCount;
    info->matrix_nnz = static_cast<int64_t>(I.L.val.size());
    info->factor_nnz = static_cast<int64_t>(F.colval.size());
    info->forward_levels = static_cast<int32_t>(F.fwdLevelPtr.size()) - 1;
    info->backward_levels = static_cast<int32_t>(F.bwdLevelPtr.size()) - 1;
    info->factorize_count = I.factorizeCount;
    info->analyze_count = I.analyzeCount;
    info->device_bytes = static_cast<int64_t>(I.bytes);
  }
  return PD_OK;
}

int pd_scene_coloring(const pd_mesh* mesh, uint32_t* color_of, int32_t* colors) {
  if (!mesh) return fail(PD_ERR_INVALID_ARGUMENT, "null argument");
  pdg::Scene s;
  int rc = sceneFromMesh(*mesh, s);
  if (rc) return rc;
  const std::string err = pdg::validateScene(s);
  if (!err.empty()) return fail(PD_ERR_INVALID_ARGUMENT, err);
  pdg::Topology t;
  pdg::buildTopology(s, t);
  if (color_of) std::memcpy(color_of, t.colorOf.data(), t.colorOf.size() * 4);
  if (colors) *colors = t.colorCount;
  return PD_OK;
}

// ------------------------------------------------------------------------------- solver
int pd_solver_create(pd_solver** out) {
  if (!out) return fail(PD_ERR_INVALID_ARGUMENT, "out is null");
  *out = new pd_solver();
  return PD_OK;
}

int pd_solver_destroy(pd_solver* s) {
  delete s;
  return PD_OK;
}

int pd_solver_analyze(pd_solver* s, int32_t n, const int32_t* cp, const int32_t* ri) {
  if (!s || !cp || !ri || n <= 0) return fail(PD_ERR_INVALID_ARGUMENT, "invalid pattern");
  const auto t0 = Clock::now();
  pdg::ScalarMatrix A;
  const std::string err = scalarFromBlocks(n, cp, ri, nullptr, A);
  if (!err.empty()) return fail(PD_ERR_UNSUPPORTED, err);
  s->n3 = n;
  s->pattern_cp.assign(cp, cp + n + 1);
  s->pattern_ri.assign(ri, ri + cp[n]);
  s->perm = minimumDegreeOrder(A);
  s->analyzedFlag = true;
  s->ready = false;
  s->stats.analyze_calls += 1;
  s->stats.last_analyze_seconds = secondsSince(t0);
  s->stats.nnz = cp[n];
  return PD_OK;
}

int pd_solver_analyzed(const pd_solver* s) { return (s && s->analyzedFlag) ? 1 : 0; }

int pd_solver_factorize(pd_solver* s, int32_t n, const int32_t* cp, const int32_t* ri, const double* val) {
  if (!s || !cp || !ri || !val) return fail(PD_ERR_INVALID_ARGUMENT, "null argument");
  if (!s->analyzedFlag) return fail(PD_ERR_STATE, "factorize before analyze");
  if (n != s->n3 || cp[n] != s->pattern_cp[n] || std::memcmp(cp, s->pattern_cp.data(), 4 * (n + 1)) != 0 ||
      std::memcmp(ri, s->pattern_ri.data(), 4 * static_cast<size_t>(cp[n])) != 0)
    return fail(PD_ERR_STATE, "structure differs from the analysed pattern");
  const auto t0 = Clock::now();
  s->ready = false;
  s->stats.factorize_calls += 1;
  std::string err = scalarFromBlocks(n, cp, ri, val, s->A);
  if (!err.empty()) return fail(PD_ERR_UNSUPPORTED, err);
  if (!pdg::factorize(s->A, s->perm, s->F, &err)) return fail(PD_ERR_FACTORIZATION, err);
  // upload the factor as a solve-only instance
  Arena A;
  const size_t m = s->A.n;
  const size_t oIperm = A.add(s->F.iperm), oLrp = A.add(s->F.rowptr), oLci = A.add(s->F.colidx),
               oLrv = A.add(s->F.rowval), oLcp = A.add(s->F.colptr), oLri = A.add(s->F.rowidx),
               oLcv = A.add(s->F.colval), oDinv = A.add(s->F.dinv), oFp = A.add(s->F.fwdLevelPtr),
               oFr = A.add(s->F.fwdRows), oBp = A.add(s->F.bwdLevelPtr), oBr = A.add(s->F.bwdRows),
               oW = A.zeros(24 * m);
  if (s->dArena) cudaFree(s->dArena);
  if (s->dB) cudaFree(s->dB);
  s->dArena = nullptr;
  s->dB = nullptr;
  PD_CUDA(cudaMalloc(&s->dArena, A.host.size()));
  PD_CUDA(cudaMemcpy(s->dArena, A.host.data(), A.host.size(), cudaMemcpyHostToDevice));
  PD_CUDA(cudaMalloc(&s->dB, 2 * 24 * m));
  s->dX = s->dB + 3 * m;
  pdg::InstanceDev d{};
  d.n = static_cast<int32_t>(m);
  d.nlevF = static_cast<int32_t>(s->F.fwdLevelPtr.size()) - 1;
  d.nlevB = static_cast<int32_t>(s->F.bwdLevelPtr.size()) - 1;
  auto P = [&](size_t off) { return s->dArena + off; };
  d.iperm = reinterpret_cast<const int32_t*>(P(oIperm));
  d.Lrp = reinterpret_cast<const int32_t*>(P(oLrp));
  d.Lci = reinterpret_cast<const int32_t*>(P(oLci));
  d.Lrv = reinterpret_cast<const double*>(P(oLrv));
  d.Lcp = reinterpret_cast<const int32_t*>(P(oLcp));
  d.Lri = reinterpret_cast<const int32_t*>(P(oLri));
  d.Lcv = reinterpret_cast<const double*>(P(oLcv));
  d.dinv = reinterpret_cast<const double*>(P(oDinv));
  d.fwdPtr = reinterpret_cast<const int32_t*>(P(oFp));
  d.fwdRows = reinterpret_cast<const int32_t*>(P(oFr));
  d.bwdPtr = reinterpret_cast<const int32_t*>(P(oBp));
  d.bwdRows = reinterpret_cast<const int32_t*>(P(oBr));
  d.w = reinterpret_cast<double*>(P(oW));
  if (!s->dDesc) PD_CUDA(cudaMalloc(&s->dDesc, sizeof(pdg::InstanceDev)));
  PD_CUDA(cudaMemcpy(s->dDesc, &d, sizeof(d), cudaMemcpyHostToDevice));
  if (s->colM != m) {  // the per-component slots, made here so that concurrent solves allocate nothing
    s->releaseColumns();
    PD_CUDA(cudaMalloc(&s->dCol, sizeof(double) * 9 * m));
    PD_CUDA(cudaMallocHost(&s->hCol, sizeof(double) * 6 * m));
    s->colM = m;
  }
  for (cudaStream_t& st : s->colStream)
    if (!st) PD_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  s->ready = true;
  s->stats.last_factorize_seconds = secondsSince(t0);
  s->stats.total_factorize_seconds += s->stats.last_factorize_seconds;
  s->stats.nnz = cp[n];
  s->stats.factor_nnz = static_cast<int64_t>(s->F.colval.size());
  return PD_OK;
}

static int solverSolve(pd_solver* s, const double* b, double* x) {
  if (!s || !b || !x) return fail(PD_ERR_INVALID_ARGUMENT, "null argument");
  if (!s->ready) return fail(PD_ERR_STATE, "solve before a successful factorize");
  const size_t m = s->A.n, bytes = 24 * m;
  PD_CUDA(cudaMemcpyAsync(s->dB, b, bytes, cudaMemcpyHostToDevice, s->stream));
  const int smem = (24 * static_cast<int>(m) <= kMaxSmem) ? 24 * static_cast<int>(m) : 0;
  const int rc = pdg::launchSolveExact(s->dDesc, s->dB, s->dX, smem, s->stream);
  if (rc != 0) return cudaFail(static_cast<cudaError_t>(rc), "solve launch");
  PD_CUDA(cudaMemcpyAsync(x, s->dX, bytes, cudaMemcpyDeviceToHost, s->stream));
  PD_CUDA(cudaStreamSynchronize(s->stream));
  return PD_OK;
}

int pd_solver_solve(pd_solver* s, const double* b, double* x) {
  const auto t0 = Clock::now();
  const int rc = solverSolve(s, b, x);
  if (rc == PD_OK) {
    s->stats.solve_calls += 1;
    s->stats.last_solve_seconds = secondsSince(t0);
    s->stats.total_solve_seconds += s->stats.last_solve_seconds;
  }
  return rc;
}

int pd_solver_parallel_components(const pd_solver* s) { return (s && s->analyzedFlag) ? 3 : 1; }

int pd_solver_solve_component(pd_solver* s, int32_t c, const double* b, double* x) {
  if (c < 0 || c > 2) return fail(PD_ERR_INVALID_ARGUMENT, "component out of range");
  if (!s || !b || !x) return fail(PD_ERR_INVALID_ARGUMENT, "null argument");
  if (!s->ready) return fail(PD_ERR_STATE, "solve before a successful factorize");
  // only column c: its entries of b in, its entries of x out, on the component's own stream and
  // buffers, so the three components run side by side and write disjoint entries of x
  const size_t m = s->A.n;
  double* hb = s->hCol + 2 * m * c;
  double* hx = hb + m;
  double* db = s->dCol + 3 * m * c;
  double* dx = db + m;
  double* dw = dx + m;
  const cudaStream_t st = s->colStream[c];
  for (size_t v = 0; v < m; ++v) hb[v] = b[3 * v + c];
  PD_CUDA(cudaMemcpyAsync(db, hb, sizeof(double) * m, cudaMemcpyHostToDevice, st));
  const int smem = (8 * static_cast<int>(m) <= kMaxSmem) ? 8 * static_cast<int>(m) : 0;
  const int rc = pdg::launchSolveColumnExact(s->dDesc, db, dx, dw, smem, st);
  if (rc != 0) return cudaFail(static_cast<cudaError_t>(rc), "component solve launch");
  PD_CUDA(cudaMemcpyAsync(hx, dx, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
  PD_CUDA(cudaStreamSynchronize(st));
  for (size_t v = 0; v < m; ++v) x[3 * v + c] = hx[v];
  return PD_OK;
}

int pd_solver_note_solve_stage(pd_solver* s, double seconds) {
  if (!s) return fail(PD_ERR_INVALID_ARGUMENT, "null handle");
  if (pd_solver_parallel_components(s) <= 1) return PD_OK;  // solve() already counted (IGlobalSolver.h:100-111)
  s->stats.solve_calls += 1;
  s->stats.last_solve_seconds = seconds;
  s->stats.total_solve_seconds += seconds;
  return PD_OK;
}

int pd_solver_stats_get(const pd_solver* s, pd_solver_stats* out) {
  if (!s || !out) return fail(PD_ERR_INVALID_ARGUMENT, "null argument");
  *out = s->stats;
  return PD_OK;
}

}  // extern "C"
