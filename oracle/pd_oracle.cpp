// pd_oracle.cpp — CPU oracle (test infrastructure) for the per-substep PD loop.
//
// A restatement of the reference CPU path; each function names the reference file:line it
// follows. Build with -ffp-contract=off: every product and sum below must round on its own,
// as in the reference (MSVC /fp:precise, no contraction). Results are independent of the
// OpenMP thread count, exactly as in the reference (colour-ordered scatter, per-component
// solves, exact max reductions).
#include "pd_oracle.h"

#include <algorithm>
#include <unordered_set>
#include <string>
#include <sstream>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <set>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- Vec3 (core/math/Vec3.h:11-52)
struct V3 {
  double x = 0, y = 0, z = 0;
};
inline V3 add(const V3& a, const V3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(const V3& a, const V3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 mul(const V3& a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double length(const V3& a) { return std::sqrt(dot(a, a)); }
inline double maxAbsComponent(const V3& a) {
  return std::fmax(std::fabs(a.x), std::fmax(std::fabs(a.y), std::fabs(a.z)));
}
inline V3 ld(const double* p) { return {p[0], p[1], p[2]}; }
inline void st(double* p, const V3& v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }
// std::max semantics of the reference ((a < b) ? b : a).
inline double smax(double a, double b) { return (a < b) ? b : a; }

constexpr double kMinLength = 1e-12;  // DistanceTerm::kMinLength (core/energy/DistanceTerm.h:31)

struct Edge {
  int a, b;
  double rest, k;
};
struct Bend {
  int a, b, c;
  double k;
};

int g_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // namespace

struct oracle_sim {
  oracle_config cfg{};
  int n = 0;
  std::vector<double> x, v, m, q;  // positions, velocities (3n), masses (n), pin positions (3n)
  std::vector<uint8_t> pinned;
  std::vector<Edge> edges;
  std::vector<Bend> bends;

  // topology (core/mesh/ConstraintColoring.h:34-81)
  std::vector<uint32_t> colorOf, cstart, corder, vstart, vedges;
  int colorCount = 0;
  std::vector<uint32_t> bstart, bstencils;
  std::vector<double> bweight;

  // scalar L in vertex indexing (CSR, sorted columns)
  std::vector<int32_t> Lrow, Lcol;
  std::vector<double> Lval;

  // factor of P·L·Pᵀ: perm[k] = vertex eliminated k-th; strictly lower CSC in elimination order
  std::vector<int32_t> perm, iperm, Fp, Fi;
  std::vector<double> Fx, D, dinv;
  std::vector<int32_t> userPerm;
  bool factorReady = false;

  // stamps (core/assemble/Assembler.cpp:111-174)
  uint64_t stampKey[4] = {0, 0, 0, 0};
  bool stampValid = false;
  uint64_t structureStamp = 0;
  bool analyzed = false;

  // per-substep buffers (core/sim/Scene.h:171-188)
  std::vector<double> predicted, before, prevPos, b, bBase, xSol, bendRhs;

  // counters
  int factorizeCount = 0, analyzeCount = 0, iterationsUsed = 0, earlyExitCount = 0;
  bool converged = false;
  double lastResidual = -1.0;
  std::vector<double>* trace = nullptr;  // when set: the gate residual of every iteration, appended
};

namespace {

// ------------------------------------------------ colouring (core/mesh/ConstraintColoring.cpp)
constexpr uint32_t kUncolored = 0xFFFFFFFFu;

// priorityOf: splitmix64 finaliser on the edge index (ConstraintColoring.cpp:23-31).
uint32_t priorityOf(uint32_t e) {
  uint64_t x = static_cast<uint64_t>(e) * 0x9E3779B97F4A7C15ULL + 0x2545F4914F6CDD1DULL;
  x ^= x >> 30;
  x *= 0xBF58476D1CE4E5B9ULL;
  x ^= x >> 27;
  x *= 0x94D049BB133111EBULL;
  x ^= x >> 31;
  return static_cast<uint32_t>(x >> 32);
}

// Vertex → incident edges in edge-index order (ConstraintColoring.cpp:35-54).
void buildAdjacency(oracle_sim& s) {
  const int nv = s.n, ne = static_cast<int>(s.edges.size());
  s.vstart.assign(nv + 1, 0);
  for (const Edge& e : s.edges) {
    s.vstart[e.a + 1] += 1;
    s.vstart[e.b + 1] += 1;
  }
  for (int v = 0; v < nv; ++v) s.vstart[v + 1] += s.vstart[v];
  s.vedges.assign(2 * static_cast<size_t>(ne), 0);
  std::vector<uint32_t> cur(s.vstart.begin(), s.vstart.end() - 1);
  for (int i = 0; i < ne; ++i) {
    s.vedges[cur[s.edges[i].a]++] = i;
    s.vedges[cur[s.edges[i].b]++] = i;
  }
}

// Vertex → bend stencils in stencil order with weights {1,-2,1} (ConstraintColoring.cpp:82-119).
void buildBendAdjacency(oracle_sim& s) {
  const int nv = s.n, nb = static_cast<int>(s.bends.size());
  s.bstart.assign(nv + 1, 0);
  for (const Bend& b : s.bends) {
    s.bstart[b.a + 1] += 1;
    s.bstart[b.b + 1] += 1;
    s.bstart[b.c + 1] += 1;
  }
  for (int v = 0; v < nv; ++v) s.bstart[v + 1] += s.bstart[v];
  s.bstencils.assign(3 * static_cast<size_t>(nb), 0);
  s.bweight.assign(3 * static_cast<size_t>(nb), 0.0);
  std::vector<uint32_t> cur(s.bstart.begin(), s.bstart.end() - 1);
  for (int i = 0; i < nb; ++i) {
    const int vert[3] = {s.bends[i].a, s.bends[i].b, s.bends[i].c};
    const double w[3] = {1.0, -2.0, 1.0};
    for (int k = 0; k < 3; ++k) {
      const uint32_t slot = cur[vert[k]]++;
      s.bstencils[slot] = i;
      s.bweight[slot] = w[k];
    }
  }
}

// Jones–Plassmann colouring with smallest available colour (ConstraintColoring.cpp:121-259).
void buildColoring(oracle_sim& s) {
  const int ne = static_cast<int>(s.edges.size());
  s.colorOf.assign(ne, kUncolored);
  s.cstart.clear();
  s.corder.clear();
  s.colorCount = 0;
  buildAdjacency(s);
  if (ne <= 0) {
    s.cstart.push_back(0);
    return;
  }
  std::vector<uint32_t> prio(ne);
  for (int i = 0; i < ne; ++i) prio[i] = priorityOf(i);
  auto better = [&](uint32_t ea, uint32_t eb) {
    return prio[ea] > prio[eb] || (prio[ea] == prio[eb] && ea < eb);
  };
  auto forEachNeighbor = [&](uint32_t e, auto&& fn) {
    const uint32_t ends[2] = {static_cast<uint32_t>(s.edges[e].a), static_cast<uint32_t>(s.edges[e].b)};
    for (uint32_t v : ends)
      for (uint32_t k = s.vstart[v]; k < s.vstart[v + 1]; ++k)
        if (s.vedges[k] != e) fn(s.vedges[k]);
  };
  std::vector<uint32_t> remaining(ne), next, cand(ne, kUncolored);
  for (int i = 0; i < ne; ++i) remaining[i] = i;
  int maxColor = -1;
  while (!remaining.empty()) {
    // Candidate pass: reads only the previous round's colours, so a serial loop gives the
    // same result as the reference's parallelFor.
    for (uint32_t ed : remaining) {
      cand[ed] = kUncolored;
      bool allColored = true, localMax = true;
      forEachNeighbor(ed, [&](uint32_t f) {
        if (s.colorOf[f] == kUncolored) {
          allColored = false;
          if (better(f, ed)) localMax = false;
        }
      });
      if (!allColored && !localMax) continue;
      uint32_t pick = 0;
      bool clash = true;
      while (clash) {
        clash = false;
        forEachNeighbor(ed, [&](uint32_t f) {
          if (!clash && s.colorOf[f] == pick) {
            clash = true;
            ++pick;
          }
        });
      }
      cand[ed] = pick;
    }
    bool any = false;
    next.clear();
    for (uint32_t ed : remaining) {
      if (cand[ed] != kUncolored) {
        s.colorOf[ed] = cand[ed];
        maxColor = std::max(maxColor, static_cast<int>(cand[ed]));
        any = true;
      } else {
        next.push_back(ed);
      }
    }
    if (!any) {
      std::fprintf(stderr, "[oracle] colouring made no progress\n");
      std::abort();
    }
    remaining.swap(next);
  }
  s.colorCount = maxColor + 1;
  s.cstart.assign(s.colorCount + 1, 0);
  for (uint32_t c : s.colorOf) s.cstart[c + 1] += 1;
  for (int c = 0; c < s.colorCount; ++c) s.cstart[c + 1] += s.cstart[c];
  s.corder.assign(ne, 0);
  std::vector<uint32_t> cur(s.cstart.begin(), s.cstart.end() - 1);
  for (int i = 0; i < ne; ++i) s.corder[cur[s.colorOf[i]]++] = i;
  for (int c = 0; c < s.colorCount; ++c) {
    std::sort(s.corder.begin() + s.cstart[c], s.corder.begin() + s.cstart[c + 1],
              [&](uint32_t a, uint32_t b) {
                const uint32_t ma = std::min(s.edges[a].a, s.edges[a].b);
                const uint32_t mb = std::min(s.edges[b].a, s.edges[b].b);
                return ma != mb ? ma < mb : a < b;
              });
  }
}

void buildTopology(oracle_sim& s) {
  buildColoring(s);
  buildBendAdjacency(s);
}

// ------------------------------------------------------------ stamps (Assembler.cpp:29-92)
uint64_t bitsOf(double v) {
  uint64_t u;
  std::memcpy(&u, &v, 8);
  return u;
}
uint64_t mixh(uint64_t h, uint64_t v) {
  h ^= v + 0x9e3779b97f4a7c15ULL + (h << 6) + (h >> 2);
  return h;
}
void computeStamp(const oracle_sim& s, uint64_t out[4]) {
  uint64_t kh = 0xcbf29ce484222325ULL, mh = 0xcbf29ce484222325ULL, ph = 0xcbf29ce484222325ULL;
  for (const Edge& e : s.edges) kh = mixh(kh, bitsOf(e.k));
  for (const Bend& b : s.bends) kh = mixh(kh, bitsOf(b.k));
  for (double m : s.m) mh = mixh(mh, bitsOf(m));
  for (uint8_t p : s.pinned) ph = mixh(ph, p ? 1ULL : 0ULL);
  out[0] = kh;
  out[1] = mh;
  out[2] = ph;
  out[3] = bitsOf(s.cfg.dt);
}
uint64_t computeStructureStamp(const oracle_sim& s) {
  uint64_t h = 0xcbf29ce484222325ULL;
  h = mixh(h, 1);  // topologyId
  h = mixh(h, static_cast<uint64_t>(s.n));
  h = mixh(h, static_cast<uint64_t>(s.edges.size()));
  for (const Edge& e : s.edges) {
    h = mixh(h, static_cast<uint32_t>(e.a));
    h = mixh(h, static_cast<uint32_t>(e.b));
  }
  h = mixh(h, static_cast<uint64_t>(s.bends.size()));
  for (const Bend& b : s.bends) {
    h = mixh(h, static_cast<uint32_t>(b.a));
    h = mixh(h, static_cast<uint32_t>(b.b));
    h = mixh(h, static_cast<uint32_t>(b.c));
  }
  for (uint8_t p : s.pinned) h = mixh(h, p ? 1ULL : 0ULL);
  return h;
}

// ------------------------------------------------ L assembly (Assembler.cpp:139-278, scalar)
// L = Ã ⊗ I₃: every 3×3 block is a scalar times I₃ and the three components receive the same
// triplet sequence, so the scalar matrix Ã carries the exact values of all three. Duplicates
// are summed left to right in triplet order, as Eigen's setFromTriplets does.
struct Trip {
  int r, c;
  double v;
};
void assembleLhs(oracle_sim& s) {
  const int n = s.n;
  const double h = s.cfg.dt;
  const double invDt2 = 1.0 / (h * h);
  std::vector<Trip> t;
  t.reserve(n + 4 * s.edges.size() + 9 * s.bends.size() + n);
  auto P = [&](int v) { return s.pinned[v] != 0; };
  for (int v = 0; v < n; ++v) t.push_back({v, v, s.m[v] * invDt2});  // (1) M/h²
  for (const Edge& e : s.edges) {                                     // (2) DistanceTerm blocks
    const bool ap = P(e.a), bp = P(e.b);
    if (ap && bp) continue;
    if (!ap) t.push_back({e.a, e.a, e.k});
    if (!bp) t.push_back({e.b, e.b, e.k});
    if (!ap && !bp) {
      t.push_back({e.a, e.b, -e.k});
      t.push_back({e.b, e.a, -e.k});
    }
  }
  const double w[3] = {1.0, -2.0, 1.0};
  for (const Bend& b : s.bends) {  // (2b) bend blocks, free-free only
    if (b.k == 0.0) continue;
    const int vert[3] = {b.a, b.b, b.c};
    if (P(b.a) && P(b.b) && P(b.c)) continue;
    for (int p = 0; p < 3; ++p) {
      if (P(vert[p])) continue;
      for (int q = 0; q < 3; ++q) {
        if (P(vert[q])) continue;
        t.push_back({vert[p], vert[q], b.k * w[p] * w[q]});
      }
    }
  }
  for (int v = 0; v < n; ++v) {  // (3) pinned rows forced to identity
    if (!P(v)) continue;
    double existing = s.m[v] * invDt2;
    for (const Edge& e : s.edges) {
      if (P(e.a) || P(e.b)) continue;
      if (e.a == v || e.b == v) existing += e.k;
    }
    existing += 0.0;  // bendDiagonalAt(v) is 0 for a pinned vertex (Assembler.cpp:309-320)
    t.push_back({v, v, 1.0 - existing});
  }
  std::stable_sort(t.begin(), t.end(), [](const Trip& a, const Trip& b) {
    return a.r != b.r ? a.r < b.r : a.c < b.c;
  });
  s.Lrow.assign(n + 1, 0);
  s.Lcol.clear();
  s.Lval.clear();
  for (size_t i = 0; i < t.size();) {
    size_t j = i;
    double acc = t[i].v;
    for (++j; j < t.size() && t[j].r == t[i].r && t[j].c == t[i].c; ++j) acc = acc + t[j].v;
    s.Lcol.push_back(t[i].c);
    s.Lval.push_back(acc);
    s.Lrow[t[i].r + 1] += 1;
    i = j;
  }
  for (int r = 0; r < n; ++r) s.Lrow[r + 1] += s.Lrow[r];
}

// Bend constant RHS (Assembler.cpp:94-137).
void assembleBendingRhs(oracle_sim& s) {
  s.bendRhs.assign(3 * static_cast<size_t>(s.n), 0.0);
  if (s.bends.empty()) return;
  const double w[3] = {1.0, -2.0, 1.0};
  for (const Bend& b : s.bends) {
    if (b.k == 0.0) continue;
    const int vert[3] = {b.a, b.b, b.c};
    V3 c{0, 0, 0};
    bool any = false;
    for (int k = 0; k < 3; ++k) {
      if (!s.pinned[vert[k]]) continue;
      any = true;
      c = add(c, mul(ld(&s.q[3 * vert[k]]), w[k]));
    }
    if (!any) continue;
    for (int k = 0; k < 3; ++k) {
      const int p = vert[k];
      if (s.pinned[p]) continue;
      const V3 contrib = mul(c, -b.k * w[k]);
      double* slot = &s.bendRhs[3 * static_cast<size_t>(p)];
      slot[0] += contrib.x;
      slot[1] += contrib.y;
      slot[2] += contrib.z;
    }
  }
}

// ------------------------------------------------------------- ordering (minimum degree)
// Plain minimum-degree elimination on the scalar graph of L (ties → smaller vertex index).
// Eigen's AMD is not available here; this ordering only changes fill and rounding order.
std::vector<int32_t> minimumDegree(const oracle_sim& s) {
  const int n = s.n;
  std::vector<std::vector<int>> adj(n);
  for (int r = 0; r < n; ++r)
    for (int k = s.Lrow[r]; k < s.Lrow[r + 1]; ++k)
      if (s.Lcol[k] != r) adj[r].push_back(s.Lcol[k]);
  for (auto& a : adj) {
    std::sort(a.begin(), a.end());
    a.erase(std::unique(a.begin(), a.end()), a.end());
  }
  std::set<std::pair<int, int>> heap;
  for (int v = 0; v < n; ++v) heap.insert({static_cast<int>(adj[v].size()), v});
  std::vector<uint8_t> gone(n, 0);
  std::vector<int32_t> order;
  order.reserve(n);
  std::vector<int> merged;
  while (!heap.empty()) {
    const int v = heap.begin()->second;
    heap.erase(heap.begin());
    gone[v] = 1;
    order.push_back(v);
    const std::vector<int> nb = adj[v];
    for (int u : nb) {
      heap.erase({static_cast<int>(adj[u].size()), u});
      merged.clear();
      // adj[u] ∪ nb, minus u and v
      std::set_union(adj[u].begin(), adj[u].end(), nb.begin(), nb.end(), std::back_inserter(merged));
      adj[u].clear();
      for (int w : merged)
        if (w != u && w != v) adj[u].push_back(w);
      heap.insert({static_cast<int>(adj[u].size()), u});
    }
    adj[v].clear();
  }
  return order;
}

// ------------------------------------------------- LDLᵀ (Eigen SimplicialLDLT, up-looking)
// Follows the published up-looking LDL algorithm (T. A. Davis, "Algorithm 849: A concise
// sparse Cholesky factorization package") that Eigen 3.4.0's SimplicialCholesky implements:
// elimination tree + column counts, then row k of L by a sparse triangular solve whose
// pattern is visited in etree-reach (topological) order.
bool factorize(oracle_sim& s) {
  const int n = s.n;
  // Upper-stored columns of A = P·L·Pᵀ: column k holds rows i ≤ k, ascending.
  std::vector<int32_t> Ap(n + 1, 0), Ai;
  std::vector<double> Ax;
  {
    std::vector<std::vector<std::pair<int, double>>> cols(n);
    for (int r = 0; r < n; ++r)
      for (int k = s.Lrow[r]; k < s.Lrow[r + 1]; ++k) {
        const int c = s.Lcol[k];
        const int pr = s.iperm[r], pc = s.iperm[c];
        if (pr <= pc) cols[pc].push_back({pr, s.Lval[k]});
      }
    for (int k = 0; k < n; ++k) {
      std::sort(cols[k].begin(), cols[k].end());
      for (auto& e : cols[k]) {
        Ai.push_back(e.first);
        Ax.push_back(e.second);
      }
      Ap[k + 1] = static_cast<int32_t>(Ai.size());
    }
  }
  // symbolic: etree + column counts
  std::vector<int32_t> parent(n, -1), tags(n, 0), nz(n, 0);
  for (int k = 0; k < n; ++k) {
    parent[k] = -1;
    tags[k] = k;
    nz[k] = 0;
    for (int p = Ap[k]; p < Ap[k + 1]; ++p) {
      int i = Ai[p];
      if (i < k) {
        for (; tags[i] != k; i = parent[i]) {
          if (parent[i] == -1) parent[i] = k;
          nz[i]++;
          tags[i] = k;
        }
      }
    }
  }
  s.Fp.assign(n + 1, 0);
  for (int k = 0; k < n; ++k) s.Fp[k + 1] = s.Fp[k] + nz[k];
  s.Fi.assign(s.Fp[n], 0);
  s.Fx.assign(s.Fp[n], 0.0);
  s.D.assign(n, 0.0);
  std::vector<double> y(n, 0.0);
  std::vector<int32_t> pattern(n), cnt(n, 0);
  for (int k = 0; k < n; ++k) {
    y[k] = 0.0;
    int top = n;
    tags[k] = k;
    cnt[k] = 0;
    for (int p = Ap[k]; p < Ap[k + 1]; ++p) {
      int i = Ai[p];
      if (i <= k) {
        y[i] += Ax[p];
        int len = 0;
        for (; tags[i] != k; i = parent[i]) {
          pattern[len++] = i;
          tags[i] = k;
        }
        while (len > 0) pattern[--top] = pattern[--len];
      }
    }
    double d = y[k] * 1.0 + 0.0;  // shift scale 1, offset 0
    y[k] = 0.0;
    for (; top < n; ++top) {
      const int i = pattern[top];
      const double yi = y[i];
      y[i] = 0.0;
      const double lki = yi / s.D[i];
      const int p2 = s.Fp[i] + cnt[i];
      int p;
      for (p = s.Fp[i]; p < p2; ++p) y[s.Fi[p]] -= s.Fx[p] * yi;
      d -= lki * yi;
      s.Fi[p] = k;
      s.Fx[p] = lki;
      ++cnt[i];
    }
    s.D[k] = d;
    if (d == 0.0) return false;
  }
  s.dinv.resize(n);
  for (int k = 0; k < n; ++k) s.dinv[k] = 1.0 / s.D[k];
  return true;
}

void analyzeAndFactorize(oracle_sim& s, bool reanalyze) {
  assembleLhs(s);
  if (reanalyze) {
    if (!s.userPerm.empty()) s.perm = s.userPerm;
    else s.perm = minimumDegree(s);
    s.iperm.assign(s.n, 0);
    for (int k = 0; k < s.n; ++k) s.iperm[s.perm[k]] = k;
    s.analyzeCount += 1;
    s.analyzed = true;
  }
  s.factorReady = factorize(s);
  if (!s.factorReady) std::fprintf(stderr, "[oracle] LDL^T failed (zero pivot)\n");
  s.factorizeCount += 1;
}

// Solve one component (EigenDirectSolver.cpp:411-448, compact factor path).
void solveComponent(const oracle_sim& s, int c, const double* bb, double* xx, double* w) {
  const int n = s.n;
  for (int k = 0; k < n; ++k) w[k] = bb[3 * static_cast<size_t>(s.perm[k]) + c];
  for (int k = 0; k < n; ++k) {
    const double yk = w[k];
    for (int e = s.Fp[k]; e < s.Fp[k + 1]; ++e) w[s.Fi[e]] -= s.Fx[e] * yk;
  }
  for (int k = 0; k < n; ++k) w[k] *= s.dinv[k];
  for (int k = n - 1; k >= 0; --k) {
    double acc = w[k];
    for (int e = s.Fp[k]; e < s.Fp[k + 1]; ++e) acc -= s.Fx[e] * w[s.Fi[e]];
    w[k] = acc;
  }
  for (int k = 0; k < n; ++k) xx[3 * static_cast<size_t>(s.perm[k]) + c] = w[k];
}

// ----------------------------------------------- projection + scatter (DistanceTerm.cpp)
inline V3 projectEdge(const double* X, const Edge& e) {  // DistanceTerm.cpp:94-102
  const V3 raw = sub(ld(X + 3 * e.a), ld(X + 3 * e.b));
  const double len = length(raw);
  if (len <= kMinLength) return V3{0, 0, 0};
  return mul(raw, e.rest / len);
}
inline void scatterEdge(const oracle_sim& s, const Edge& e, const V3& d, double* out) {  // :121-152
  const bool ap = s.pinned[e.a] != 0, bp = s.pinned[e.b] != 0;
  if (ap && bp) return;
  const V3 c = mul(d, e.k);
  double* oa = out + 3 * static_cast<size_t>(e.a);
  double* ob = out + 3 * static_cast<size_t>(e.b);
  if (!ap) {
    oa[0] += c.x;
    oa[1] += c.y;
    oa[2] += c.z;
  }
  if (!bp) {
    ob[0] -= c.x;
    ob[1] -= c.y;
    ob[2] -= c.z;
  }
  if (ap && !bp) {
    const double* q = &s.q[3 * static_cast<size_t>(e.a)];
    ob[0] += e.k * q[0];
    ob[1] += e.k * q[1];
    ob[2] += e.k * q[2];
  } else if (bp && !ap) {
    const double* q = &s.q[3 * static_cast<size_t>(e.b)];
    oa[0] += e.k * q[0];
    oa[1] += e.k * q[1];
    oa[2] += e.k * q[2];
  }
}
// Fused projection + scatter, must run inside a parallel region (DistanceTerm.cpp:279-317).
void projectAndScatterInRegion(const oracle_sim& s, const double* base, double* bout,
                               const double* extra) {
  const long long dim = 3LL * s.n;
#pragma omp for
  for (long long i = 0; i < dim; ++i) bout[i] = base[i] + (extra ? extra[i] : 0.0);
  for (int c = 0; c < s.colorCount; ++c) {
    const long long b0 = s.cstart[c], b1 = s.cstart[c + 1];
    if (b0 == b1) continue;
#pragma omp for
    for (long long k = b0; k < b1; ++k) {
      const Edge& e = s.edges[s.corder[k]];
      scatterEdge(s, e, projectEdge(s.x.data(), e), bout);
    }
  }
}

// ------------------------------------------------------- residual (Integrator.cpp:92-263)
inline V3 bendForceAt(const oracle_sim& s, const double* X, int v) {
  V3 f{0, 0, 0};
  if (s.bstencils.empty()) return f;
  for (uint32_t k = s.bstart[v]; k < s.bstart[v + 1]; ++k) {
    const Bend& b = s.bends[s.bstencils[k]];
    const double* xa = X + 3 * b.a;
    const double* xb = X + 3 * b.b;
    const double* xc = X + 3 * b.c;
    const V3 second{xa[0] - 2.0 * xb[0] + xc[0], xa[1] - 2.0 * xb[1] + xc[1],
                    xa[2] - 2.0 * xb[2] + xc[2]};
    f = add(f, mul(second, -b.k * s.bweight[k]));
  }
  return f;
}
inline double vertexResidual(const oracle_sim& s, const double* X, double mass, double invH2, int v) {
  V3 f{0, 0, 0};
  for (uint32_t k = s.vstart[v]; k < s.vstart[v + 1]; ++k) {
    const Edge& e = s.edges[s.vedges[k]];
    const V3 rel = sub(ld(X + 3 * e.a), ld(X + 3 * e.b));
    const double len = length(rel);
    const V3 d = (len <= kMinLength) ? V3{} : mul(rel, e.rest / len);
    const V3 contrib = sub(mul(rel, e.k), mul(d, e.k));
    if (e.a == v) f = add(f, contrib);
    else f = sub(f, contrib);
  }
  f = add(f, bendForceAt(s, X, v));
  const V3 xv = ld(X + 3 * v);
  const V3 inertia = mul(sub(xv, ld(&s.predicted[3 * v])), mass * invH2);
  return length(add(inertia, f)) / mass;
}

void ensureBuffers(oracle_sim& s) {
  const size_t dim = 3 * static_cast<size_t>(s.n);
  s.predicted.resize(dim);
  s.before.resize(dim);
  s.prevPos.resize(dim);
  s.b.resize(dim);
  s.bBase.resize(dim);
  s.xSol.resize(dim);
  if (s.bends.empty()) s.bendRhs.clear();
}

// ----------------------------------------------------- stepOnce (Integrator.cpp:312-797)
// Refactorization by stamp and the bending RHS of the current pins (Integrator.cpp:341-372).
void refreshFactor(oracle_sim& s) {
  uint64_t now[4];
  computeStamp(s, now);
  const bool same = s.stampValid && now[0] == s.stampKey[0] && now[1] == s.stampKey[1] &&
                    now[2] == s.stampKey[2] && now[3] == s.stampKey[3];
  if (!same) {
    const uint64_t structureNow = computeStructureStamp(s);
    const bool re = !s.analyzed || structureNow != s.structureStamp;
    analyzeAndFactorize(s, re);
    s.structureStamp = structureNow;
    std::memcpy(s.stampKey, now, sizeof(now));
    s.stampValid = true;
    assembleBendingRhs(s);
  } else if (!s.bends.empty()) {
    assembleBendingRhs(s);
  }
}

// Whether iteration k blends, and its weight ω_k from ω_{k−1} (Integrator.cpp:590-617): mode 1
// ω = 2/(2−ρ²) at k = S+1, then 4/(4−ρ²ω); mode 2 ω_k = 1/(m + δ·cos(π(2j−1)/(2T))), j = k+1,
// T = the iteration budget, from k = 0.
bool chebBlends(const oracle_config& cfg, int k) {
  return cfg.cheb_mode == 2 || (cfg.cheb_mode == 1 && k > cfg.cheb_start);
}

double chebOmega(const oracle_config& cfg, int k, double prev) {
  if (cfg.cheb_mode == 1) {
    if (k == cfg.cheb_start + 1) return 2.0 / (2.0 - cfg.cheb_rho * cfg.cheb_rho);
    return 4.0 / (4.0 - cfg.cheb_rho * cfg.cheb_rho * prev);
  }
  const double pi = 3.14159265358979323846;
  const double T = static_cast<double>(cfg.max_iterations);
  const double j = static_cast<double>(k + 1);
  const double theta = pi * (2.0 * j - 1.0) / (2.0 * T);
  return 1.0 / (cfg.cheb_m + cfg.cheb_d * std::cos(theta));
}

int stepOnce(oracle_sim& s) {
  const oracle_config& cfg = s.cfg;
  const int n = s.n;
  const double h = cfg.dt;
  const double invH = 1.0 / h;
  const double invH2 = 1.0 / (h * h);
  ensureBuffers(s);
  refreshFactor(s);
  if (!s.factorReady) return -1;

  const int threads = cfg.threads > 0 ? cfg.threads : g_threads();
  const bool useParallel = threads > 1 && n >= 512 && static_cast<int>(s.edges.size()) >= 512;
  const bool wantResidual = cfg.residual_tolerance > 0.0;
  const int slots = std::max(1, threads);
  std::vector<double> pDiff(slots, 0.0), pScale(slots, 0.0), pRes(slots, 0.0);
  std::vector<int> pResV(slots, -1);
  std::vector<double> work(3 * static_cast<size_t>(n));
  s.converged = false;
  s.iterationsUsed = 0;
  const double* extra = s.bends.empty() ? nullptr : s.bendRhs.data();
  bool stop = false;

#pragma omp parallel num_threads(threads) if (useParallel)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    {  // predict (Integrator.cpp:447-463)
      const V3 gh2 = mul(V3{cfg.gravity[0], cfg.gravity[1], cfg.gravity[2]}, h * h);
#pragma omp for
      for (long long v = 0; v < n; ++v) {
        const V3 p = ld(&s.x[3 * v]);
        st(&s.before[3 * v], p);
        st(&s.predicted[3 * v], add(add(p, mul(ld(&s.v[3 * v]), h)), gh2));
        st(&s.prevPos[3 * v], p);
      }
    }
#pragma omp single
    {  // bBase = (M/h²) x̂ (Assembler.cpp:280-307)
      for (int v = 0; v < n; ++v) {
        const double mh2 = s.m[v] * invH2;
        for (int c = 0; c < 3; ++c) s.bBase[3 * v + c] = mh2 * s.predicted[3 * v + c];
      }
    }
    double omega = 1.0;  // over-relaxation weight, one copy per thread (Integrator.cpp:529)
    for (int k = 0; k < cfg.max_iterations; ++k) {
      projectAndScatterInRegion(s, s.bBase.data(), s.b.data(), extra);
#pragma omp for schedule(static, 1)
      for (int c = 0; c < 3; ++c) {
        for (int v = 0; v < n; ++v)  // applyPinRhsComponent (Assembler.cpp:319-332)
          if (s.pinned[v]) s.b[3 * v + c] = s.q[3 * v + c];
        solveComponent(s, c, s.b.data(), s.xSol.data(), work.data() + static_cast<size_t>(c) * n);
      }
      const bool blend = chebBlends(cfg, k);
      if (blend) omega = chebOmega(cfg, k, omega);
      double lDiff = 0.0, lScale = 0.0, lRes = 0.0;
      int lResV = -1;
#pragma omp for nowait
      for (long long v = 0; v < n; ++v) {  // unpack + scan + residual (Integrator.cpp:618-663)
        const V3 xNew = ld(&s.xSol[3 * v]);
        if (blend) {  // x = x_prev + (x_solve − x_prev)·ω; the residual stays that of x_solve (:633-641)
          const V3 xPrev = ld(&s.prevPos[3 * v]);
          const V3 xPut = add(xPrev, mul(sub(xNew, xPrev), omega));
          st(&s.x[3 * v], xPut);
          lDiff = smax(lDiff, maxAbsComponent(sub(xPut, xPrev)));
          st(&s.prevPos[3 * v], xPut);
        } else {
          st(&s.x[3 * v], xNew);
          lDiff = smax(lDiff, maxAbsComponent(sub(xNew, ld(&s.prevPos[3 * v]))));
          st(&s.prevPos[3 * v], xNew);
        }
        lScale = smax(lScale, maxAbsComponent(sub(ld(&s.predicted[3 * v]), ld(&s.before[3 * v]))));
        if (wantResidual) {
          const double mass = s.m[v];
          if (!s.pinned[v] && mass > 0.0) {
            const double r = vertexResidual(s, s.xSol.data(), mass, invH2, static_cast<int>(v));
            if (r > lRes) {
              lRes = r;
              lResV = static_cast<int>(v);
            }
          }
        }
      }
      if (tid < slots) {
        pDiff[tid] = lDiff;
        pScale[tid] = lScale;
        pRes[tid] = lRes;
        pResV[tid] = lResV;
      }
#pragma omp barrier
#pragma omp single
      {  // gate (Integrator.cpp:676-747)
        double diff = 0.0, scale = 0.0, res = 0.0;
        int resV = -1;
        const int used = useParallel ? slots : 1;
        for (int t = 0; t < used; ++t) {
          diff = smax(diff, pDiff[t]);
          scale = smax(scale, pScale[t]);
          if (pResV[t] >= 0 && (pRes[t] > res || (pRes[t] == res && resV < 0))) {
            res = pRes[t];
            resV = pResV[t];
          }
        }
        const V3 g{cfg.gravity[0], cfg.gravity[1], cfg.gravity[2]};
        scale = smax(scale, length(g) * h * h);
        const double rel = (scale > 0.0) ? diff / scale : diff;
        const bool absHit = (cfg.abs_tolerance > 0.0) && (diff <= cfg.abs_tolerance);
        const bool relHit = (cfg.rel_tolerance > 0.0) && (rel <= cfg.rel_tolerance);
        const double residual = wantResidual ? res : -1.0;
        bool resHit = false;
        if (cfg.residual_tolerance > 0.0) {
          const double gScale = smax(length(g), 1.0e-12);
          resHit = (residual <= cfg.residual_tolerance * gScale);
        }
        s.lastResidual = residual;
        if (s.trace) s.trace->push_back(residual);
        const bool conv = (cfg.residual_tolerance > 0.0) ? resHit : (absHit || relHit);
        s.converged = conv;
        if (conv) s.earlyExitCount += 1;
        s.iterationsUsed = k + 1;
        stop = conv;
      }
      if (stop) break;
    }
    {  // velocity + damping + pin resnap (Integrator.cpp:774-791)
      const double damp = 1.0 - cfg.velocity_damping;
#pragma omp for nowait
      for (long long v = 0; v < n; ++v) {
        V3 vn = mul(sub(ld(&s.x[3 * v]), ld(&s.before[3 * v])), damp * invH);
        if (s.pinned[v]) {
          vn = V3{0, 0, 0};
          st(&s.x[3 * v], ld(&s.q[3 * v]));
        }
        st(&s.v[3 * v], vn);
      }
    }
  }
  return s.iterationsUsed;
}

}  // namespace

// ---------------------------------------------------------------------- OBJ meshes
namespace {

struct ObjMesh {
  std::vector<V3> verts;
  std::vector<std::array<int, 3>> tris;
  std::vector<int> ea, eb;
  std::vector<double> rest, mass;
};

// Mesh::loadObj (core/mesh/Mesh.cpp:56-127): "v" lines read three numbers, "f" lines the integer
// before the first '/' of up to three tokens (1-based); a face with fewer than three is dropped, a
// token that is not a number fails the load. Indices outside the vertex list also fail here (the
// reference would read out of range). Edges: each triangle's (t0,t1), (t1,t2), (t2,t0) in order,
// skipping a == b and pairs already seen.
bool parseObj(const char* text, double density, ObjMesh& out) {
  std::istringstream in(text);
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ss(line);
    std::string tag;
    ss >> tag;
    if (tag == "v") {
      double x = 0, y = 0, z = 0;
      ss >> x >> y >> z;
      out.verts.push_back(V3{x, y, z});
    } else if (tag == "f") {
      std::array<int, 3> idx{};
      int count = 0;
      std::string token;
      while (count < 3 && ss >> token) {
        const std::size_t slash = token.find('/');
        const std::string first = slash == std::string::npos ? token : token.substr(0, slash);
        try {
          idx[count] = std::stoi(first) - 1;
        } catch (...) {
          return false;
        }
        ++count;
      }
      if (count == 3) out.tris.push_back(idx);
    }
  }
  const int n = static_cast<int>(out.verts.size());
  if (n == 0 || out.tris.empty()) return false;
  for (const auto& t : out.tris)
    for (int k = 0; k < 3; ++k)
      if (t[k] < 0 || t[k] >= n) return false;
  std::unordered_set<uint64_t> seen;
  for (const auto& t : out.tris) {
    for (int k = 0; k < 3; ++k) {
      const int a = t[k], b = t[(k + 1) % 3];
      if (a == b) continue;
      const uint64_t key = (static_cast<uint64_t>(static_cast<uint32_t>(std::min(a, b))) << 32) |
                           static_cast<uint32_t>(std::max(a, b));
      if (!seen.insert(key).second) continue;
      out.ea.push_back(a);
      out.eb.push_back(b);
      out.rest.push_back(length(sub(out.verts[b], out.verts[a])));
    }
  }
  // Mesh::computeMassesFromSurfaces (Mesh.cpp:129-153) with makeScene's density
  out.mass.assign(n, 0.0);
  const double rho = density > 0.0 ? density : 1.0;
  for (const auto& t : out.tris) {
    const V3 p0 = out.verts[t[0]], p1 = out.verts[t[1]], p2 = out.verts[t[2]];
    const V3 u = sub(p1, p0), w = sub(p2, p0);
    const V3 c{u.y * w.z - u.z * w.y, u.z * w.x - u.x * w.z, u.x * w.y - u.y * w.x};
    const double area = 0.5 * length(c);
    for (int k = 0; k < 3; ++k) out.mass[t[k]] += rho * area / 3.0;
  }
  double minPositive = 1e300;
  for (double m : out.mass)
    if (m > 1e-12) minPositive = std::min(minPositive, m);
  if (minPositive > 1e299) minPositive = 1.0;
  for (double& m : out.mass)
    if (m < 1e-12) m = minPositive;
  return true;
}

}  // namespace

extern "C" int oracle_obj_counts(const char* text, int* nv, int* ne) {
  ObjMesh m;
  if (!text || !parseObj(text, 1.0, m)) return -1;
  *nv = static_cast<int>(m.verts.size());
  *ne = static_cast<int>(m.ea.size());
  return 0;
}

extern "C" int oracle_make_obj(const char* text, double stiffness, double density, double* pos, double* mass,
                               uint8_t* pinned, int* edges, double* rest, double* k) {
  ObjMesh m;
  if (!text || !parseObj(text, density, m)) return -1;
  for (size_t v = 0; v < m.verts.size(); ++v) {
    pos[3 * v] = m.verts[v].x;
    pos[3 * v + 1] = m.verts[v].y;
    pos[3 * v + 2] = m.verts[v].z;
    mass[v] = m.mass[v];
    pinned[v] = 0;
  }
  for (size_t e = 0; e < m.ea.size(); ++e) {
    edges[2 * e] = m.ea[e];
    edges[2 * e + 1] = m.eb[e];
    rest[e] = m.rest[e];
    k[e] = stiffness;
  }
  return 0;
}

// ---------------------------------------------------------------------- grid generation
extern "C" void oracle_grid_counts(const oracle_grid_spec* g, int* nv, int* ne, int* nb) {
  const int nx = g->nx, ny = g->ny;
  int v = 0, e = 0, b = 0;
  if (nx >= 2 && ny >= 2) {
    v = nx * ny;
    e = 2 * nx * ny - nx - ny;
    if (g->shear_stiffness > 0.0) e += (nx - 1) * (ny - 1);
    if (g->bend_stiffness > 0.0 && !(nx < 3 && ny < 3)) {
      const int stride = g->bend_stride > 0 ? g->bend_stride : 1;
      const bool rows = g->bend_sampling == 0 || g->bend_sampling == 1;
      const bool cols = g->bend_sampling == 0 || g->bend_sampling == 2;
      const bool checker = g->bend_sampling == 3;
      for (int j = 0; j < ny; ++j)
        for (int i = 1; i + 1 < nx; ++i) {
          if ((i - 1) % stride != 0) continue;
          if (rows) ++b;
          if (checker && ((i + j) & 1) == 0) ++b;
        }
      for (int i = 0; i < nx; ++i)
        for (int j = 1; j + 1 < ny; ++j) {
          if ((j - 1) % stride != 0) continue;
          if (cols) ++b;
          if (checker && ((i + j) & 1) != 0) ++b;
        }
    }
  }
  *nv = v;
  *ne = e;
  *nb = b;
}

// makeGrid + computeMassesFromEdges + addShearDiagonals + addBendingStencils + default pins
// (core/mesh/Mesh.cpp:12-54,155-285; core/sim/Scene.cpp:39-177).
extern "C" int oracle_make_grid(const oracle_grid_spec* g, double* pos, double* mass, uint8_t* pinned,
                                int32_t* eab, double* erest, double* ek, int32_t* babc, double* bk) {
  const int nx = g->nx, ny = g->ny;
  if (nx < 2 || ny < 2) return -1;
  const int n = nx * ny;
  const double sp = g->spacing;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const int v = j * nx + i;
      pos[3 * v + 0] = static_cast<double>(i) * sp;
      pos[3 * v + 1] = 0.0;
      pos[3 * v + 2] = static_cast<double>(j) * sp;
    }
  int e = 0;
  auto addEdge = [&](int a, int b, double k) {
    const V3 d = sub(ld(pos + 3 * b), ld(pos + 3 * a));
    eab[2 * e] = a;
    eab[2 * e + 1] = b;
    erest[e] = length(d);
    ek[e] = k;
    ++e;
  };
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const int v = j * nx + i;
      if (i + 1 < nx) addEdge(v, v + 1, g->stiffness);
      if (j + 1 < ny) addEdge(v, v + nx, g->stiffness);
    }
  const int structural = e;
  // masses: edge-lumped rule on the structural edges (Mesh.cpp:155-181) or uniform
  if (g->mass_mode == 0) {
    const double density = g->density > 0.0 ? g->density : 1.0;
    for (int v = 0; v < n; ++v) mass[v] = 0.0;
    for (int k = 0; k < structural; ++k) {
      const double share = density * erest[k] * erest[k] * 0.5;
      mass[eab[2 * k]] += share;
      mass[eab[2 * k + 1]] += share;
    }
    double minPos = 1e300;
    for (int v = 0; v < n; ++v)
      if (mass[v] > 1e-12) minPos = std::min(minPos, mass[v]);
    if (minPos > 1e299) minPos = 1.0;
    for (int v = 0; v < n; ++v)
      if (mass[v] < 1e-12) mass[v] = minPos;
  } else {
    const double each = g->total_mass / static_cast<double>(n);
    for (int v = 0; v < n; ++v) mass[v] = each;
  }
  if (g->shear_stiffness > 0.0)
    for (int j = 0; j + 1 < ny; ++j)
      for (int i = 0; i + 1 < nx; ++i) addEdge(j * nx + i, (j + 1) * nx + (i + 1), g->shear_stiffness);
  int b = 0;
  if (g->bend_stiffness > 0.0 && !(nx < 3 && ny < 3)) {
    const int stride = g->bend_stride > 0 ? g->bend_stride : 1;
    const bool rows = g->bend_sampling == 0 || g->bend_sampling == 1;
    const bool cols = g->bend_sampling == 0 || g->bend_sampling == 2;
    const bool checker = g->bend_sampling == 3;
    auto add3 = [&](int a, int m, int c) {
      babc[3 * b] = a;
      babc[3 * b + 1] = m;
      babc[3 * b + 2] = c;
      bk[b] = g->bend_stiffness;
      ++b;
    };
    if (rows)
      for (int j = 0; j < ny; ++j)
        for (int i = 1; i + 1 < nx; ++i) {
          if ((i - 1) % stride != 0) continue;
          add3(j * nx + i - 1, j * nx + i, j * nx + i + 1);
        }
    if (cols)
      for (int i = 0; i < nx; ++i)
        for (int j = 1; j + 1 < ny; ++j) {
          if ((j - 1) % stride != 0) continue;
          add3((j - 1) * nx + i, j * nx + i, (j + 1) * nx + i);
        }
    if (checker) {
      for (int j = 0; j < ny; ++j)
        for (int i = 1; i + 1 < nx; ++i) {
          if ((i - 1) % stride != 0) continue;
          if (((i + j) & 1) != 0) continue;
          add3(j * nx + i - 1, j * nx + i, j * nx + i + 1);
        }
      for (int i = 0; i < nx; ++i)
        for (int j = 1; j + 1 < ny; ++j) {
          if ((j - 1) % stride != 0) continue;
          if (((i + j) & 1) == 0) continue;
          add3((j - 1) * nx + i, j * nx + i, (j + 1) * nx + i);
        }
    }
  }
  for (int v = 0; v < n; ++v) pinned[v] = 0;
  switch (g->pin_mode) {
    case 0: pinned[(ny - 1) * nx] = 1; pinned[(ny - 1) * nx + nx - 1] = 1; break;
    case 1: pinned[0] = 1; pinned[nx - 1] = 1; break;
    case 2: for (int i = 0; i < nx; ++i) pinned[(ny - 1) * nx + i] = 1; break;
    case 3: pinned[(ny - 1) * nx] = 1; break;
    default: break;
  }
  return 0;
}

// ------------------------------------------------------------------------------- C API
extern "C" oracle_sim* oracle_sim_create(int n, const double* pos, const double* vel,
                                         const double* mass, const uint8_t* pinned,
                                         const double* pinpos, int ne, const int32_t* eab,
                                         const double* erest, const double* ek, int nb,
                                         const int32_t* babc, const double* bk,
                                         const oracle_config* cfg, const int32_t* perm) {
  if (n < 0 || ne < 0 || nb < 0 || cfg == nullptr) return nullptr;
  auto* s = new oracle_sim();
  s->cfg = *cfg;
  s->n = n;
  s->x.assign(pos, pos + 3 * static_cast<size_t>(n));
  if (vel) s->v.assign(vel, vel + 3 * static_cast<size_t>(n));
  else s->v.assign(3 * static_cast<size_t>(n), 0.0);
  s->m.assign(mass, mass + n);
  s->pinned.assign(pinned, pinned + n);
  if (pinpos) s->q.assign(pinpos, pinpos + 3 * static_cast<size_t>(n));
  else s->q = s->x;  // refreshPinPositions (core/sim/Scene.cpp:202-207)
  for (int i = 0; i < ne; ++i) {
    if (eab[2 * i] < 0 || eab[2 * i] >= n || eab[2 * i + 1] < 0 || eab[2 * i + 1] >= n) {
      delete s;
      return nullptr;
    }
    s->edges.push_back(Edge{eab[2 * i], eab[2 * i + 1], erest[i], ek[i]});
  }
  for (int i = 0; i < nb; ++i) {
    for (int k = 0; k < 3; ++k)
      if (babc[3 * i + k] < 0 || babc[3 * i + k] >= n) {
        delete s;
        return nullptr;
      }
    s->bends.push_back(Bend{babc[3 * i], babc[3 * i + 1], babc[3 * i + 2], bk[i]});
  }
  if (perm) s->userPerm.assign(perm, perm + n);
  buildTopology(*s);
  ensureBuffers(*s);
  return s;
}

extern "C" void oracle_sim_destroy(oracle_sim* s) { delete s; }

extern "C" int oracle_sim_step(oracle_sim* s, int substeps, int32_t* iters, uint8_t* conv) {
  for (int k = 0; k < substeps; ++k) {
    const int used = stepOnce(*s);
    if (used < 0) return -1;
    if (iters) iters[k] = used;
    if (conv) conv[k] = s->converged ? 1 : 0;
  }
  return 0;
}

extern "C" int oracle_sim_step_traced(oracle_sim* s, int substeps, double* trace) {
  const int K = std::max(1, s->cfg.max_iterations);
  std::vector<double> t;
  s->trace = &t;
  int rc = 0;
  for (int k = 0; k < substeps && rc == 0; ++k) {
    t.clear();
    if (stepOnce(*s) < 0) rc = -1;
    for (int j = 0; j < K; ++j) trace[static_cast<size_t>(k) * K + j] = j < static_cast<int>(t.size()) ? t[j] : NAN;
  }
  s->trace = nullptr;
  return rc;
}

extern "C" void oracle_sim_get_state(const oracle_sim* s, double* pos, double* vel) {
  if (pos) std::memcpy(pos, s->x.data(), s->x.size() * sizeof(double));
  if (vel) std::memcpy(vel, s->v.data(), s->v.size() * sizeof(double));
}
extern "C" void oracle_sim_set_state(oracle_sim* s, const double* pos, const double* vel) {
  if (pos) std::memcpy(s->x.data(), pos, s->x.size() * sizeof(double));
  if (vel) std::memcpy(s->v.data(), vel, s->v.size() * sizeof(double));
}
extern "C" void oracle_sim_set_pin_positions(oracle_sim* s, const double* q) {
  std::memcpy(s->q.data(), q, s->q.size() * sizeof(double));
}
extern "C" void oracle_sim_set_config(oracle_sim* s, const oracle_config* cfg) { s->cfg = *cfg; }
extern "C" void oracle_sim_set_edge_stiffness(oracle_sim* s, const double* ek) {
  for (size_t i = 0; i < s->edges.size(); ++i) s->edges[i].k = ek[i];
}

extern "C" double oracle_sim_nonlinear_residual(oracle_sim* s) {
  // Serial form (Integrator.cpp:113-205): force accumulated in global edge order, then bends.
  const int n = s->n;
  const double invH2 = 1.0 / (s->cfg.dt * s->cfg.dt);
  std::vector<double> force(3 * static_cast<size_t>(n), 0.0);
  for (const Edge& e : s->edges) {
    const V3 rel = sub(ld(&s->x[3 * e.a]), ld(&s->x[3 * e.b]));
    const double len = length(rel);
    const V3 d = (len <= kMinLength) ? V3{} : mul(rel, e.rest / len);
    const V3 c = sub(mul(rel, e.k), mul(d, e.k));
    for (int k = 0; k < 3; ++k) {
      force[3 * e.a + k] += (&c.x)[k];
      force[3 * e.b + k] -= (&c.x)[k];
    }
  }
  if (!s->bstencils.empty())
    for (int v = 0; v < n; ++v) {
      const V3 fb = bendForceAt(*s, s->x.data(), v);
      force[3 * v] += fb.x;
      force[3 * v + 1] += fb.y;
      force[3 * v + 2] += fb.z;
    }
  double worst = 0.0;
  for (int v = 0; v < n; ++v) {
    if (s->pinned[v]) continue;
    const double mass = s->m[v];
    if (mass <= 0.0) continue;
    const V3 inertia = mul(sub(ld(&s->x[3 * v]), ld(&s->predicted[3 * v])), mass * invH2);
    const V3 tot{inertia.x + force[3 * v], inertia.y + force[3 * v + 1], inertia.z + force[3 * v + 2]};
    const double r = length(tot) / mass;
    if (r > worst) worst = r;
  }
  return worst;
}

namespace {
double surrogateEnergy(const oracle_sim& s) {  // Integrator.cpp:804-826
  double e = 0.0;
  for (const Edge& ed : s.edges) {
    const double len = length(sub(ld(&s.x[3 * ed.a]), ld(&s.x[3 * ed.b])));
    const double d = len - ed.rest;
    e += 0.5 * ed.k * d * d;
  }
  for (const Bend& b : s.bends) {
    const double* pa = &s.x[3 * b.a];
    const double* pb = &s.x[3 * b.b];
    const double* pc = &s.x[3 * b.c];
    const V3 second{pa[0] - 2.0 * pb[0] + pc[0], pa[1] - 2.0 * pb[1] + pc[1], pa[2] - 2.0 * pb[2] + pc[2]};
    e += 0.5 * b.k * dot(second, second);
  }
  return e;
}
}  // namespace

extern "C" void oracle_sim_stats(oracle_sim* s, oracle_stats* o) {
  o->last_residual = s->lastResidual;
  o->iterations_used = s->iterationsUsed;
  o->converged = s->converged ? 1 : 0;
  o->early_exit_count = s->earlyExitCount;
  o->factorize_count = s->factorizeCount;
  o->analyze_count = s->analyzeCount;
  o->color_count = s->colorCount;
  o->matrix_nnz = static_cast<int64_t>(s->Lval.size());
  o->factor_nnz = s->Fp.empty() ? 0 : s->Fp.back();
  double worst = 0.0, sum = 0.0;  // Mesh.cpp:351-372
  for (const Edge& e : s->edges) {
    const double len = length(sub(ld(&s->x[3 * e.a]), ld(&s->x[3 * e.b])));
    if (e.rest <= 0.0) continue;
    const double r = std::fabs(len - e.rest) / e.rest;
    worst = std::max(worst, r);
    sum += r;
  }
  o->max_strain = worst;
  o->mean_strain = s->edges.empty() ? 0.0 : sum / static_cast<double>(s->edges.size());
  const double el = surrogateEnergy(*s);
  double kin = 0.0, grav = 0.0, vmax = 0.0;  // Integrator.cpp:828-846
  const V3 g{s->cfg.gravity[0], s->cfg.gravity[1], s->cfg.gravity[2]};
  for (int v = 0; v < s->n; ++v) {
    const V3 vel = ld(&s->v[3 * v]);
    kin += 0.5 * s->m[v] * dot(vel, vel);
    grav -= s->m[v] * dot(g, ld(&s->x[3 * v]));
    vmax = std::max(vmax, length(vel));
  }
  o->elastic_energy = el;
  o->total_energy = kin + el + grav;
  o->max_speed = vmax;
}

extern "C" int64_t oracle_sim_factor(oracle_sim* s, int32_t* perm, int32_t* colptr, int32_t* rowidx,
                                     double* val, double* dinv) {
  if (!s->factorReady) {
    uint64_t now[4];
    computeStamp(*s, now);
    analyzeAndFactorize(*s, true);
    s->structureStamp = computeStructureStamp(*s);
    std::memcpy(s->stampKey, now, sizeof(now));
    s->stampValid = true;
    assembleBendingRhs(*s);
  }
  const int n = s->n;
  if (perm) std::memcpy(perm, s->perm.data(), n * sizeof(int32_t));
  if (colptr) std::memcpy(colptr, s->Fp.data(), (n + 1) * sizeof(int32_t));
  if (rowidx) std::memcpy(rowidx, s->Fi.data(), s->Fi.size() * sizeof(int32_t));
  if (val) std::memcpy(val, s->Fx.data(), s->Fx.size() * sizeof(double));
  if (dinv) std::memcpy(dinv, s->dinv.data(), n * sizeof(double));
  return s->Fp.empty() ? 0 : s->Fp.back();
}

extern "C" int64_t oracle_sim_matrix(oracle_sim* s, int32_t* rowptr, int32_t* colidx, double* val) {
  if (s->Lrow.empty()) assembleLhs(*s);
  if (rowptr) std::memcpy(rowptr, s->Lrow.data(), s->Lrow.size() * sizeof(int32_t));
  if (colidx) std::memcpy(colidx, s->Lcol.data(), s->Lcol.size() * sizeof(int32_t));
  if (val) std::memcpy(val, s->Lval.data(), s->Lval.size() * sizeof(double));
  return static_cast<int64_t>(s->Lval.size());
}

extern "C" int oracle_sim_solve(oracle_sim* s, const double* b, double* x) {
  if (!s->factorReady) oracle_sim_factor(s, nullptr, nullptr, nullptr, nullptr, nullptr);
  if (!s->factorReady) return -1;
  std::vector<double> w(s->n);
  for (int c = 0; c < 3; ++c) solveComponent(*s, c, b, x, w.data());
  return 0;
}

// Spectrum of the linearised PD iteration (_verify/iteration_spectrum.cpp:126-338) at the current
// positions: T = I − A⁻¹(M/h² + N), N = Σ_e κ_e A_eᵀ(n_e n_eᵀ)A_e with n_e = unit(x_a − x_b)
// (:133-142, :229-263), pinned rows of the right-hand side zeroed (:255-262). Power iteration from
// the reference's start vector — std::mt19937(12345), (rng() % 2000)/1000 − 1 on every free
// component in vertex order (:319-324) — recording ‖y‖/‖x‖ for the last 20 iterations (:282-306):
// out[0] = ρ(T) (last estimate), out[1] = the one before, out[2] = λ_max(B) for B = I − T from the
// same start, out[3] = the one before. Bending stencils (which the reference's tool refuses, :113-116)
// enter as their full term k·A_sᵀA_s: their projection is constant, so B gains that block of A.
extern "C" int oracle_sim_spectrum(oracle_sim* s, int iters, double* out) {
  if (!s->factorReady) oracle_sim_factor(s, nullptr, nullptr, nullptr, nullptr, nullptr);
  if (!s->factorReady) return -1;
  const int n = s->n, dim = 3 * n;
  const double invH2 = 1.0 / (s->cfg.dt * s->cfg.dt);
  std::vector<V3> nE(s->edges.size());
  for (size_t c = 0; c < s->edges.size(); ++c) {
    const Edge& e = s->edges[c];
    const V3 rel = sub(ld(&s->x[3 * static_cast<size_t>(e.a)]), ld(&s->x[3 * static_cast<size_t>(e.b)]));
    const double len = length(rel);
    nE[c] = (len > 0.0) ? mul(rel, 1.0 / len) : V3{0, 0, 0};
  }
  std::vector<double> rhs(dim), sol(dim), w(n);
  auto applyInertiaPlusN = [&](const std::vector<double>& x) {
    std::fill(rhs.begin(), rhs.end(), 0.0);
    for (int v = 0; v < n; ++v) {
      if (s->pinned[v]) continue;
      const double d = s->m[v] * invH2;
      for (int c = 0; c < 3; ++c) rhs[3 * v + c] = d * x[3 * v + c];
    }
    for (size_t c = 0; c < s->edges.size(); ++c) {
      const Edge& e = s->edges[c];
      const V3& g = nE[c];
      if (e.k == 0.0 || (g.x == 0.0 && g.y == 0.0 && g.z == 0.0)) continue;
      const V3 rel{x[3 * e.a] - x[3 * e.b], x[3 * e.a + 1] - x[3 * e.b + 1], x[3 * e.a + 2] - x[3 * e.b + 2]};
      const double dot = g.x * rel.x + g.y * rel.y + g.z * rel.z;
      const V3 sc = mul(g, e.k * dot);
      rhs[3 * e.a] += sc.x;
      rhs[3 * e.a + 1] += sc.y;
      rhs[3 * e.a + 2] += sc.z;
      rhs[3 * e.b] -= sc.x;
      rhs[3 * e.b + 1] -= sc.y;
      rhs[3 * e.b + 2] -= sc.z;
    }
    for (int v = 0; v < n; ++v) {  // k·A_sᵀA_s of the stencils at v, in stencil order
      if (s->pinned[v] || s->bstencils.empty()) continue;
      for (uint32_t k = s->bstart[v]; k < s->bstart[v + 1]; ++k) {
        const Bend& b = s->bends[s->bstencils[k]];
        const double fac = -b.k * s->bweight[k];
        for (int c = 0; c < 3; ++c)
          rhs[3 * v + c] -= fac * (x[3 * b.a + c] - 2.0 * x[3 * b.b + c] + x[3 * b.c + c]);
      }
    }
    for (int v = 0; v < n; ++v)
      if (s->pinned[v]) rhs[3 * v] = rhs[3 * v + 1] = rhs[3 * v + 2] = 0.0;
  };
  auto norm = [](const std::vector<double>& a) {
    double acc = 0.0;
    for (double t : a) acc += t * t;
    return std::sqrt(acc);
  };
  auto power = [&](bool plain, std::vector<double> x, double* last, double* prev) {
    std::vector<double> y(dim);
    *last = *prev = 0.0;
    for (int it = 0; it < iters; ++it) {
      applyInertiaPlusN(x);
      for (int c = 0; c < 3; ++c) solveComponent(*s, c, rhs.data(), sol.data(), w.data());
      for (int i = 0; i < dim; ++i) y[i] = plain ? x[i] - sol[i] : sol[i];
      const double ny = norm(y);
      if (ny <= 0.0) break;
      if (it >= iters - 20) {
        *prev = *last;
        *last = ny / norm(x);
      }
      for (int i = 0; i < dim; ++i) x[i] = y[i] / ny;
    }
  };
  std::vector<double> x0(dim, 0.0);
  std::mt19937 rng(12345);
  for (int v = 0; v < n; ++v) {
    if (s->pinned[v]) continue;
    for (int d = 0; d < 3; ++d) x0[3 * v + d] = static_cast<double>(rng() % 2000) / 1000.0 - 1.0;
  }
  power(true, x0, &out[0], &out[1]);
  power(false, x0, &out[2], &out[3]);
  return 0;
}

extern "C" int oracle_sim_rhs(oracle_sim* s, const double* base, double* b, int overwrite_pins) {
  if (!s->factorReady) oracle_sim_factor(s, nullptr, nullptr, nullptr, nullptr, nullptr);
  assembleBendingRhs(*s);
  const double* extra = s->bends.empty() ? nullptr : s->bendRhs.data();
#pragma omp parallel num_threads(1)
  { projectAndScatterInRegion(*s, base, b, extra); }
  if (overwrite_pins)
    for (int v = 0; v < s->n; ++v)
      if (s->pinned[v])
        for (int c = 0; c < 3; ++c) b[3 * v + c] = s->q[3 * v + c];
  return 0;
}

extern "C" int oracle_sim_coloring(oracle_sim* s, uint32_t* color_of, uint32_t* start, uint32_t* order,
                                   uint32_t* vstart, uint32_t* vedges) {
  if (color_of) std::memcpy(color_of, s->colorOf.data(), s->colorOf.size() * 4);
  if (start) std::memcpy(start, s->cstart.data(), s->cstart.size() * 4);
  if (order) std::memcpy(order, s->corder.data(), s->corder.size() * 4);
  if (vstart) std::memcpy(vstart, s->vstart.data(), s->vstart.size() * 4);
  if (vedges) std::memcpy(vedges, s->vedges.data(), s->vedges.size() * 4);
  return s->colorCount;
}

extern "C" void oracle_sim_bend_rhs(oracle_sim* s, double* out) {
  assembleBendingRhs(*s);
  if (s->bendRhs.empty()) std::memset(out, 0, 3 * static_cast<size_t>(s->n) * sizeof(double));
  else std::memcpy(out, s->bendRhs.data(), s->bendRhs.size() * sizeof(double));
}

extern "C" void oracle_project_one(const double* pa, const double* pb, double rest, double* out) {
  const V3 d = sub(ld(pa), ld(pb));
  const double len = length(d);
  if (len <= kMinLength) {
    out[0] = out[1] = out[2] = 0.0;
    return;
  }
  st(out, mul(d, rest / len));
}

// ------------------------------------------------------------ reference gradient (adjoint)
// The differentiable substep: the reference's stepOnce with the iteration count fixed at
// max_iterations (the gate is not differentiable) and an external force f entering the
// prediction as x̂ = x + h·v + h²·g + h²·f/m. Serial FP64, summation in edge order.
namespace {

struct GradWork {
  std::vector<double> xhat, b, col, w;
};

// One substep from (X, V) in place; iterates[k] (K+1 vectors of 3n) receives x^0..x^K if given.
void forwardSubstep(oracle_sim& s, const double* force, std::vector<double>& X, std::vector<double>& V,
                    std::vector<double>* iterates, GradWork& g) {
  const int n = s.n, K = s.cfg.max_iterations;
  const size_t dim = 3 * static_cast<size_t>(n);
  const double h = s.cfg.dt, invH2 = 1.0 / (h * h), h2 = h * h;
  const double damp = (1.0 - s.cfg.velocity_damping) * (1.0 / h);
  g.xhat.assign(dim, 0.0);
  g.b.assign(dim, 0.0);
  g.col.assign(dim, 0.0);
  g.w.assign(n, 0.0);
  for (int v = 0; v < n; ++v)
    for (int c = 0; c < 3; ++c) {
      const size_t i = 3 * static_cast<size_t>(v) + c;
      double xh = (X[i] + V[i] * h) + s.cfg.gravity[c] * h2;
      if (force && s.m[v] > 0.0) xh += force[i] * (h2 / s.m[v]);
      g.xhat[i] = xh;
    }
  std::vector<double> xk = X, xn = X;
  if (iterates) std::copy(xk.begin(), xk.end(), iterates[0].begin());
  for (int k = 0; k < K; ++k) {
    for (int v = 0; v < n; ++v)
      for (int c = 0; c < 3; ++c) {
        const size_t i = 3 * static_cast<size_t>(v) + c;
        g.b[i] = s.m[v] * invH2 * g.xhat[i] + (s.bendRhs.empty() ? 0.0 : s.bendRhs[i]);
      }
    for (const Edge& e : s.edges) scatterEdge(s, e, projectEdge(xk.data(), e), g.b.data());
    for (int v = 0; v < n; ++v)
      if (s.pinned[v])
        for (int c = 0; c < 3; ++c) g.b[3 * v + c] = s.q[3 * v + c];
    for (int c = 0; c < 3; ++c) solveComponent(s, c, g.b.data(), g.col.data(), g.w.data());
    xk = g.col;
    if (iterates) std::copy(xk.begin(), xk.end(), iterates[k + 1].begin());
  }
  for (int v = 0; v < n; ++v)
    for (int c = 0; c < 3; ++c) {
      const size_t i = 3 * static_cast<size_t>(v) + c;
      if (s.pinned[v]) {
        V[i] = 0.0;
        X[i] = s.q[i];
      } else {
        V[i] = (xk[i] - xn[i]) * damp;
        X[i] = xk[i];
      }
    }
}

}  // namespace

extern "C" int oracle_sim_gradient(oracle_sim* s, int substeps, const double* targets, const double* force,
                                   double* loss, double* dkappa, double* dv0, double* dforce) {
  ensureBuffers(*s);
  refreshFactor(*s);
  // the over-relaxed iteration is not differentiated
  if (!s->factorReady || substeps < 0 || s->cfg.cheb_mode != 0) return -1;
  const int n = s->n, K = s->cfg.max_iterations, ne = static_cast<int>(s->edges.size());
  const size_t dim = 3 * static_cast<size_t>(n);
  const double h = s->cfg.dt, invH2 = 1.0 / (h * h), h2 = h * h;
  const double damp = (1.0 - s->cfg.velocity_damping) * (1.0 / h);
  GradWork g;
  // forward with a checkpoint (x, v) at the start of every substep
  std::vector<std::vector<double>> ckX(substeps), ckV(substeps);
  std::vector<double> X = s->x, V = s->v;
  for (int step = 0; step < substeps; ++step) {
    ckX[step] = X;
    ckV[step] = V;
    forwardSubstep(*s, force, X, V, nullptr, g);
  }
  int nfree = 0;
  for (int v = 0; v < n; ++v) nfree += s->pinned[v] ? 0 : 1;
  double l = 0.0;
  std::vector<double> xb(dim, 0.0), vb(dim, 0.0), fb(dim, 0.0), kb(ne, 0.0);
  for (int v = 0; v < n; ++v) {
    if (s->pinned[v]) continue;
    for (int c = 0; c < 3; ++c) {
      const size_t i = 3 * static_cast<size_t>(v) + c;
      const double d = X[i] - targets[i];
      l += d * d;
      xb[i] = 2.0 * d / nfree;
    }
  }
  if (loss) *loss = (nfree > 0) ? l / nfree : 0.0;
  if (!dkappa && !dv0 && !dforce) return 0;
  // reverse, substep by substep, recomputing each substep's iterates from its checkpoint
  std::vector<std::vector<double>> it(K + 1, std::vector<double>(dim));
  std::vector<double> xkb(dim), xnb(dim), xhb(dim), lam(dim), rhs(dim);
  for (int step = substeps - 1; step >= 0; --step) {
    X = ckX[step];
    V = ckV[step];
    forwardSubstep(*s, force, X, V, it.data(), g);  // g.xhat holds x̂ of this substep
    for (int v = 0; v < n; ++v)
      for (int c = 0; c < 3; ++c) {
        const size_t i = 3 * static_cast<size_t>(v) + c;
        const bool p = s->pinned[v] != 0;
        xkb[i] = p ? 0.0 : xb[i] + damp * vb[i];  // x' = x^K, v' = (x^K − x_n)·damp
        xnb[i] = p ? 0.0 : -damp * vb[i];
        xhb[i] = 0.0;
      }
    for (int k = K - 1; k >= 0; --k) {
      for (size_t i = 0; i < dim; ++i) rhs[i] = xkb[i];  // pinned rows are zero
      for (int c = 0; c < 3; ++c) solveComponent(*s, c, rhs.data(), lam.data(), g.w.data());
      for (int v = 0; v < n; ++v) {
        if (s->pinned[v]) continue;
        for (int c = 0; c < 3; ++c) xhb[3 * v + c] += s->m[v] * invH2 * lam[3 * v + c];
      }
      std::fill(xkb.begin(), xkb.end(), 0.0);
      const double* xk = it[k].data();
      const double* xk1 = it[k + 1].data();
      for (int e = 0; e < ne; ++e) {
        const Edge& ed = s->edges[e];
        const bool ap = s->pinned[ed.a] != 0, bp = s->pinned[ed.b] != 0;
        if (ap && bp) continue;
        const V3 la = ap ? V3{} : ld(&lam[3 * ed.a]), lb = bp ? V3{} : ld(&lam[3 * ed.b]);
        const V3 le = sub(la, lb);
        const V3 rel = sub(ld(xk + 3 * ed.a), ld(xk + 3 * ed.b));
        const double len = length(rel);
        V3 d{}, jl{};
        if (len > kMinLength) {
          d = mul(rel, ed.rest / len);
          const V3 u = mul(rel, 1.0 / len);
          jl = mul(sub(le, mul(u, dot(u, le))), ed.rest / len);  // ∂d/∂rel · λ_e (symmetric)
        }
        const V3 rel1 = sub(ld(xk1 + 3 * ed.a), ld(xk1 + 3 * ed.b));
        kb[e] += dot(le, sub(d, rel1));
        const V3 gk = mul(jl, ed.k);
        if (!ap) st(&xkb[3 * ed.a], add(ld(&xkb[3 * ed.a]), gk));
        if (!bp) st(&xkb[3 * ed.b], sub(ld(&xkb[3 * ed.b]), gk));
      }
    }
    // x^0 = x_n; x̂ = x_n + h·v_n + h²·g + h²·f/m
    for (int v = 0; v < n; ++v)
      for (int c = 0; c < 3; ++c) {
        const size_t i = 3 * static_cast<size_t>(v) + c;
        if (s->pinned[v]) {
          xb[i] = vb[i] = 0.0;
          continue;
        }
        xb[i] = xnb[i] + xkb[i] + xhb[i];
        vb[i] = h * xhb[i];
        if (s->m[v] > 0.0) fb[i] += (h2 / s->m[v]) * xhb[i];
      }
  }
  if (dkappa) std::copy(kb.begin(), kb.end(), dkappa);
  if (dv0) std::copy(vb.begin(), vb.end(), dv0);
  if (dforce) std::copy(fb.begin(), fb.end(), dforce);
  return 0;
}
