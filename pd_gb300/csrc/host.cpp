// host.cpp — one-time host preparation of a cloth instance (see host.hpp).
#include "host.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <cctype>
#include <cstdlib>
#include <numeric>
#include <string>

namespace pdg {

namespace {
constexpr uint32_t kUncolored = 0xFFFFFFFFu;

// Edge priority for the colouring: splitmix64 finaliser of the edge index
// (core/mesh/ConstraintColoring.cpp:23-31). Colours must match the reference bit for bit,
// because the colour order is the per-vertex summation order of the scatter.
uint32_t edgePriority(uint32_t e) {
  uint64_t x = static_cast<uint64_t>(e) * 0x9E3779B97F4A7C15ULL + 0x2545F4914F6CDD1DULL;
  x ^= x >> 30;
  x *= 0xBF58476D1CE4E5B9ULL;
  x ^= x >> 27;
  x *= 0x94D049BB133111EBULL;
  x ^= x >> 31;
  return static_cast<uint32_t>(x >> 32);
}

uint64_t hashCombine(uint64_t h, uint64_t v) {  // Assembler.cpp:104-107
  h ^= v + 0x9e3779b97f4a7c15ULL + (h << 6) + (h >> 2);
  return h;
}
uint64_t bitsOf(double d) {
  uint64_t u;
  std::memcpy(&u, &d, sizeof(u));
  return u;
}
}  // namespace

std::string validateScene(const Scene& s) {
  if (s.n <= 0) return "scene has no vertices";
  const size_t n = static_cast<size_t>(s.n);
  if (s.x.size() != 3 * n || s.v.size() != 3 * n || s.q.size() != 3 * n || s.m.size() != n ||
      s.pinned.size() != n)
    return "vertex arrays are not sized to the vertex count";
  for (size_t i = 0; i < s.edges.size(); ++i) {
    const Edge& e = s.edges[i];
    if (e.a < 0 || e.a >= s.n || e.b < 0 || e.b >= s.n) return "edge " + std::to_string(i) + " has an endpoint out of range";
    if (e.a == e.b) return "edge " + std::to_string(i) + " joins a vertex to itself";
  }
  for (size_t i = 0; i < s.bends.size(); ++i) {
    const Bend& b = s.bends[i];
    if (b.a < 0 || b.a >= s.n || b.b < 0 || b.b >= s.n || b.c < 0 || b.c >= s.n)
      return "bend stencil " + std::to_string(i) + " has a vertex out of range";
  }
  for (double v : s.x)
    if (!std::isfinite(v)) return "positions contain a non-finite value";
  return {};
}

// ------------------------------------------------------------------------------ topology
void buildTopology(const Scene& s, Topology& t) {
  const int nv = s.n;
  const int ne = static_cast<int>(s.edges.size());
  // edge-order incidence (ConstraintColoring.cpp:35-54)
  t.rstart.assign(nv + 1, 0);
  for (const Edge& e : s.edges) {
    t.rstart[e.a + 1] += 1;
    t.rstart[e.b + 1] += 1;
  }
  for (int v = 0; v < nv; ++v) t.rstart[v + 1] += t.rstart[v];
  t.rinc.assign(2 * static_cast<size_t>(ne), 0);
  {
    std::vector<int32_t> cur(t.rstart.begin(), t.rstart.end() - 1);
    for (int i = 0; i < ne; ++i) {
      t.rinc[cur[s.edges[i].a]++] = (i << 1) | 0;
      t.rinc[cur[s.edges[i].b]++] = (i << 1) | 1;
    }
  }
  // Jones–Plassmann colouring with the smallest free colour (ConstraintColoring.cpp:121-259)
  t.colorOf.assign(ne, kUncolored);
  int maxColor = -1;
  if (ne > 0) {
    std::vector<uint32_t> prio(ne);
    for (int i = 0; i < ne; ++i) prio[i] = edgePriority(static_cast<uint32_t>(i));
    auto neighbours = [&](int e, auto&& fn) {
      const int ends[2] = {s.edges[e].a, s.edges[e].b};
      for (int v : ends)
        for (int k = t.rstart[v]; k < t.rstart[v + 1]; ++k) {
          const int f = t.rinc[k] >> 1;
          if (f != e) fn(f);
        }
    };
    std::vector<int> remaining(ne), next;
    std::iota(remaining.begin(), remaining.end(), 0);
    std::vector<uint32_t> cand(ne, kUncolored);
    while (!remaining.empty()) {
      for (int e : remaining) {
        cand[e] = kUncolored;
        bool allColored = true, localMax = true;
        neighbours(e, [&](int f) {
          if (t.colorOf[f] == kUncolored) {
            allColored = false;
            if (prio[f] > prio[e] || (prio[f] == prio[e] && f < e)) localMax = false;
          }
        });
        if (!allColored && !localMax) continue;
        uint32_t pick = 0;
        for (bool clash = true; clash;) {
          clash = false;
          neighbours(e, [&](int f) {
            if (!clash && t.colorOf[f] == pick) {
              clash = true;
              ++pick;
            }
          });
        }
        cand[e] = pick;
      }
      next.clear();
      for (int e : remaining) {
        if (cand[e] != kUncolored) {
          t.colorOf[e] = cand[e];
          maxColor = std::max(maxColor, static_cast<int>(cand[e]));
        } else {
          next.push_back(e);
        }
      }
      if (next.size() == remaining.size()) break;  // cannot happen: the top-priority edge always colours
      remaining.swap(next);
    }
  }
  t.colorCount = maxColor + 1;
  // colour-order incidence: each vertex meets each colour at most once, so sorting a vertex's
  // incident edges by colour reproduces the per-vertex order of the colour-by-colour scatter.
  t.sstart = t.rstart;
  t.sinc = t.rinc;
  for (int v = 0; v < nv; ++v)
    std::sort(t.sinc.begin() + t.sstart[v], t.sinc.begin() + t.sstart[v + 1],
              [&](int32_t p, int32_t q) { return t.colorOf[p >> 1] < t.colorOf[q >> 1]; });
  // bend incidence in stencil order (ConstraintColoring.cpp:82-119) with (-k)·w_v precomputed
  const int nb = static_cast<int>(s.bends.size());
  t.bstart.assign(nv + 1, 0);
  for (const Bend& b : s.bends) {
    t.bstart[b.a + 1] += 1;
    t.bstart[b.b + 1] += 1;
    t.bstart[b.c + 1] += 1;
  }
  for (int v = 0; v < nv; ++v) t.bstart[v + 1] += t.bstart[v];
  t.binc.assign(3 * static_cast<size_t>(nb), 0);
  t.bfac.assign(3 * static_cast<size_t>(nb), 0.0);
  std::vector<int32_t> cur(t.bstart.begin(), t.bstart.end() - 1);
  const double w[3] = {1.0, -2.0, 1.0};
  for (int i = 0; i < nb; ++i) {
    const int vert[3] = {s.bends[i].a, s.bends[i].b, s.bends[i].c};
    for (int k = 0; k < 3; ++k) {
      const int slot = cur[vert[k]]++;
      t.binc[slot] = i;
      t.bfac[slot] = -s.bends[i].k * w[k];
    }
  }
}

// ------------------------------------------------------------------------------ assembly
// Ã with L = Ã ⊗ I₃ (Assembler.cpp:139-278). The triplet sequence and the left-to-right sum of
// duplicates follow the reference (Eigen's setFromTriplets sums duplicates in insertion order),
// so every entry has the reference's bits.
void assembleMatrix(const Scene& s, double dt, ScalarMatrix& L) {
  struct T {
    int32_t r, c;
    double v;
  };
  const int n = s.n;
  const double invDt2 = 1.0 / (dt * dt);
  std::vector<T> t;
  t.reserve(2 * static_cast<size_t>(n) + 4 * s.edges.size() + 9 * s.bends.size());
  auto pin = [&](int v) { return s.pinned[v] != 0; };
  for (int v = 0; v < n; ++v) t.push_back({v, v, s.m[v] * invDt2});
  for (const Edge& e : s.edges) {
    const bool ap = pin(e.a), bp = pin(e.b);
    if (ap && bp) continue;
    if (!ap) t.push_back({e.a, e.a, e.k});
    if (!bp) t.push_back({e.b, e.b, e.k});
    if (!ap && !bp) {
      t.push_back({e.a, e.b, -e.k});
      t.push_back({e.b, e.a, -e.k});
    }
  }
  const double w[3] = {1.0, -2.0, 1.0};
  for (const Bend& b : s.bends) {
    if (b.k == 0.0) continue;
    if (pin(b.a) && pin(b.b) && pin(b.c)) continue;
    const int vert[3] = {b.a, b.b, b.c};
    for (int p = 0; p < 3; ++p) {
      if (pin(vert[p])) continue;
      for (int q = 0; q < 3; ++q) {
        if (pin(vert[q])) continue;
        t.push_back({vert[p], vert[q], b.k * w[p] * w[q]});
      }
    }
  }
  for (int v = 0; v < n; ++v) {
    if (!pin(v)) continue;
    // Only free-free edges add to a diagonal; a pinned vertex has none, and its bend diagonal is 0.
    double existing = s.m[v] * invDt2;
    existing += 0.0;
    t.push_back({v, v, 1.0 - existing});
  }
  std::stable_sort(t.begin(), t.end(),
                   [](const T& a, const T& b) { return a.r != b.r ? a.r < b.r : a.c < b.c; });
  L.n = n;
  L.rowptr.assign(n + 1, 0);
  L.col.clear();
  L.val.clear();
  for (size_t i = 0; i < t.size();) {
    double acc = t[i].v;
    size_t j = i + 1;
    for (; j < t.size() && t[j].r == t[i].r && t[j].c == t[i].c; ++j) acc = acc + t[j].v;
    L.col.push_back(t[i].c);
    L.val.push_back(acc);
    L.rowptr[t[i].r + 1] += 1;
    i = j;
  }
  for (int r = 0; r < n; ++r) L.rowptr[r + 1] += L.rowptr[r];
}

// Constant bending RHS for stencils that touch pinned vertices (Assembler.cpp:94-137).
void assembleBendingRhs(const Scene& s, std::vector<double>& out) {
  out.assign(3 * static_cast<size_t>(s.n), 0.0);
  const double w[3] = {1.0, -2.0, 1.0};
  for (const Bend& b : s.bends) {
    if (b.k == 0.0) continue;
    const int vert[3] = {b.a, b.b, b.c};
    double c[3] = {0.0, 0.0, 0.0};
    bool any = false;
    for (int k = 0; k < 3; ++k) {
      if (!s.pinned[vert[k]]) continue;
      any = true;
      for (int d = 0; d < 3; ++d) c[d] = c[d] + s.q[3 * static_cast<size_t>(vert[k]) + d] * w[k];
    }
    if (!any) continue;
    for (int k = 0; k < 3; ++k) {
      const int p = vert[k];
      if (s.pinned[p]) continue;
      const double f = -b.k * w[k];
      for (int d = 0; d < 3; ++d) out[3 * static_cast<size_t>(p) + d] += c[d] * f;
    }
  }
}

// ------------------------------------------------------------------------------ ordering
std::vector<int32_t> nestedDissection(const Scene& s, const ScalarMatrix& L, int leafSize, SupernodeTree* tree) {
  const int n = s.n;
  std::vector<int32_t> order;
  order.reserve(n);
  std::vector<int64_t> mark(n, -1);
  int64_t stamp = 0;
  // Each call appends its vertices to `order` and returns the id of the supernode that owns its
  // last columns (its separator, or itself for a leaf); children get that id as parent.
  std::vector<int32_t> snBegin, snEnd, snParent;
  auto newNode = [&](int32_t b, int32_t e) {
    snBegin.push_back(b);
    snEnd.push_back(e);
    snParent.push_back(-1);
    return static_cast<int32_t>(snBegin.size()) - 1;
  };
  std::function<int32_t(std::vector<int32_t>&)> nd = [&](std::vector<int32_t>& verts) -> int32_t {
    if (static_cast<int>(verts.size()) <= leafSize) {
      std::sort(verts.begin(), verts.end());
      const int32_t b = static_cast<int32_t>(order.size());
      order.insert(order.end(), verts.begin(), verts.end());
      return newNode(b, static_cast<int32_t>(order.size()));
    }
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int v : verts)
      for (int d = 0; d < 3; ++d) {
        lo[d] = std::min(lo[d], s.x[3 * static_cast<size_t>(v) + d]);
        hi[d] = std::max(hi[d], s.x[3 * static_cast<size_t>(v) + d]);
      }
    int axis = 0;
    for (int d = 1; d < 3; ++d)
      if (hi[d] - lo[d] > hi[axis] - lo[axis]) axis = d;
    std::sort(verts.begin(), verts.end(), [&](int32_t a, int32_t b) {
      const double ca = s.x[3 * static_cast<size_t>(a) + axis], cb = s.x[3 * static_cast<size_t>(b) + axis];
      return ca != cb ? ca < cb : a < b;
    });
    const size_t half = verts.size() / 2;
    std::vector<int32_t> left(verts.begin(), verts.begin() + half), right, sep;
    const int64_t id = ++stamp;
    for (int v : left) mark[v] = id;
    for (size_t i = half; i < verts.size(); ++i) {
      const int v = verts[i];
      bool touches = false;
      for (int k = L.rowptr[v]; k < L.rowptr[v + 1] && !touches; ++k) touches = (mark[L.col[k]] == id);
      (touches ? sep : right).push_back(v);
    }
    if (right.empty() || left.empty()) {  // no progress: treat as a leaf
      std::sort(verts.begin(), verts.end());
      const int32_t b = static_cast<int32_t>(order.size());
      order.insert(order.end(), verts.begin(), verts.end());
      return newNode(b, static_cast<int32_t>(order.size()));
    }
    const int32_t cl = nd(left);
    const int32_t cr = nd(right);
    std::sort(sep.begin(), sep.end());
    const int32_t b = static_cast<int32_t>(order.size());
    order.insert(order.end(), sep.begin(), sep.end());
    const int32_t me = newNode(b, static_cast<int32_t>(order.size()));
    snParent[cl] = me;
    snParent[cr] = me;
    return me;
  };
  std::vector<int32_t> all(n);
  std::iota(all.begin(), all.end(), 0);
  nd(all);
  if (tree) {
    // nodes were created in postorder, so their ranges are already ascending and contiguous
    tree->start.assign(snBegin.size() + 1, 0);
    for (size_t i = 0; i < snBegin.size(); ++i) tree->start[i] = snBegin[i];
    tree->start[snBegin.size()] = n;
    tree->parent = snParent;
  }
  return order;
}

// Supernodal data of the factor: splits between off-block and in-block entries, the dense
// inverse of every diagonal block, and rows grouped by tree level.
void buildSupernodal(Factor& f, const SupernodeTree& tree) {
  const int n = f.n;
  const int ns = static_cast<int>(tree.parent.size());
  f.snStart = tree.start;
  f.snParent = tree.parent;
  f.rowSn.assign(n, 0);
  for (int s = 0; s < ns; ++s)
    for (int i = f.snStart[s]; i < f.snStart[s + 1]; ++i) f.rowSn[i] = s;
  f.offEnd.assign(n, 0);
  f.offBeg.assign(n, 0);
  for (int i = 0; i < n; ++i) {
    const int s0 = f.snStart[f.rowSn[i]], s1 = f.snStart[f.rowSn[i] + 1];
    int p = f.rowptr[i];
    while (p < f.rowptr[i + 1] && f.colidx[p] < s0) ++p;
    f.offEnd[i] = p;
    p = f.colptr[i];
    while (p < f.colptr[i + 1] && f.rowidx[p] < s1) ++p;
    f.offBeg[i] = p;
  }
  // dense inverses of the unit-lower diagonal blocks
  f.snInvOff.assign(ns + 1, 0);
  for (int s = 0; s < ns; ++s) {
    const int64_t sz = f.snStart[s + 1] - f.snStart[s];
    f.snInvOff[s + 1] = f.snInvOff[s] + sz * (sz + 1) / 2;
  }
  f.invL.assign(f.snInvOff[ns], 0.0);
  f.invLT.assign(f.snInvOff[ns], 0.0);
  std::vector<double> B, X;
  for (int s = 0; s < ns; ++s) {
    const int s0 = f.snStart[s], sz = f.snStart[s + 1] - s0;
    if (sz == 0) continue;
    B.assign(static_cast<size_t>(sz) * sz, 0.0);
    for (int r = 0; r < sz; ++r)
      for (int p = f.offEnd[s0 + r]; p < f.rowptr[s0 + r + 1]; ++p) B[static_cast<size_t>(r) * sz + (f.colidx[p] - s0)] = f.rowval[p];
    X.assign(static_cast<size_t>(sz) * sz, 0.0);
    for (int c = 0; c < sz; ++c) {  // column c of L_SS⁻¹ by forward substitution
      X[static_cast<size_t>(c) * sz + c] = 1.0;
      for (int r = c + 1; r < sz; ++r) {
        double acc = 0.0;
        for (int t = c; t < r; ++t) acc += B[static_cast<size_t>(r) * sz + t] * X[static_cast<size_t>(t) * sz + c];
        X[static_cast<size_t>(r) * sz + c] = -acc;
      }
    }
    double* lo = f.invL.data() + f.snInvOff[s];
    double* up = f.invLT.data() + f.snInvOff[s];
    for (int r = 0, k = 0; r < sz; ++r)
      for (int c = 0; c <= r; ++c) lo[k++] = X[static_cast<size_t>(r) * sz + c];
    for (int r = 0, k = 0; r < sz; ++r)  // row r of the transpose: X[c][r] for c = r..sz−1
      for (int c = r; c < sz; ++c) up[k++] = X[static_cast<size_t>(c) * sz + r];
  }
  // levels: leaves 0, a parent one above its highest child; rows grouped by level
  f.snLevel.assign(ns, 0);
  for (int s = 0; s < ns; ++s)  // postorder: children precede parents
    if (f.snParent[s] >= 0) f.snLevel[f.snParent[s]] = std::max(f.snLevel[f.snParent[s]], f.snLevel[s] + 1);
  int nlev = 0;
  for (int s = 0; s < ns; ++s) nlev = std::max(nlev, f.snLevel[s] + 1);
  f.lvlRowPtr.assign(nlev + 1, 0);
  for (int s = 0; s < ns; ++s) f.lvlRowPtr[f.snLevel[s] + 1] += f.snStart[s + 1] - f.snStart[s];
  for (int l = 0; l < nlev; ++l) f.lvlRowPtr[l + 1] += f.lvlRowPtr[l];
  f.lvlRows.assign(n, 0);
  std::vector<int32_t> cur(f.lvlRowPtr.begin(), f.lvlRowPtr.end() - 1);
  for (int s = 0; s < ns; ++s)
    for (int i = f.snStart[s]; i < f.snStart[s + 1]; ++i) f.lvlRows[cur[f.snLevel[s]]++] = i;
}

namespace {
// Row length of row i of the supernodal solve for phase ph (fwd gather, fwd dense, bwd gather, bwd dense).
int phaseLength(const Factor& f, int i, int ph) {
  const int s = f.rowSn[i], s0 = f.snStart[s], sz = f.snStart[s + 1] - s0;
  switch (ph) {
    case 0: return f.offEnd[i] - f.rowptr[i];
    case 1: return i - s0 + 1;
    case 2: return f.colptr[i + 1] - f.offBeg[i];
    default: return sz - (i - s0);
  }
}
}  // namespace

std::vector<int32_t> chooseGroupWidths32(const Factor& f, int ctaThreads, int ctas, double latencyScale) {
  const int nlev = static_cast<int>(f.lvlRowPtr.size()) - 1;
  std::vector<int32_t> g(4 * static_cast<size_t>(std::max(nlev, 0)), 1);
  for (int l = 0; l < nlev; ++l)
    for (int ph = 0; ph < 4; ++ph) {
      const int R = f.lvlRowPtr[l + 1] - f.lvlRowPtr[l];
      if (R == 0) continue;
      double sum = 0.0;
      int lmax = 0;
      for (int t = f.lvlRowPtr[l]; t < f.lvlRowPtr[l + 1]; ++t) {
        const int len = phaseLength(f, f.lvlRows[t], ph);
        sum += len;
        lmax = std::max(lmax, len);
      }
      const double lavg = sum / R;
      double best = 1e300;
      int bestG = 1;
      for (int G = 1, lg = 0; G <= 32; G *= 2, ++lg) {
        // one CTA of 256 threads: issue-bound term (1 warp instruction per cycle per SMSP) against
        // the longest group's latency chain: an L2 round trip (~600 cycles) per four unrolled
        // trips of the row loop, ~8 cycles per dependent FMA, ~30 per shuffle step
        const double trips = std::ceil(static_cast<double>(lmax) / G);
        const double issue = R * G / 32.0 * (3.0 * std::ceil(lavg / G) + 4.0 * lg + 6.0) / (4.0 * ctas);
        const double chain = latencyScale * std::ceil(R * G / static_cast<double>(ctaThreads * ctas)) *
                             (600.0 * std::ceil(trips / 4.0) + 8.0 * trips + 30.0 * lg + 600.0);
        const double cost = std::max(issue, chain);
        if (cost < best) {
          best = cost;
          bestG = G;
        }
      }
      g[4 * static_cast<size_t>(l) + ph] = bestG;
    }
  return g;
}

void buildRefactorMaps(Factor& f) {
  const int n = f.n;
  const int64_t nnz = f.colptr[n];
  f.cscToCsr.assign(nnz, 0);
  std::vector<int32_t> cur(f.rowptr.begin(), f.rowptr.end() - 1);
  for (int c = 0; c < n; ++c)  // the CSR was filled column by column: same walk
    for (int p = f.colptr[c]; p < f.colptr[c + 1]; ++p) f.cscToCsr[p] = cur[f.rowidx[p]]++;
  auto find = [&](int row, int col) {
    const int32_t* b = f.Acol.data() + f.Aptr[row];
    const int32_t* e = f.Acol.data() + f.Aptr[row + 1];
    const int32_t* it = std::lower_bound(b, e, col);
    return (it != e && *it == col) ? static_cast<int32_t>(it - f.Acol.data()) : -1;
  };
  f.aPosCsc.assign(nnz, -1);
  for (int c = 0; c < n; ++c)
    for (int p = f.colptr[c]; p < f.colptr[c + 1]; ++p) f.aPosCsc[p] = find(f.rowidx[p], c);
  f.aPosDiag.assign(n, -1);
  for (int j = 0; j < n; ++j) f.aPosDiag[j] = find(j, j);
  const int ns = static_cast<int>(f.snLevel.size());
  int nlev = 0;
  for (int s = 0; s < ns; ++s) nlev = std::max(nlev, f.snLevel[s] + 1);
  f.snLevelPtr.assign(nlev + 1, 0);
  for (int s = 0; s < ns; ++s) f.snLevelPtr[f.snLevel[s] + 1] += 1;
  for (int l = 0; l < nlev; ++l) f.snLevelPtr[l + 1] += f.snLevelPtr[l];
  f.snByLevel.assign(ns, 0);
  std::vector<int32_t> at(f.snLevelPtr.begin(), f.snLevelPtr.end() - 1);
  for (int s = 0; s < ns; ++s) f.snByLevel[at[f.snLevel[s]]++] = s;
  f.maxRowLen = 0;
  for (int r = 0; r < n; ++r) f.maxRowLen = std::max(f.maxRowLen, f.rowptr[r + 1] - f.rowptr[r]);
}

void refreshAval(Factor& f, const ScalarMatrix& A) {
  const int n = f.n;
  std::vector<std::pair<int32_t, double>> row;
  for (int i = 0; i < n; ++i) {
    const int v = f.perm[i];
    row.clear();
    for (int p = A.rowptr[v]; p < A.rowptr[v + 1]; ++p) row.push_back({f.iperm[A.col[p]], A.val[p]});
    std::sort(row.begin(), row.end(), [](auto& a, auto& b) { return a.first < b.first; });
    for (size_t t = 0; t < row.size(); ++t) f.Aval[f.Aptr[i] + t] = row[t].second;
  }
}

void buildMixed(Factor& f, const ScalarMatrix& A) {
  auto toF = [](const std::vector<double>& v) { return std::vector<float>(v.begin(), v.end()); };
  f.rowval32 = toF(f.rowval);
  f.colval32 = toF(f.colval);
  f.invL32 = toF(f.invL);
  f.invLT32 = toF(f.invLT);
  f.dinv32 = toF(f.dinv);
  const int n = f.n;
  f.Aptr.assign(n + 1, 0);
  f.Acol.clear();
  f.Aval.clear();
  std::vector<std::pair<int32_t, double>> row;
  for (int i = 0; i < n; ++i) {
    const int v = f.perm[i];
    row.clear();
    for (int p = A.rowptr[v]; p < A.rowptr[v + 1]; ++p) row.push_back({f.iperm[A.col[p]], A.val[p]});
    std::sort(row.begin(), row.end(), [](auto& a, auto& b) { return a.first < b.first; });
    for (auto& e : row) {
      f.Acol.push_back(e.first);
      f.Aval.push_back(e.second);
    }
    f.Aptr[i + 1] = static_cast<int32_t>(f.Acol.size());
  }
}

std::vector<int32_t> chooseGroupWidths(const Factor& f, int teamCtas, double latencyScale) {
  const int nlev = static_cast<int>(f.lvlRowPtr.size()) - 1;
  std::vector<int32_t> g(4 * static_cast<size_t>(std::max(nlev, 0)), 1);
  // every CTA of the FP64 kernels runs 256 threads
  const double smsps = 4.0 * teamCtas, threads = 256.0 * teamCtas;
  for (int l = 0; l < nlev; ++l) {
    for (int ph = 0; ph < 4; ++ph) {
      const int R = f.lvlRowPtr[l + 1] - f.lvlRowPtr[l];
      if (R == 0) continue;
      double sum = 0.0;
      int lmax = 0;
      for (int t = f.lvlRowPtr[l]; t < f.lvlRowPtr[l + 1]; ++t) {
        const int i = f.lvlRows[t];
        const int s = f.rowSn[i], s0 = f.snStart[s], sz = f.snStart[s + 1] - s0;
        int len = 0;
        switch (ph) {
          case 0: len = f.offEnd[i] - f.rowptr[i]; break;
          case 1: len = i - s0 + 1; break;
          case 2: len = f.colptr[i + 1] - f.offBeg[i]; break;
          default: len = sz - (i - s0); break;
        }
        sum += len;
        lmax = std::max(lmax, len);
      }
      const double lavg = sum / R;
      double best = 1e300;
      int bestG = 1;
      for (int G = 1, lg = 0; G <= 32; G *= 2, ++lg) {
        // cycles: FP64 warp instructions spread over the team's SMSPs (~80 cycles each) against
        // the longest group's chain — an L2 round trip (~700 cycles) per four unrolled trips,
        // 64 cycles per dependent FP64 FMA, ~100 per shuffle-and-add step, one more round trip
        const double perRowInstr = 3.0 * std::ceil(lavg / G) + 3.0 * lg + 3.0;
        const double total = R * G / 32.0 * perRowInstr * 80.0;
        const double rowsPerGroup = std::ceil(R * G / threads);
        const double trips = std::ceil(static_cast<double>(lmax) / G);
        const double chain =
            latencyScale * rowsPerGroup * (700.0 * std::ceil(trips / 4.0) + 64.0 * trips + 100.0 * lg + 700.0);
        const double cost = std::max(total / smsps, chain);
        if (cost < best) {
          best = cost;
          bestG = G;
        }
      }
      g[4 * static_cast<size_t>(l) + ph] = bestG;
    }
  }
  return g;
}

// ----------------------------------------------------------------------- factorization
// Up-looking LDLᵀ: the published algorithm of T. A. Davis' LDL package, which Eigen 3.4.0's
// SimplicialLDLT implements. Row k of L comes from a sparse triangular solve whose pattern is
// the etree reach of column k of P·Ã·Pᵀ (upper part), visited in topological order.
bool factorize(const ScalarMatrix& A, const std::vector<int32_t>& perm, Factor& f, std::string* err) {
  const int n = A.n;
  if (static_cast<int>(perm.size()) != n) {
    if (err) *err = "permutation size does not match the matrix";
    return false;
  }
  f.n = n;
  f.perm = perm;
  f.iperm.assign(n, -1);
  for (int k = 0; k < n; ++k) {
    if (perm[k] < 0 || perm[k] >= n || f.iperm[perm[k]] != -1) {
      if (err) *err = "ordering is not a permutation";
      return false;
    }
    f.iperm[perm[k]] = k;
  }
  // upper-stored columns of P·Ã·Pᵀ, rows ascending
  std::vector<int32_t> Ap(n + 1, 0), Ai;
  std::vector<double> Ax;
  {
    std::vector<int32_t> cnt(n + 1, 0);
    for (int r = 0; r < n; ++r)
      for (int k = A.rowptr[r]; k < A.rowptr[r + 1]; ++k) {
        const int pr = f.iperm[r], pc = f.iperm[A.col[k]];
        if (pr <= pc) cnt[pc + 1] += 1;
      }
    for (int k = 0; k < n; ++k) cnt[k + 1] += cnt[k];
    Ap = cnt;
    Ai.assign(Ap[n], 0);
    Ax.assign(Ap[n], 0.0);
    std::vector<int32_t> cur(Ap.begin(), Ap.end() - 1);
    for (int r = 0; r < n; ++r)
      for (int k = A.rowptr[r]; k < A.rowptr[r + 1]; ++k) {
        const int pr = f.iperm[r], pc = f.iperm[A.col[k]];
        if (pr <= pc) {
          Ai[cur[pc]] = pr;
          Ax[cur[pc]] = A.val[k];
          cur[pc]++;
        }
      }
    std::vector<std::pair<int32_t, double>> tmp;
    for (int k = 0; k < n; ++k) {
      tmp.clear();
      for (int p = Ap[k]; p < Ap[k + 1]; ++p) tmp.push_back({Ai[p], Ax[p]});
      std::sort(tmp.begin(), tmp.end(), [](auto& a, auto& b) { return a.first < b.first; });
      for (int p = Ap[k], i = 0; p < Ap[k + 1]; ++p, ++i) {
        Ai[p] = tmp[i].first;
        Ax[p] = tmp[i].second;
      }
    }
  }
  // symbolic: elimination tree and column counts
  std::vector<int32_t> tags(n), nz(n);
  f.parent.assign(n, -1);
  for (int k = 0; k < n; ++k) {
    f.parent[k] = -1;
    tags[k] = k;
    nz[k] = 0;
    for (int p = Ap[k]; p < Ap[k + 1]; ++p) {
      int i = Ai[p];
      if (i < k)
        for (; tags[i] != k; i = f.parent[i]) {
          if (f.parent[i] == -1) f.parent[i] = k;
          nz[i]++;
          tags[i] = k;
        }
    }
  }
  f.colptr.assign(n + 1, 0);
  for (int k = 0; k < n; ++k) f.colptr[k + 1] = f.colptr[k] + nz[k];
  f.rowidx.assign(f.colptr[n], 0);
  f.colval.assign(f.colptr[n], 0.0);
  f.d.assign(n, 0.0);
  // numeric
  std::vector<double> y(n, 0.0);
  std::vector<int32_t> pattern(n), fill(n, 0);
  for (int k = 0; k < n; ++k) {
    y[k] = 0.0;
    int top = n;
    tags[k] = k;
    fill[k] = 0;
    for (int p = Ap[k]; p < Ap[k + 1]; ++p) {
      int i = Ai[p];
      if (i <= k) {
        y[i] += Ax[p];
        int len = 0;
        for (; tags[i] != k; i = f.parent[i]) {
          pattern[len++] = i;
          tags[i] = k;
        }
        while (len > 0) pattern[--top] = pattern[--len];
      }
    }
    double dk = y[k] * 1.0 + 0.0;
    y[k] = 0.0;
    for (; top < n; ++top) {
      const int i = pattern[top];
      const double yi = y[i];
      y[i] = 0.0;
      const double lki = yi / f.d[i];
      const int p2 = f.colptr[i] + fill[i];
      int p;
      for (p = f.colptr[i]; p < p2; ++p) y[f.rowidx[p]] -= f.colval[p] * yi;
      dk -= lki * yi;
      f.rowidx[p] = k;
      f.colval[p] = lki;
      ++fill[i];
    }
    f.d[k] = dk;
    if (dk == 0.0 || !std::isfinite(dk)) {
      if (err) *err = "LDL^T pivot " + std::to_string(k) + " is zero or not finite: L is not positive definite";
      return false;
    }
  }
  f.dinv.resize(n);
  for (int k = 0; k < n; ++k) f.dinv[k] = 1.0 / f.d[k];
  // row-major copy for the forward gather (columns ascending within a row)
  f.rowptr.assign(n + 1, 0);
  for (int p = 0; p < f.colptr[n]; ++p) f.rowptr[f.rowidx[p] + 1] += 1;
  for (int r = 0; r < n; ++r) f.rowptr[r + 1] += f.rowptr[r];
  f.colidx.assign(f.colptr[n], 0);
  f.rowval.assign(f.colptr[n], 0.0);
  std::vector<int32_t> cur(f.rowptr.begin(), f.rowptr.end() - 1);
  for (int c = 0; c < n; ++c)
    for (int p = f.colptr[c]; p < f.colptr[c + 1]; ++p) {
      const int r = f.rowidx[p];
      f.colidx[cur[r]] = c;
      f.rowval[cur[r]] = f.colval[p];
      cur[r]++;
    }
  buildSchedules(f);
  return true;
}

void buildSchedules(Factor& f) {
  const int n = f.n;
  std::vector<int32_t> lev(n, 0);
  int maxLev = -1;
  for (int r = 0; r < n; ++r) {
    int l = 0;
    for (int p = f.rowptr[r]; p < f.rowptr[r + 1]; ++p) l = std::max(l, lev[f.colidx[p]] + 1);
    lev[r] = l;
    maxLev = std::max(maxLev, l);
  }
  auto group = [&](std::vector<int32_t>& ptr, std::vector<int32_t>& rows, int levels) {
    ptr.assign(levels + 1, 0);
    for (int r = 0; r < n; ++r) ptr[lev[r] + 1] += 1;
    for (int l = 0; l < levels; ++l) ptr[l + 1] += ptr[l];
    rows.assign(n, 0);
    std::vector<int32_t> cur(ptr.begin(), ptr.end() - 1);
    for (int r = 0; r < n; ++r) rows[cur[lev[r]]++] = r;
  };
  group(f.fwdLevelPtr, f.fwdRows, maxLev + 1);
  maxLev = -1;
  for (int k = n - 1; k >= 0; --k) {
    int l = 0;
    for (int p = f.colptr[k]; p < f.colptr[k + 1]; ++p) l = std::max(l, lev[f.rowidx[p]] + 1);
    lev[k] = l;
    maxLev = std::max(maxLev, l);
  }
  group(f.bwdLevelPtr, f.bwdRows, maxLev + 1);
}

Stamp computeStamp(const Scene& s, double dt) {
  Stamp st;
  uint64_t kh = 0xcbf29ce484222325ULL, mh = kh, ph = kh, sh = kh;
  for (const Edge& e : s.edges) kh = hashCombine(kh, bitsOf(e.k));
  for (const Bend& b : s.bends) kh = hashCombine(kh, bitsOf(b.k));
  for (double m : s.m) mh = hashCombine(mh, bitsOf(m));
  for (uint8_t p : s.pinned) ph = hashCombine(ph, p ? 1ULL : 0ULL);
  sh = hashCombine(sh, 1);
  sh = hashCombine(sh, static_cast<uint64_t>(s.n));
  sh = hashCombine(sh, static_cast<uint64_t>(s.edges.size()));
  for (const Edge& e : s.edges) {
    sh = hashCombine(sh, static_cast<uint32_t>(e.a));
    sh = hashCombine(sh, static_cast<uint32_t>(e.b));
  }
  sh = hashCombine(sh, static_cast<uint64_t>(s.bends.size()));
  for (const Bend& b : s.bends) {
    sh = hashCombine(sh, static_cast<uint32_t>(b.a));
    sh = hashCombine(sh, static_cast<uint32_t>(b.b));
    sh = hashCombine(sh, static_cast<uint32_t>(b.c));
  }
  for (uint8_t p : s.pinned) sh = hashCombine(sh, p ? 1ULL : 0ULL);
  st.k = kh;
  st.m = mh;
  st.pin = ph;
  st.dt = bitsOf(dt);
  st.structure = sh;
  return st;
}

}  // namespace pdg

namespace pdg {

// ------------------------------------------------------------------------------ grid scene
namespace {
template <class F>
void forEachBend(const GridSpec& g, F&& add) {
  const int nx = g.nx, ny = g.ny;
  if (!(g.bendStiffness > 0.0) || (nx < 3 && ny < 3)) return;
  const int stride = g.bendStride > 0 ? g.bendStride : 1;
  const bool rows = g.bendSampling == 0 || g.bendSampling == 1;
  const bool cols = g.bendSampling == 0 || g.bendSampling == 2;
  const bool checker = g.bendSampling == 3;
  // rows first, then columns, i / j ascending: the stencil order is the residual's sum order
  if (rows)
    for (int j = 0; j < ny; ++j)
      for (int i = 1; i + 1 < nx; ++i)
        if ((i - 1) % stride == 0) add(j * nx + i - 1, j * nx + i, j * nx + i + 1);
  if (cols)
    for (int i = 0; i < nx; ++i)
      for (int j = 1; j + 1 < ny; ++j)
        if ((j - 1) % stride == 0) add((j - 1) * nx + i, j * nx + i, (j + 1) * nx + i);
  if (checker) {
    for (int j = 0; j < ny; ++j)
      for (int i = 1; i + 1 < nx; ++i)
        if ((i - 1) % stride == 0 && ((i + j) & 1) == 0) add(j * nx + i - 1, j * nx + i, j * nx + i + 1);
    for (int i = 0; i < nx; ++i)
      for (int j = 1; j + 1 < ny; ++j)
        if ((j - 1) % stride == 0 && ((i + j) & 1) != 0) add((j - 1) * nx + i, j * nx + i, (j + 1) * nx + i);
  }
}
}  // namespace

bool gridCounts(const GridSpec& g, int* nv, int* ne, int* nb) {
  if (g.nx < 2 || g.ny < 2) return false;
  *nv = g.nx * g.ny;
  *ne = 2 * g.nx * g.ny - g.nx - g.ny + ((g.shearStiffness > 0.0) ? (g.nx - 1) * (g.ny - 1) : 0);
  int b = 0;
  forEachBend(g, [&](int, int, int) { ++b; });
  *nb = b;
  return true;
}

bool makeGrid(const GridSpec& g, Scene& s) {
  const int nx = g.nx, ny = g.ny;
  if (nx < 2 || ny < 2) return false;
  const int n = nx * ny;
  s = Scene{};
  s.n = n;
  s.x.assign(3 * static_cast<size_t>(n), 0.0);
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const int v = j * nx + i;
      s.x[3 * v] = static_cast<double>(i) * g.spacing;
      s.x[3 * v + 2] = static_cast<double>(j) * g.spacing;
    }
  auto addEdge = [&](int a, int b, double k) {
    const double dx = s.x[3 * b] - s.x[3 * a], dy = s.x[3 * b + 1] - s.x[3 * a + 1], dz = s.x[3 * b + 2] - s.x[3 * a + 2];
    s.edges.push_back(Edge{a, b, std::sqrt(dx * dx + dy * dy + dz * dz), k});
  };
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const int v = j * nx + i;
      if (i + 1 < nx) addEdge(v, v + 1, g.stiffness);
      if (j + 1 < ny) addEdge(v, v + nx, g.stiffness);
    }
  s.m.assign(n, 0.0);
  if (g.massMode == 0) {  // Mesh::computeMassesFromEdges on the structural edges
    const double density = g.density > 0.0 ? g.density : 1.0;
    for (const Edge& e : s.edges) {
      const double share = density * e.rest * e.rest * 0.5;
      s.m[e.a] += share;
      s.m[e.b] += share;
    }
    double minPos = 1e300;
    for (double m : s.m)
      if (m > 1e-12) minPos = std::min(minPos, m);
    if (minPos > 1e299) minPos = 1.0;
    for (double& m : s.m)
      if (m < 1e-12) m = minPos;
  } else {
    const double each = g.totalMass / static_cast<double>(n);
    for (double& m : s.m) m = each;
  }
  if (g.shearStiffness > 0.0)
    for (int j = 0; j + 1 < ny; ++j)
      for (int i = 0; i + 1 < nx; ++i) addEdge(j * nx + i, (j + 1) * nx + i + 1, g.shearStiffness);
  forEachBend(g, [&](int a, int b, int c) { s.bends.push_back(Bend{a, b, c, g.bendStiffness}); });
  s.pinned.assign(n, 0);
  switch (g.pinMode) {
    case 0: s.pinned[(ny - 1) * nx] = 1; s.pinned[(ny - 1) * nx + nx - 1] = 1; break;
    case 1: s.pinned[0] = 1; s.pinned[nx - 1] = 1; break;
    case 2: for (int i = 0; i < nx; ++i) s.pinned[(ny - 1) * nx + i] = 1; break;
    case 3: s.pinned[(ny - 1) * nx] = 1; break;
    default: break;
  }
  s.v.assign(3 * static_cast<size_t>(n), 0.0);
  s.q = s.x;
  return true;
}


namespace {

// Whitespace-separated tokens of one line.
std::vector<std::string> tokensOf(const std::string& line) {
  std::vector<std::string> out;
  size_t i = 0;
  while (i < line.size()) {
    while (i < line.size() && std::isspace(static_cast<unsigned char>(line[i]))) ++i;
    size_t j = i;
    while (j < line.size() && !std::isspace(static_cast<unsigned char>(line[j]))) ++j;
    if (j > i) out.emplace_back(line, i, j - i);
    i = j;
  }
  return out;
}

}  // namespace

bool makeObj(const std::string& text, double stiffness, double density, Scene& s, std::string* err) {
  auto failWith = [&](const std::string& m) {
    if (err) *err = m;
    return false;
  };
  std::vector<double> pos;
  std::vector<int> tri;
  size_t start = 0;
  int lineNo = 0;
  while (start <= text.size()) {
    size_t end = text.find('\n', start);
    if (end == std::string::npos) end = text.size();
    const std::string line = text.substr(start, end - start);
    start = end + 1;
    ++lineNo;
    const std::vector<std::string> tok = tokensOf(line);
    if (tok.empty()) continue;
    if (tok[0] == "v") {
      double c[3] = {0.0, 0.0, 0.0};
      for (int k = 0; k < 3 && k + 1 < static_cast<int>(tok.size()); ++k) {
        char* e = nullptr;
        c[k] = std::strtod(tok[k + 1].c_str(), &e);
        if (e == tok[k + 1].c_str() || *e != '\0') return failWith("line " + std::to_string(lineNo) + ": bad coordinate");
      }
      pos.insert(pos.end(), c, c + 3);
    } else if (tok[0] == "f") {
      if (tok.size() < 4) continue;  // fewer than three corners: skipped, as the reference does
      for (int k = 0; k < 3; ++k) {
        const std::string first = tok[k + 1].substr(0, tok[k + 1].find('/'));
        char* e = nullptr;
        const long idx = std::strtol(first.c_str(), &e, 10);
        if (e == first.c_str()) return failWith("line " + std::to_string(lineNo) + ": bad face index");
        tri.push_back(static_cast<int>(idx) - 1);
      }
    }
  }
  const int n = static_cast<int>(pos.size() / 3);
  if (n == 0 || tri.empty()) return failWith("no vertices or no triangles");
  for (int i : tri)
    if (i < 0 || i >= n) return failWith("face index out of range (indices are 1-based, negative ones unsupported)");
  s = Scene{};
  s.n = n;
  s.x = pos;
  // unique triangle edges in first-seen order, oriented as first seen
  std::vector<uint64_t> seen;
  seen.reserve(tri.size());
  for (size_t t = 0; t < tri.size(); t += 3) {
    for (int k = 0; k < 3; ++k) {
      const int a = tri[t + k], b = tri[t + (k + 1) % 3];
      if (a == b) continue;
      const uint64_t key = (static_cast<uint64_t>(std::min(a, b)) << 32) | static_cast<uint32_t>(std::max(a, b));
      seen.push_back(key);
    }
  }
  {
    std::vector<uint64_t> sorted = seen;
    std::sort(sorted.begin(), sorted.end());
    std::vector<uint8_t> used(sorted.size(), 0);
    for (size_t t = 0; t < tri.size(); t += 3) {
      for (int k = 0; k < 3; ++k) {
        const int a = tri[t + k], b = tri[t + (k + 1) % 3];
        if (a == b) continue;
        const uint64_t key = (static_cast<uint64_t>(std::min(a, b)) << 32) | static_cast<uint32_t>(std::max(a, b));
        const size_t at = static_cast<size_t>(std::lower_bound(sorted.begin(), sorted.end(), key) - sorted.begin());
        // duplicates of a key are adjacent in `sorted`; the first occurrence claims them all
        if (used[at]) continue;
        for (size_t u = at; u < sorted.size() && sorted[u] == key; ++u) used[u] = 1;
        const double dx = s.x[3 * b] - s.x[3 * a], dy = s.x[3 * b + 1] - s.x[3 * a + 1],
                     dz = s.x[3 * b + 2] - s.x[3 * a + 2];
        s.edges.push_back(Edge{a, b, std::sqrt(dx * dx + dy * dy + dz * dz), stiffness});
      }
    }
  }
  // surface masses: each triangle adds density·area/3 to its corners, in triangle order
  const double rho = density > 0.0 ? density : 1.0;
  s.m.assign(n, 0.0);
  for (size_t t = 0; t < tri.size(); t += 3) {
    const double* p0 = &s.x[3 * tri[t]];
    const double* p1 = &s.x[3 * tri[t + 1]];
    const double* p2 = &s.x[3 * tri[t + 2]];
    const double u0 = p1[0] - p0[0], u1 = p1[1] - p0[1], u2 = p1[2] - p0[2];
    const double w0 = p2[0] - p0[0], w1 = p2[1] - p0[1], w2 = p2[2] - p0[2];
    const double c0 = u1 * w2 - u2 * w1, c1 = u2 * w0 - u0 * w2, c2 = u0 * w1 - u1 * w0;
    const double area = 0.5 * std::sqrt(c0 * c0 + c1 * c1 + c2 * c2);
    for (int k = 0; k < 3; ++k) s.m[tri[t + k]] += rho * area / 3.0;
  }
  double minPos = 1e300;
  for (double m : s.m)
    if (m > 1e-12) minPos = std::min(minPos, m);
  if (minPos > 1e299) minPos = 1.0;
  for (double& m : s.m)
    if (m < 1e-12) m = minPos;
  s.pinned.assign(n, 0);
  s.v.assign(3 * static_cast<size_t>(n), 0.0);
  s.q = s.x;
  return true;
}

}  // namespace pdg
