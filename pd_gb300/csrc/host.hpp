// host.hpp — host-side preparation of a cloth instance for the GPU substep.
//
// Everything here is one-time (or once-per-stamp-change) work that the reference does on the
// CPU before its per-substep loop: topology (colouring and incidence CSRs), assembly of the
// constant matrix L, a fill-reducing ordering, the LDLᵀ factorization and, new here, the
// level schedules that let the GPU run the triangular solves in the reference's exact order.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace pdg {

struct Edge {
  int32_t a, b;
  double rest, k;
};
struct Bend {
  int32_t a, b, c;
  double k;
};

// Raw scene of one cloth (positions etc. interleaved [x,y,z] per vertex).
struct Scene {
  int32_t n = 0;
  std::vector<double> x, v, m, q;
  std::vector<uint8_t> pinned;
  std::vector<Edge> edges;
  std::vector<Bend> bends;
};

// Topology shared by the scatter and residual gathers (core/mesh/ConstraintColoring.h:34-81).
struct Topology {
  int colorCount = 0;
  std::vector<uint32_t> colorOf;
  // vertex → incident edges in colour order (the reference's per-vertex scatter summation order)
  std::vector<int32_t> sstart, sinc;  // sinc = edge << 1 | (vertex is endpoint b)
  // vertex → incident edges in edge-index order (residual gather order, vertexEdges)
  std::vector<int32_t> rstart, rinc;
  // vertex → bend stencils in stencil order, with the stencil's (-k)·w_v factor
  std::vector<int32_t> bstart, binc;
  std::vector<double> bfac;
};

// Scalar matrix Ã (n×n, L = Ã ⊗ I₃) in CSR with sorted columns.
struct ScalarMatrix {
  int32_t n = 0;
  std::vector<int32_t> rowptr, col;
  std::vector<double> val;
};

// LDLᵀ factor of P·Ã·Pᵀ: perm[k] = vertex eliminated k-th; L strictly lower, unit diagonal.
struct Factor {
  int32_t n = 0;
  std::vector<int32_t> perm, iperm;
  std::vector<int32_t> colptr, rowidx;  // CSC, rows ascending (backward solve gathers columns)
  std::vector<double> colval;
  std::vector<int32_t> rowptr, colidx;  // CSR, columns ascending (forward solve gathers rows)
  std::vector<double> rowval;
  std::vector<double> d, dinv;
  std::vector<int32_t> parent;          // elimination tree
  // level schedules: rows grouped by dependency depth (forward: leaves first; backward: root first)
  std::vector<int32_t> fwdLevelPtr, fwdRows, bwdLevelPtr, bwdRows;

  // Supernodal form (nested-dissection tree nodes = contiguous column ranges). For a row i of
  // supernode S = [s0, s1): CSR entries [rowptr[i], offEnd[i]) are the off-block columns (< s0,
  // all in descendant supernodes); CSC entries [offBeg[k], colptr[k+1]) of a column k in S are the
  // rows ≥ s1 (all in ancestors). The unit-lower diagonal block of S is kept as its dense inverse.
  std::vector<int32_t> snStart, snParent, snLevel, rowSn, offEnd, offBeg;
  std::vector<int64_t> snInvOff;          // offset of S's packed inverse (s(s+1)/2 entries)
  std::vector<double> invL, invLT;        // packed rows of L_SS⁻¹ and of (L_SS⁻¹)ᵀ
  std::vector<int32_t> lvlRowPtr, lvlRows; // rows grouped by supernode level (leaves = level 0)

  // Mixed precision: FP32 copies of the factor values, the dense inverses and D⁻¹, and Ã in
  // elimination order (rows and columns permuted) for the FP64 refinement residual b − Ã·x.
  std::vector<float> rowval32, colval32, invL32, invLT32, dinv32;
  std::vector<int32_t> Aptr, Acol;
  std::vector<double> Aval;

  // Numeric refactorization on the device (same pattern, new values of Ã): the CSR position of
  // each CSC entry, the position in Aval of Ã(row, column) for each CSC entry (−1 for fill) and of
  // each diagonal, and the supernodes grouped by level (leaves first).
  std::vector<int32_t> cscToCsr, aPosCsc, aPosDiag, snLevelPtr, snByLevel;
  int32_t maxRowLen = 0;
};

// Nested-dissection tree produced with an ordering: supernode ranges in elimination order.
struct SupernodeTree {
  std::vector<int32_t> start;   // ranges [start[s], start[s+1])
  std::vector<int32_t> parent;  // −1 for roots
};

void buildTopology(const Scene& s, Topology& t);
void assembleMatrix(const Scene& s, double dt, ScalarMatrix& L);
void assembleBendingRhs(const Scene& s, std::vector<double>& out);
// Nested dissection by recursive coordinate bisection of the rest positions (vertex separators
// taken from the graph of Ã), leaves in index order.
std::vector<int32_t> nestedDissection(const Scene& s, const ScalarMatrix& L, int leafSize = 24,
                                      SupernodeTree* tree = nullptr);
// Fills the supernodal fields of a factorized Factor from the tree of its ordering.
void buildSupernodal(Factor& f, const SupernodeTree& tree);
// Lanes per row (1..32) for each level and phase of the supernodal solve run by `teamCtas` CTAs
// of 256 threads, from a cost model of FP64 warp instructions: on GB300 an FP64 warp
// instruction occupies its SMSP's pipe for ~80 cycles whatever its active lanes, so narrow groups
// waste fewer lanes while wide groups spread a level's few long rows over more SMSPs.
// latencyScale weights the dependent-latency term against the issue term (1: the model as
// calibrated; the autotuner tries others).
std::vector<int32_t> chooseGroupWidths(const Factor& f, int teamCtas, double latencyScale = 1.0);
// The same for an FP32 solve run by `ctas` CTAs of `ctaThreads` threads, where latency dominates.
std::vector<int32_t> chooseGroupWidths32(const Factor& f, int ctaThreads, int ctas = 1, double latencyScale = 1.0);
// Fills the mixed-precision fields of a factorized Factor (needs the supernodal fields).
void buildMixed(Factor& f, const ScalarMatrix& A);
// Fills the refactorization maps of a factor whose supernodal and mixed fields are built.
void buildRefactorMaps(Factor& f);
// Ã's values in elimination order (Aval) for a matrix with the pattern buildMixed saw.
void refreshAval(Factor& f, const ScalarMatrix& A);

// Up-looking LDLᵀ (Davis' LDL algorithm, as in Eigen's SimplicialLDLT). Returns false on a zero pivot.
bool factorize(const ScalarMatrix& L, const std::vector<int32_t>& perm, Factor& f, std::string* err);
void buildSchedules(Factor& f);

// Regular-grid scene (Mesh::makeGrid, computeMassesFromEdges, addShearDiagonals,
// addBendingStencils and the default pins of makeScene).
struct GridSpec {
  int nx = 40, ny = 40;
  double spacing = 0.025, stiffness = 2.3e3, density = 1.0;
  double shearStiffness = 0.0, bendStiffness = 0.0;
  int bendSampling = 0, bendStride = 1;
  int massMode = 0;  // 0 edge-lumped, 1 uniform totalMass
  double totalMass = 1.0;
  int pinMode = 0;   // 0 corners of row ny-1, 1 corners of row 0, 2 row ny-1, 3 corner (0,ny-1), 4 none
};
bool gridCounts(const GridSpec& g, int* nv, int* ne, int* nb);
bool makeGrid(const GridSpec& g, Scene& s);

// Triangle mesh from OBJ text (Mesh::loadObj + makeScene's surface masses, core/mesh/Mesh.cpp:56-153,
// core/sim/Scene.cpp:44-64): "v x y z" vertices, the first three corner indices of each "f" line
// ("a", "a/b", "a/b/c", "a//c"; 1-based); distance constraints are the triangles' unique edges in
// first-seen order at `stiffness`; masses density·area/3 per corner; no pins. False with a message
// for a file the reference could not load or would index out of range.
bool makeObj(const std::string& text, double stiffness, double density, Scene& s, std::string* err);

// Hashes that decide refactorization (core/assemble/Assembler.cpp:29-92).
struct Stamp {
  uint64_t k = 0, m = 0, pin = 0, dt = 0, structure = 0;
};
Stamp computeStamp(const Scene& s, double dt);

// Validation of raw inputs; returns an error message or empty.
std::string validateScene(const Scene& s);

}  // namespace pdg
