// C++ host-layer tests (include/pd_gb300.hpp) written like the reference's own chain tests:
// tests/chain/spring_vertical.cpp (one-step closed form, equilibrium, pinned vertex exact,
// factorize-once counting, linear residual with factor reuse), _verify/check.cpp items and the
// IGlobalSolver contract (core/solver/IGlobalSolver.h:45-127). Built and run by
// tests/test_cpp_host_api.py; prints "ok" and exits 0 when every check holds.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "pd_gb300.hpp"

using namespace pd::gpu;

namespace {

int failures = 0;

void expect(bool ok, const char* what) {
  if (!ok) {
    std::printf("FAILED: %s\n", what);
    ++failures;
  }
}

constexpr double H = 1.0 / 120.0, M = 0.05, ELL = 0.1, K = 1.0e4, G = 9.81;

// One free vertex hanging from a pinned one (tests/chain/spring_vertical.cpp).
SimContext spring(double y0, double kd = 0.0) {
  Mesh m;
  m.positions = {Vec3{0.0, 0.0, 0.0}, Vec3{0.0, y0, 0.0}};
  m.velocities.assign(2, Vec3{});
  m.masses = {M, M};
  m.pinned = {1, 0};
  m.pinPositions = m.positions;
  m.edges = {Edge{0, 1, ELL, K}};
  SceneConfig c;
  c.dt = H;
  c.velocityDamping = kd;
  c.maxIterations = 40;
  c.relTolerance = 0.0;
  c.absTolerance = 1e-18;
  c.residualTolerance = 1e-3;
  c.precision = PD_PRECISION_FP64_EXACT;
  return SimContext(std::move(m), c);
}

void springClosedForm() {
  SimContext ctx = spring(0.12);
  stepOnce(ctx);
  const double mh2 = M / (H * H), yhat = 0.12 - H * H * G;
  const double want = (mh2 * yhat + K * ELL) / (mh2 + K);
  expect(std::fabs(ctx.mesh.positions[1].y - want) < 1e-12, "one substep matches the closed form");
  expect(ctx.mesh.positions[0].y == 0.0, "pinned vertex exact after one substep");
}

void springEquilibriumAndCounters() {
  SimContext ctx = spring(0.12);
  double worstPin = 0.0;
  for (int s = 0; s < 20000; ++s) {
    stepOnce(ctx);
    worstPin = std::fmax(worstPin, std::fabs(ctx.mesh.positions[0].y));
  }
  expect(std::fabs(ctx.mesh.positions[1].y - (ELL - M * G / K)) < 1e-6 * ELL, "equilibrium length");
  expect(worstPin == 0.0, "pinned vertex exact over 20000 substeps");
  expect(ctx.factorizeCount == 1, "one factorization for a fixed scene");
  ctx.mesh.pinPositions[0].y = 0.01;  // a pin drag changes the RHS only
  stepOnce(ctx);
  expect(ctx.factorizeCount == 1, "pin drag does not refactorize");
  expect(ctx.mesh.positions[0].y == 0.01, "pinned vertex follows its target");
  ctx.mesh.edges[0].stiffness = 2.0 * K;  // a stiffness edit changes the stamp
  stepOnce(ctx);
  expect(ctx.factorizeCount == 2, "stiffness edit refactorizes once");
  stepOnce(ctx);
  expect(ctx.factorizeCount == 2, "and only once");
}

void gridSceneFrame() {
  SceneConfig c;
  c.gridNx = 12;
  c.gridNy = 9;
  c.gridSpacing = 0.05;
  c.shearStiffness = 800.0;
  c.bendStiffness = 30.0;
  c.precision = PD_PRECISION_MIXED;
  SimContext ctx = makeScene(c);
  const std::vector<Vec3> start = ctx.mesh.positions;
  for (int f = 0; f < 5; ++f) stepFrame(ctx);
  double moved = 0.0, pinErr = 0.0;
  for (int v = 0; v < ctx.mesh.vertexCount(); ++v) {
    const double d = std::fabs(ctx.mesh.positions[v].y - start[v].y);
    if (ctx.mesh.isPinned(v)) pinErr = std::fmax(pinErr, d);
    else moved = std::fmax(moved, d);
  }
  expect(moved > 0.0, "free vertices fall");
  expect(pinErr == 0.0, "pinned vertices stay");
  expect(ctx.iterationsUsed >= 1 && ctx.iterationsUsed <= c.maxIterations, "iterations within the budget");
}

// Ã ⊗ I₃ for a chain of n vertices (mass diagonal + κ Laplacian), CSC of the 3n × 3n matrix.
struct Csc {
  int n3 = 0;
  std::vector<int32_t> outer, inner;
  std::vector<double> values;
};

Csc chainMatrix(int n, double mh2, double k) {
  Csc A;
  A.n3 = 3 * n;
  A.outer.push_back(0);
  for (int v = 0; v < n; ++v)
    for (int c = 0; c < 3; ++c) {
      auto add = [&](int u, double val) {
        A.inner.push_back(3 * u + c);
        A.values.push_back(val);
      };
      if (v > 0) add(v - 1, -k);
      add(v, mh2 + (v > 0 ? k : 0.0) + (v + 1 < n ? k : 0.0));
      if (v + 1 < n) add(v + 1, -k);
      A.outer.push_back(static_cast<int32_t>(A.inner.size()));
    }
  return A;
}

void globalSolverContract() {
  const int n = 50;
  Csc A = chainMatrix(n, 720.0, 1.0e4);
  CscMatrix view{A.n3, A.outer.data(), A.inner.data(), A.values.data()};
  GpuDirectSolver solver;
  std::vector<double> b(A.n3, 1.0), x;
  bool threw = false;
  try {
    solver.solve(b, x);  // before analyze / factorize: a precondition violation
  } catch (const Error& e) {
    threw = e.code() == PD_ERR_STATE;
  }
  expect(threw, "solve before factorize throws PD_ERR_STATE");
  expect(!solver.analyzed(), "not analysed yet");
  solver.analyze(A.n3, view);
  expect(solver.analyzed(), "analysed");
  solver.factorize(view);
  expect(solver.parallelComponents() == 3, "three independent components");
  double worst = 0.0;
  std::srand(7);
  for (int r = 0; r < 3; ++r) {  // factor reuse: one factorization, several right-hand sides
    for (double& t : b) t = static_cast<double>(std::rand() % 2001) / 1000.0 - 1.0;
    solver.solve(b, x);
    double res = 0.0, bmax = 0.0;
    for (int col = 0; col < A.n3; ++col) bmax = std::fmax(bmax, std::fabs(b[col]));
    std::vector<double> Ax(A.n3, 0.0);
    for (int col = 0; col < A.n3; ++col)
      for (int p = A.outer[col]; p < A.outer[col + 1]; ++p) Ax[A.inner[p]] += A.values[p] * x[col];
    for (int i = 0; i < A.n3; ++i) res = std::fmax(res, std::fabs(Ax[i] - b[i]));
    worst = std::fmax(worst, res / bmax);
  }
  expect(worst < 1e-12, "linear residual below 1e-12 with the factor reused");
  std::vector<double> xc(A.n3, -7.0);
  solver.solveComponent(1, b, xc);
  bool others = true, same = true;
  for (int v = 0; v < n; ++v) {
    others = others && xc[3 * v] == -7.0 && xc[3 * v + 2] == -7.0;
    same = same && xc[3 * v + 1] == x[3 * v + 1];
  }
  expect(others, "solveComponent writes only its component");
  expect(same, "solveComponent equals the full solve on its component");
  solver.noteSolveStage(0.25);
  const GpuDirectSolver::Stats& st = solver.stats();
  expect(st.analyzeCalls == 1 && st.factorizeCalls == 1, "one analyze, one factorize");
  expect(st.solveCalls >= 3 && st.nnz == static_cast<long long>(A.values.size()), "solve count and nnz");
  Csc B = chainMatrix(n + 1, 720.0, 1.0e4);  // another structure than the analysed one
  CscMatrix other{B.n3, B.outer.data(), B.inner.data(), B.values.data()};
  threw = false;
  try {
    solver.factorize(other);
  } catch (const Error& e) {
    threw = e.code() == PD_ERR_INVALID_ARGUMENT || e.code() == PD_ERR_STATE;
  }
  expect(threw, "factorize of another structure throws");
}

}  // namespace

int main() {
  try {
    springClosedForm();
    springEquilibriumAndCounters();
    gridSceneFrame();
    globalSolverContract();
  } catch (const Error& e) {
    std::printf("FAILED: unexpected pd_gb300 error %d: %s\n", e.code(), e.what());
    return 2;
  }
  if (failures) return 1;
  std::printf("ok\n");
  return 0;
}
