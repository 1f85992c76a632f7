// pd_gb300.hpp — C++ host layer over the C ABI (pd_gb300.h), with the reference's own names:
// SceneConfig / Mesh / SimContext / makeScene / stepOnce (core/sim/Scene.h:14-244,
// core/sim/Integrator.h:14, core/mesh/Mesh.h:21-125) and the IGlobalSolver verbs of the global solve
// (core/solver/IGlobalSolver.h:45-127) in GpuDirectSolver. Header-only, C++17, no Eigen: vectors
// are std::vector<Vec3> / std::vector<double>, matrices compressed-column arrays.
//
// Differences a caller sees: where the reference prints and aborts on a precondition violation
// (core/solver/EigenDirectSolver.cpp:304-314,363-400) this layer throws pd::gpu::Error carrying the
// PD_ERR_* code; a failed factorization throws too (the reference leaves ready = false,
// :284-291). stepOnce steps on the GPU and brings ctx.mesh.positions / velocities back, so the
// SimContext stays the state of record as in the reference.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "pd_gb300.h"

namespace pd {
namespace gpu {

using Scalar = double;

struct Vec3 {
  Scalar x = 0.0, y = 0.0, z = 0.0;
};
static_assert(sizeof(Vec3) == 3 * sizeof(Scalar), "Vec3 must be three packed doubles");

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

inline void check(int rc) {
  if (rc != PD_OK) throw Error(rc, std::string("pd_gb300: ") + pd_last_error());
}

// core/sim/Scene.h:14-137, plus the synthetic-scene and GPU knobs of pd_scene_config.
struct SceneConfig {
  Scalar dt = 1.0 / 120.0;
  int substepsPerFrame = 2;
  Vec3 gravity{0.0, -9.81, 0.0};
  Scalar stiffness = 2.3e3;
  Scalar density = 1.0;
  Scalar velocityDamping = 0.02;
  int maxIterations = 10;
  Scalar relTolerance = 1.0e-3;
  Scalar absTolerance = 1.0e-12;
  Scalar residualTolerance = 1.0e-3;
  int gridNx = 40;
  int gridNy = 40;
  Scalar gridSpacing = 0.025;
  Scalar shearStiffness = 0.0;
  Scalar bendStiffness = 0.0;
  int bendSampling = 0;  // BendSampling::Standard
  int bendStride = 1;
  // not in the reference
  int massMode = 0;      // 0: the reference's edge-lumped masses; 1: uniform totalMass
  Scalar totalMass = 1.0;
  int pinMode = 0;       // 0: corners of row ny−1 (the reference's default)
  int precision = PD_PRECISION_FP64_EXACT;
  int clusterCtas = 0;
  int denseMaxVertices = 0;
  int chebMode = PD_CHEB_OFF;
  Scalar chebRho = 0.98;
  int chebStart = 10;
  Scalar chebM = 1.0, chebD = 1.0;

  pd_scene_config c() const {
    pd_scene_config o;
    pd_scene_config_default(&o);
    o.dt = dt;
    o.substeps_per_frame = substepsPerFrame;
    o.gravity[0] = gravity.x;
    o.gravity[1] = gravity.y;
    o.gravity[2] = gravity.z;
    o.stiffness = stiffness;
    o.density = density;
    o.velocity_damping = velocityDamping;
    o.max_iterations = maxIterations;
    o.rel_tolerance = relTolerance;
    o.abs_tolerance = absTolerance;
    o.residual_tolerance = residualTolerance;
    o.grid_nx = gridNx;
    o.grid_ny = gridNy;
    o.grid_spacing = gridSpacing;
    o.shear_stiffness = shearStiffness;
    o.bend_stiffness = bendStiffness;
    o.bend_sampling = bendSampling;
    o.bend_stride = bendStride;
    o.mass_mode = massMode;
    o.total_mass = totalMass;
    o.pin_mode = pinMode;
    o.precision = precision;
    o.cluster_ctas = clusterCtas;
    o.dense_max_vertices = denseMaxVertices;
    o.cheb_mode = chebMode;
    o.cheb_rho = chebRho;
    o.cheb_start = chebStart;
    o.cheb_m = chebM;
    o.cheb_d = chebD;
    return o;
  }
};

// core/mesh/Mesh.h:21-58
struct Edge {
  int a = -1;
  int b = -1;
  Scalar restLength = 0.0;
  Scalar stiffness = 0.0;
};

struct BendStencil {
  int a = -1;
  int b = -1;
  int c = -1;
  Scalar stiffness = 0.0;
};

// core/mesh/Mesh.h:90-125 (the vertex and constraint arrays)
struct Mesh {
  std::vector<Vec3> positions;
  std::vector<Vec3> velocities;
  std::vector<Scalar> masses;
  std::vector<uint8_t> pinned;
  std::vector<Vec3> pinPositions;
  std::vector<Edge> edges;
  std::vector<BendStencil> bends;

  int vertexCount() const { return static_cast<int>(positions.size()); }
  int edgeCount() const { return static_cast<int>(edges.size()); }
  int bendCount() const { return static_cast<int>(bends.size()); }
  bool isPinned(int v) const { return pinned[static_cast<size_t>(v)] != 0; }
};

// Mesh::makeGrid + makeScene's grid construction for `cfg` (pd_make_grid): positions, masses,
// default pins (pinPositions = positions), structural / shear edges and bending stencils.
inline Mesh makeGridMesh(const SceneConfig& cfg) {
  const pd_scene_config c = cfg.c();
  int32_t nv = 0, ne = 0, nb = 0;
  check(pd_grid_counts(&c, &nv, &ne, &nb));
  Mesh m;
  m.positions.resize(nv);
  m.velocities.assign(nv, Vec3{});
  m.masses.resize(nv);
  m.pinned.resize(nv);
  std::vector<int32_t> ab(2 * static_cast<size_t>(ne)), abc(3 * static_cast<size_t>(nb));
  std::vector<double> rest(ne), k(ne), bk(nb);
  check(pd_make_grid(&c, &m.positions[0].x, m.masses.data(), m.pinned.data(), ab.data(), rest.data(), k.data(),
                     abc.data(), bk.data()));
  m.pinPositions = m.positions;
  m.edges.resize(ne);
  for (int e = 0; e < ne; ++e) m.edges[e] = Edge{ab[2 * e], ab[2 * e + 1], rest[e], k[e]};
  m.bends.resize(nb);
  for (int b = 0; b < nb; ++b) m.bends[b] = BendStencil{abc[3 * b], abc[3 * b + 1], abc[3 * b + 2], bk[b]};
  return m;
}

// core/sim/Scene.h:140-149, in seconds (see pd_sim_set_stage_timing for what each stage covers
// on the GPU).
struct StageTimes {
  double predict = 0.0, localStep = 0.0, scatter = 0.0, assemble = 0.0, solve = 0.0, unpackScan = 0.0,
         velocity = 0.0, total = 0.0;
};

// core/sim/Scene.h:151-192: the configuration, the mesh (the state of record, on the host) and the
// counters stepOnce maintains; the GPU copy of the scene lives in the pd_sim handle.
class SimContext {
 public:
  SceneConfig config;
  Mesh mesh;
  StageTimes times;  // filled while stage timing is on (setStageTiming)
  int factorizeCount = 0;
  int iterationsUsed = 0;
  int earlyExitCount = 0;
  bool converged = false;
  Scalar lastResidual = -1.0;

  SimContext(Mesh m, const SceneConfig& cfg) : config(cfg), mesh(std::move(m)) {
    const pd_scene_config c = config.c();
    const pd_mesh pm = view();
    check(pd_sim_create(&pm, &c, &h_));
    remember();
    pullCounters();
  }
  SimContext(const SimContext&) = delete;
  SimContext& operator=(const SimContext&) = delete;
  SimContext(SimContext&& o) noexcept { *this = std::move(o); }
  SimContext& operator=(SimContext&& o) noexcept {
    if (this != &o) {
      release();
      config = std::move(o.config);
      mesh = std::move(o.mesh);
      factorizeCount = o.factorizeCount;
      iterationsUsed = o.iterationsUsed;
      earlyExitCount = o.earlyExitCount;
      converged = o.converged;
      lastResidual = o.lastResidual;
      h_ = o.h_;
      o.h_ = nullptr;
      lastK_ = std::move(o.lastK_);
      lastPinned_ = std::move(o.lastPinned_);
      lastPins_ = std::move(o.lastPins_);
      lastCfg_ = o.lastCfg_;
      times = o.times;
      timing_ = o.timing_;
      boundX_ = boundV_ = nullptr;  // re-bound at the next step
    }
    return *this;
  }
  ~SimContext() { release(); }

  pd_sim* handle() const { return h_; }

  void setStageTiming(bool on) {
    check(pd_sim_set_stage_timing(h_, on ? 1 : 0));
    timing_ = on;
  }

  // Field by field (a byte compare would also see the struct's padding, which c() leaves
  // unspecified, and call pd_sim_set_config on every substep).
  static bool sameConfig(const pd_scene_config& a, const pd_scene_config& b) {
    return a.dt == b.dt && a.substeps_per_frame == b.substeps_per_frame && a.gravity[0] == b.gravity[0] &&
           a.gravity[1] == b.gravity[1] && a.gravity[2] == b.gravity[2] && a.stiffness == b.stiffness &&
           a.density == b.density && a.velocity_damping == b.velocity_damping &&
           a.max_iterations == b.max_iterations && a.rel_tolerance == b.rel_tolerance &&
           a.abs_tolerance == b.abs_tolerance && a.residual_tolerance == b.residual_tolerance &&
           a.grid_nx == b.grid_nx && a.grid_ny == b.grid_ny && a.grid_spacing == b.grid_spacing &&
           a.shear_stiffness == b.shear_stiffness && a.bend_stiffness == b.bend_stiffness &&
           a.bend_sampling == b.bend_sampling && a.bend_stride == b.bend_stride && a.mass_mode == b.mass_mode &&
           a.total_mass == b.total_mass && a.pin_mode == b.pin_mode && a.precision == b.precision &&
           a.cluster_ctas == b.cluster_ctas && a.dense_max_vertices == b.dense_max_vertices &&
           a.cheb_mode == b.cheb_mode && a.cheb_rho == b.cheb_rho && a.cheb_start == b.cheb_start &&
           a.cheb_m == b.cheb_m && a.cheb_d == b.cheb_d;
  }

  // What the reference's stepOnce reads from the context at each substep: edits of the pin
  // targets go to the GPU as RHS changes; edits of the stiffnesses, the pin mask or dt refactorize
  // there (the reference's stamp rule, core/assemble/Assembler.cpp:111-174). Bending stiffness
  // and mass edits need a new SimContext.
  void pushEdits() {
    const size_t ne = mesh.edges.size(), n = mesh.positions.size();
    bool kChanged = false;
    for (size_t e = 0; e < ne && !kChanged; ++e) kChanged = mesh.edges[e].stiffness != lastK_[e];
    if (kChanged) {
      for (size_t e = 0; e < ne; ++e) lastK_[e] = mesh.edges[e].stiffness;
      check(pd_sim_set_edge_stiffness(h_, 0, lastK_.data()));
    }
    if (mesh.pinned != lastPinned_) {
      check(pd_sim_set_pinned(h_, 0, mesh.pinned.data(), &mesh.pinPositions[0].x));
      lastPinned_ = mesh.pinned;
      lastPins_ = mesh.pinPositions;
    }
    bool pinsMoved = false;
    for (size_t v = 0; v < n && !pinsMoved; ++v)
      pinsMoved = mesh.pinPositions[v].x != lastPins_[v].x || mesh.pinPositions[v].y != lastPins_[v].y ||
                  mesh.pinPositions[v].z != lastPins_[v].z;
    if (pinsMoved) {
      check(pd_sim_set_pin_positions(h_, 0, &mesh.pinPositions[0].x));
      lastPins_ = mesh.pinPositions;
    }
    const pd_scene_config c = config.c();
    if (!sameConfig(c, lastCfg_)) {
      check(pd_sim_set_config(h_, &c));
      lastCfg_ = c;
    }
  }

  // One substep on the GPU from mesh.positions / velocities, written back into them.
  int step() {
    pushEdits();
    double* x = &mesh.positions[0].x;
    double* v = &mesh.velocities[0].x;
    if (x != boundX_ || v != boundV_) {  // the vectors moved (or first step): bind them again
      check(pd_sim_bind_host(h_, &x, &v));
      boundX_ = x;
      boundV_ = v;
    }
    check(pd_sim_step_host(h_, 1));
    pullCounters();
    return iterationsUsed;
  }

 private:
  pd_mesh view() {
    static thread_local std::vector<int32_t> ab, abc;
    static thread_local std::vector<double> rest, k, bk;
    ab.clear();
    rest.clear();
    k.clear();
    abc.clear();
    bk.clear();
    for (const Edge& e : mesh.edges) {
      ab.push_back(e.a);
      ab.push_back(e.b);
      rest.push_back(e.restLength);
      k.push_back(e.stiffness);
    }
    for (const BendStencil& s : mesh.bends) {
      abc.push_back(s.a);
      abc.push_back(s.b);
      abc.push_back(s.c);
      bk.push_back(s.stiffness);
    }
    if (mesh.velocities.size() != mesh.positions.size()) mesh.velocities.assign(mesh.positions.size(), Vec3{});
    if (mesh.pinPositions.size() != mesh.positions.size()) mesh.pinPositions = mesh.positions;
    pd_mesh pm{};
    pm.n_vertices = mesh.vertexCount();
    pm.positions = &mesh.positions[0].x;
    pm.velocities = &mesh.velocities[0].x;
    pm.masses = mesh.masses.data();
    pm.pinned = mesh.pinned.data();
    pm.pin_positions = &mesh.pinPositions[0].x;
    pm.n_edges = mesh.edgeCount();
    pm.edges = ab.data();
    pm.edge_rest = rest.data();
    pm.edge_stiffness = k.data();
    pm.n_bends = mesh.bendCount();
    pm.bends = abc.data();
    pm.bend_stiffness = bk.data();
    return pm;
  }
  void remember() {
    lastK_.resize(mesh.edges.size());
    for (size_t e = 0; e < mesh.edges.size(); ++e) lastK_[e] = mesh.edges[e].stiffness;
    lastPinned_ = mesh.pinned;
    lastPins_ = mesh.pinPositions;
    lastCfg_ = config.c();
  }
  void pullCounters() {
    pd_sim_stats st{};
    check(pd_sim_get_stats(h_, 0, &st));
    pd_sim_info info{};
    check(pd_sim_get_info(h_, 0, &info));
    iterationsUsed = st.iterations_used;
    converged = st.converged != 0;
    earlyExitCount = st.early_exit_count;
    lastResidual = st.last_residual;
    factorizeCount = info.factorize_count;
    if (timing_) {
      pd_stage_times t{};
      check(pd_sim_get_stage_times(h_, 0, &t));
      times = StageTimes{t.predict, t.local_step, t.scatter, t.assemble, t.solve, t.unpack_scan, t.velocity, t.total};
    }
  }
  void release() {
    if (h_) pd_sim_destroy(h_);
    h_ = nullptr;
  }

  pd_sim* h_ = nullptr;
  bool timing_ = false;
  double* boundX_ = nullptr;
  double* boundV_ = nullptr;
  std::vector<double> lastK_;
  std::vector<uint8_t> lastPinned_;
  std::vector<Vec3> lastPins_;
  pd_scene_config lastCfg_{};
};

// core/sim/Scene.h:244: the grid scene of `config`, factorized once.
inline SimContext makeScene(const SceneConfig& config) { return SimContext(makeGridMesh(config), config); }

// core/sim/Integrator.h:14: one substep; returns the PD iterations used.
inline int stepOnce(SimContext& ctx) { return ctx.step(); }

// core/sim/Integrator.h:20
inline void resetStageTimes(SimContext& ctx) {
  check(pd_sim_reset_stage_times(ctx.handle()));
  ctx.times = StageTimes{};
}

// core/sim/Integrator.h:17: substepsPerFrame substeps.
inline void stepFrame(SimContext& ctx) {
  for (int s = 0; s < ctx.config.substepsPerFrame; ++s) ctx.step();
}

// Eigen's compressed-column storage of an n × n matrix (outer = column pointers, inner = rows).
struct CscMatrix {
  int n = 0;
  const int32_t* outer = nullptr;
  const int32_t* inner = nullptr;
  const double* values = nullptr;
};

// IGlobalSolver (core/solver/IGlobalSolver.h:45-127): analyze / factorize on the host, every solve
// on the GPU.
class GpuDirectSolver {
 public:
  struct Stats {  // IGlobalSolver::Stats (:114-125)
    int analyzeCalls = 0;
    int factorizeCalls = 0;
    int solveCalls = 0;
    double lastAnalyzeSeconds = 0.0;
    double lastFactorizeSeconds = 0.0;
    double lastSolveSeconds = 0.0;
    double totalFactorizeSeconds = 0.0;
    double totalSolveSeconds = 0.0;
    long long nnz = 0;
    long long factorNnz = 0;
  };

  GpuDirectSolver() { check(pd_solver_create(&h_)); }
  ~GpuDirectSolver() {
    if (h_) pd_solver_destroy(h_);
  }
  GpuDirectSolver(const GpuDirectSolver&) = delete;
  GpuDirectSolver& operator=(const GpuDirectSolver&) = delete;

  void analyze(int n, const CscMatrix& A) { check(pd_solver_analyze(h_, n, A.outer, A.inner)); }
  void factorize(const CscMatrix& L) { check(pd_solver_factorize(h_, L.n, L.outer, L.inner, L.values)); }
  bool analyzed() const { return pd_solver_analyzed(h_) != 0; }
  void solve(const std::vector<double>& b, std::vector<double>& x) {
    x.resize(b.size());
    check(pd_solver_solve(h_, b.data(), x.data()));
  }
  int parallelComponents() const { return pd_solver_parallel_components(h_); }
  void solveComponent(int c, const std::vector<double>& b, std::vector<double>& x) {
    if (x.size() != b.size()) throw Error(PD_ERR_INVALID_ARGUMENT, "solveComponent: x must be pre-sized like b");
    check(pd_solver_solve_component(h_, c, b.data(), x.data()));
  }
  void noteSolveStage(double seconds) { check(pd_solver_note_solve_stage(h_, seconds)); }
  const Stats& stats() const {
    pd_solver_stats s{};
    check(pd_solver_stats_get(h_, &s));
    stats_ = Stats{s.analyze_calls,        s.factorize_calls,        s.solve_calls,
                   s.last_analyze_seconds, s.last_factorize_seconds, s.last_solve_seconds,
                   s.total_factorize_seconds, s.total_solve_seconds, s.nnz, s.factor_nnz};
    return stats_;
  }

 private:
  pd_solver* h_ = nullptr;
  mutable Stats stats_;
};

}  // namespace gpu
}  // namespace pd
