/*
 * pd_oracle.h — CPU oracle for the per-substep Projective Dynamics loop.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker that the CUDA path is
 * compared against; only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / reference arm may load it. Nothing in the product links it.
 *
 * It restates, in plain C++ with OpenMP, the reference CPU path of pd_ipc:
 *   core/mesh/Mesh.cpp              grid / shear / bend generation, edge-lumped masses
 *   core/mesh/ConstraintColoring.cpp  Jones–Plassmann edge colouring, incidence CSRs
 *   core/energy/DistanceTerm.cpp    projection + colour-ordered scatter
 *   core/assemble/Assembler.cpp     L = M/h² + Σκ AᵀA + bend blocks, pin rows, RHS pieces
 *   core/solver/EigenDirectSolver.cpp  permute / forward / D⁻¹ / backward solve order
 *   core/sim/Integrator.cpp         stepOnce: predict, K iterations, gate, velocity
 * The LDLᵀ factorization in the reference comes from Eigen 3.4.0
 * (SimplicialLDLT, i.e. T. Davis' up-looking LDL algorithm) and its ordering
 * from Eigen's AMD. Eigen is not available here, so both are restated: the
 * factorization follows the published up-looking LDL algorithm operation for
 * operation; the default ordering is a plain minimum-degree ordering, and any
 * caller-supplied vertex permutation can replace it.
 *
 * All arithmetic is IEEE binary64 with no FMA contraction (build with
 * -ffp-contract=off), matching MSVC /fp:precise used by the reference.
 */
#ifndef PD_ORACLE_H
#define PD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_config {
  double dt;
  double gravity[3];
  double velocity_damping;
  int max_iterations;
  double rel_tolerance;
  double abs_tolerance;
  double residual_tolerance;
  int threads; /* 0 = all OpenMP threads */
  /* Over-relaxation of the iterates (Integrator.cpp:476-617; the reference reads these from
   * PD_CHEB, PD_CHEB_RHO, PD_CHEB_START, PD_CHEB_MODE, PD_CHEB_M, PD_CHEB_D):
   * 0 off, 1 ρ recurrence after cheb_start plain iterations, 2 Chebyshev roots over [m−δ, m+δ]. */
  int cheb_mode;
  double cheb_rho;
  int cheb_start;
  double cheb_m;
  double cheb_d;
} oracle_config;

/* Regular grid scene (restates makeGrid + makeScene, core/sim/Scene.cpp:39-177). */
typedef struct oracle_grid_spec {
  int nx, ny;
  double spacing;
  double stiffness;       /* structural edges */
  double density;         /* edge-lumped mass rule when mass_mode == 0 */
  double shear_stiffness; /* > 0 adds one diagonal per quad */
  double bend_stiffness;  /* > 0 adds row/column midpoint stencils */
  int bend_sampling;      /* 0 standard, 1 rows, 2 cols, 3 checkerboard */
  int bend_stride;        /* >= 1 */
  int mass_mode;          /* 0 = reference edge-lumped rule, 1 = uniform, total_mass split evenly */
  double total_mass;      /* used when mass_mode == 1 */
  int pin_mode;           /* 0 = two corners of row ny-1 (reference default), 1 = two corners of row 0,
                             2 = whole row ny-1, 3 = corner (0, ny-1) only, 4 = none */
} oracle_grid_spec;

/* Triangle mesh from OBJ text (restates Mesh::loadObj and Mesh::computeMassesFromSurfaces,
 * core/mesh/Mesh.cpp:56-153, as makeScene applies them, core/sim/Scene.cpp:44-64). Returns 0, or
 * -1 where the reference's loader fails or would index out of range. */
int oracle_obj_counts(const char* text, int* n_vertices, int* n_edges);
int oracle_make_obj(const char* text, double stiffness, double density, double* positions, double* masses,
                    uint8_t* pinned, int* edges, double* edge_rest, double* edge_k);

/* Counts of a grid scene, so callers can size the arrays of oracle_make_grid. */
void oracle_grid_counts(const oracle_grid_spec* spec, int* n_vertices, int* n_edges, int* n_bends);

/* Fills vertex / edge / bend arrays of a grid scene. Arrays sized by oracle_grid_counts. */
int oracle_make_grid(const oracle_grid_spec* spec, double* positions, double* masses, uint8_t* pinned,
                     int32_t* edge_ab, double* edge_rest, double* edge_k, int32_t* bend_abc,
                     double* bend_k);

typedef struct oracle_sim oracle_sim;

/* Creates a simulation context from raw arrays (copied). perm: optional vertex elimination
 * order (perm[k] = vertex eliminated k-th); NULL = the oracle's own minimum-degree order. */
oracle_sim* oracle_sim_create(int n, const double* positions, const double* velocities,
                              const double* masses, const uint8_t* pinned,
                              const double* pin_positions, int n_edges, const int32_t* edge_ab,
                              const double* edge_rest, const double* edge_k, int n_bends,
                              const int32_t* bend_abc, const double* bend_k,
                              const oracle_config* cfg, const int32_t* perm);
void oracle_sim_destroy(oracle_sim* s);

/* Runs `substeps` calls of stepOnce. iterations / converged (nullable) receive per-substep values. */
int oracle_sim_step(oracle_sim* s, int substeps, int32_t* iterations, uint8_t* converged);
/* The same, recording the gate residual after every iteration: trace[k·K + j] for substep k and
 * iteration j + 1 (K = max(1, max_iterations); NaN past the substep's last iteration). */
int oracle_sim_step_traced(oracle_sim* s, int substeps, double* trace);

void oracle_sim_get_state(const oracle_sim* s, double* positions, double* velocities);
void oracle_sim_set_state(oracle_sim* s, const double* positions, const double* velocities);
void oracle_sim_set_pin_positions(oracle_sim* s, const double* pin_positions);
void oracle_sim_set_config(oracle_sim* s, const oracle_config* cfg);
void oracle_sim_set_edge_stiffness(oracle_sim* s, const double* edge_k);

typedef struct oracle_stats {
  double last_residual;
  int iterations_used;
  int converged;
  int early_exit_count;
  int factorize_count;
  int analyze_count;
  int color_count;
  int64_t matrix_nnz;  /* scalar L (n x n) nonzeros */
  int64_t factor_nnz;  /* strictly lower scalar factor nonzeros */
  double max_strain;
  double mean_strain;
  double elastic_energy;
  double total_energy;
  double max_speed;
} oracle_stats;
void oracle_sim_stats(oracle_sim* s, oracle_stats* out);

/* Serial nonlinear residual of the current state (core/sim/Integrator.cpp:113-205). */
double oracle_sim_nonlinear_residual(oracle_sim* s);

/* Current factor: perm[n], colptr[n+1], rowidx[nnz], val[nnz], dinv[n] (nullable parts skipped).
 * Returns nnz. Row indices are positions in elimination order. */
int64_t oracle_sim_factor(oracle_sim* s, int32_t* perm, int32_t* colptr, int32_t* rowidx,
                          double* val, double* dinv);

/* Scalar L (n x n, vertex indexing) as CSR with sorted columns; returns nnz. */
int64_t oracle_sim_matrix(oracle_sim* s, int32_t* rowptr, int32_t* colidx, double* val);

/* One 3-column solve L x = b with the current factor (b, x: 3n interleaved, pinned rows of b
 * taken as given). */
int oracle_sim_solve(oracle_sim* s, const double* b, double* x);

/* Right-hand side of the first PD iteration for the current state: bBase + bendRhs + scatter,
 * pinned rows overwritten with the pin positions (3n interleaved). */
int oracle_sim_rhs(oracle_sim* s, const double* base, double* b, int overwrite_pins);

/* Edge colouring and incidence CSRs (ConstraintColoring). Sizes: color_of[ne], start[colors+1],
 * order[ne], vstart[n+1], vedges[2ne]. Returns colour count. */
int oracle_sim_coloring(oracle_sim* s, uint32_t* color_of, uint32_t* start, uint32_t* order,
                        uint32_t* vstart, uint32_t* vedges);

/* Bending constant RHS (assembleBendingRhs), 3n interleaved. */
void oracle_sim_bend_rhs(oracle_sim* s, double* out);

/* Loss L = mean over free vertices of |x − target|² after `substeps` substeps from the current
 * state (which is left unchanged), with the iteration count fixed at max_iterations and an
 * external per-vertex force f (3n, NULL = 0) entering the prediction as h²·f/m; and, by the
 * adjoint method with per-substep checkpoints, its gradient w.r.t. the per-edge stiffness
 * (n_edges), the initial velocities (3n) and f (3n). NULL outputs are skipped. Serial FP64. */
int oracle_sim_gradient(oracle_sim* s, int substeps, const double* targets, const double* force,
                        double* loss, double* dkappa, double* dv0, double* dforce);

/* Power iteration on the linearised PD map at the current positions (the reference's
 * _verify/iteration_spectrum.cpp): out[0], out[1] = the last two estimates of ρ(T),
 * T = I − A⁻¹(M/h² + N + Σ_s k·A_sᵀA_s); out[2], out[3] = those of λ_max(B), B = I − T. */
int oracle_sim_spectrum(oracle_sim* s, int iters, double* out);

/* Closed-form projection of one edge (DistanceTerm::projectOne). */
void oracle_project_one(const double* pa, const double* pb, double rest, double* out);

#ifdef __cplusplus
}
#endif

#endif
