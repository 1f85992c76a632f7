/*
 * pd_gb300.h — C ABI of the GB300-native Projective Dynamics substep.
 *
 * Two drop-in surfaces, both plain C (pointers, sizes, status codes; no C++ or torch types):
 *
 *  1. pd_solver_*  replaces the reference's global-step solver interface
 *     IGlobalSolver / EigenDirectSolver (core/solver/IGlobalSolver.h:45-127,
 *     core/solver/EigenDirectSolver.h:33-54): analyze / factorize / analyzed / solve /
 *     parallelComponents / solveComponent / noteSolveStage / stats. The LDLᵀ factor is computed
 *     on the host once per factorize; every solve runs on the GPU.
 *
 *  2. pd_sim_*  replaces the reference's whole substep, stepOnce(SimContext&)
 *     (core/sim/Integrator.h:14-38, core/sim/Integrator.cpp:312-797), configured by the
 *     SceneConfig knobs (core/sim/Scene.h:14-137). The entire substep — predict, K PD iterations
 *     (projection, scatter with pin elimination, pinned-row overwrite, triangular solves,
 *     residual gate), velocity update — runs on the GPU; a batch of cloths runs in one launch.
 *
 * Errors: every function returns PD_OK (0) or a PD_ERR_* code; pd_last_error() returns the
 * message of the calling thread's last failure. Where the reference prints and abort()s on a
 * violated precondition (EigenDirectSolver.cpp:304-314, 363-400), these functions return
 * PD_ERR_INVALID_ARGUMENT / PD_ERR_STATE instead. A factorization failure
 * (EigenDirectSolver.cpp:284-291) returns PD_ERR_FACTORIZATION: a pd_solver is left unready, as
 * in the reference; a pd_sim keeps its previous factor and refactorizes at its next stiffness
 * or pin-mask edit (pd_sim_set_edge_stiffness, pd_sim_set_pinned) or dt change (pd_sim_set_config).
 *
 * Threading: a handle is used by one host thread at a time, except pd_solver_solve_component,
 * which three threads may call at once for the three components. All device work of a pd_sim is
 * ordered on the handle's CUDA stream.
 *
 * Devices: a process uses one GPU, the current device when it first creates a handle. Kernel
 * attributes (shared-memory limits, non-portable cluster sizes) and co-resident capacities are
 * set and cached once per process; run one process per GPU for several GPUs.
 */
#ifndef PD_GB300_H
#define PD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PD_OK 0
#define PD_ERR_INVALID_ARGUMENT 1
#define PD_ERR_STATE 2
#define PD_ERR_FACTORIZATION 3
#define PD_ERR_CUDA 4
#define PD_ERR_UNSUPPORTED 5
#define PD_ERR_NO_MEMORY 6

/* Arithmetic of the GPU substep. */
#define PD_PRECISION_FP64_EXACT 0 /* FP64, reference operation order, bit-identical to the CPU path */
#define PD_PRECISION_FP64 1       /* FP64, supernodal solve (reordered sums, FMA); matches to rounding */
#define PD_PRECISION_FP32_PROJECTION 2 /* projection in FP32 accumulated into an FP64 b; FP64 solve */
#define PD_PRECISION_FP32_SOLVE 3 /* FP32 supernodal solve + one FP64 iterative-refinement step */
#define PD_PRECISION_MIXED 4      /* FP32 arithmetic in correction form: each PD iteration adds
                                     Ã⁻¹·(b − Ã·x), computed in FP32, to positions kept as FP32 hi/lo
                                     pairs (~48-bit significands); the explicit FP32 inverse for small
                                     cloths, an FP32 supernodal solve above; state read and written
                                     as FP64 */

/* Mirror of SceneConfig (core/sim/Scene.h:14-137) plus the fields the synthetic scenes need. */
typedef struct pd_scene_config {
  double dt;                 /* substep h (default 1/120) */
  int32_t substeps_per_frame;
  double gravity[3];         /* default (0, -9.81, 0) */
  double stiffness;          /* distance constraint κ (default 2300) */
  double density;            /* edge-lumped mass density (default 1) */
  double velocity_damping;   /* k_d (default 0.02) */
  int32_t max_iterations;    /* PD iterations per substep (default 10) */
  double rel_tolerance;      /* displacement gate, used when residual_tolerance <= 0 */
  double abs_tolerance;
  double residual_tolerance; /* residual gate, × |g| (default 1e-3); <= 0 disables */
  int32_t grid_nx, grid_ny;  /* regular grid (default 40 × 40) */
  double grid_spacing;       /* default 0.025 */
  double shear_stiffness;    /* > 0: one diagonal per quad (Mesh::addShearDiagonals) */
  double bend_stiffness;     /* > 0: midpoint bend stencils (Mesh::addBendingStencils) */
  int32_t bend_sampling;     /* 0 standard, 1 rows, 2 cols, 3 checkerboard */
  int32_t bend_stride;       /* >= 1 */
  int32_t mass_mode;         /* 0: reference edge-lumped masses; 1: uniform, total_mass split evenly */
  double total_mass;
  int32_t pin_mode;          /* 0: corners of row ny-1 (reference default); 1: corners of row 0;
                                2: whole row ny-1; 3: corner (0, ny-1); 4: none */
  int32_t precision;         /* PD_PRECISION_* */
  int32_t cluster_ctas;      /* CTAs sharing one cloth: a thread-block cluster (1..16) for the
                                supernodal and FP32_SOLVE dense kernels, a team of co-resident CTAs
                                (up to the SM count) for the MIXED dense kernel; 0 = automatic
                                (the SMs shared out over the cloths), 1 = one CTA per cloth */
  int32_t dense_max_vertices; /* FP32_SOLVE / MIXED with a cluster: solve with the explicit FP32
                                 inverse of Ã when every cloth has at most this many vertices
                                 (0 = PD_DENSE_DEFAULT_MAX_VERTICES, < 0 = never) */
  /* Over-relaxed iterates, x ← x_prev + ω_k·(x_solve − x_prev), with the gate's residual taken
   * at x_solve (core/sim/Integrator.cpp:476-645; the reference reads these from the environment
   * variables PD_CHEB, PD_CHEB_RHO, PD_CHEB_START, PD_CHEB_MODE, PD_CHEB_M, PD_CHEB_D). */
  int32_t cheb_mode;         /* PD_CHEB_OFF (default), PD_CHEB_RHO, PD_CHEB_INTERVAL */
  double cheb_rho;           /* ρ of PD_CHEB_RHO (default 0.98) */
  int32_t cheb_start;        /* plain iterations before PD_CHEB_RHO blends (default 10) */
  double cheb_m, cheb_d;     /* PD_CHEB_INTERVAL: spectrum centre and half-width (default 1, 1) */
} pd_scene_config;

/* cheb_mode: ω_k = 2/(2−ρ²) at k = cheb_start+1, then 4/(4−ρ²·ω_{k−1}); or, from k = 0,
 * ω_k = 1/(m + δ·cos(π(2k+1)/(2K))) with K = max_iterations. */
#define PD_CHEB_OFF 0
#define PD_CHEB_RHO 1
#define PD_CHEB_INTERVAL 2

#define PD_DENSE_DEFAULT_MAX_VERTICES 3072

/* Borrowed host arrays describing one cloth; vectors are [x,y,z] interleaved per vertex.
 * velocities / pin_positions may be NULL (zero velocity; pins at the current positions, as
 * refreshPinPositions does, core/sim/Scene.cpp:202-207). */
typedef struct pd_mesh {
  int32_t n_vertices;
  const double* positions;
  const double* velocities;
  const double* masses;
  const uint8_t* pinned;
  const double* pin_positions;
  int32_t n_edges;
  const int32_t* edges;        /* 2 per edge (a, b) */
  const double* edge_rest;
  const double* edge_stiffness;
  int32_t n_bends;
  const int32_t* bends;        /* 3 per stencil (a, b, c), b the middle vertex */
  const double* bend_stiffness;
} pd_mesh;

/* Message of this thread's last failure ("" if none). */
const char* pd_last_error(void);
/* Fills the SceneConfig defaults (core/sim/Scene.h:14-137). */
void pd_scene_config_default(pd_scene_config* cfg);

/* ---- Scene construction: Mesh::makeGrid + makeScene (core/mesh/Mesh.cpp:12-54,155-285,
 *      core/sim/Scene.cpp:39-177). Call pd_grid_counts to size the arrays first. ---- */
int pd_grid_counts(const pd_scene_config* cfg, int32_t* n_vertices, int32_t* n_edges, int32_t* n_bends);
int pd_make_grid(const pd_scene_config* cfg, double* positions, double* masses, uint8_t* pinned,
                 int32_t* edges, double* edge_rest, double* edge_stiffness, int32_t* bends,
                 double* bend_stiffness);

/* ---- Triangle meshes from the text of an OBJ file: Mesh::loadObj + makeScene (core/mesh/
 *      Mesh.cpp:56-153, core/sim/Scene.cpp:44-64). "v x y z" vertices; the first three corner
 *      indices of each "f" line ("a", "a/b", "a/b/c", "a//c", 1-based); distance constraints are the
 *      triangles' unique edges in first-seen order at cfg->stiffness; masses cfg->density·area/3 per
 *      triangle corner; no shear, bend or pins (set pins in the returned flags). A file the
 *      reference could not load, or whose indices it would read out of range, is
 *      PD_ERR_INVALID_ARGUMENT (the reference falls back to a grid). Call pd_obj_counts to size the
 *      arrays. ---- */
int pd_obj_counts(const char* obj_text, int32_t* n_vertices, int32_t* n_edges);
int pd_make_obj(const pd_scene_config* cfg, const char* obj_text, double* positions, double* masses, uint8_t* pinned,
                int32_t* edges, double* edge_rest, double* edge_stiffness);

/* ---- Global solver: IGlobalSolver (core/solver/IGlobalSolver.h:45-127) ---- */
typedef struct pd_solver pd_solver;

typedef struct pd_solver_stats {   /* IGlobalSolver::Stats (core/solver/IGlobalSolver.h:114-126) */
  int32_t analyze_calls;
  int32_t factorize_calls;
  int32_t solve_calls;
  double last_analyze_seconds;
  double last_factorize_seconds;
  double last_solve_seconds;
  double total_factorize_seconds;
  double total_solve_seconds;
  int64_t nnz;                     /* nonzeros of the analysed 3n × 3n matrix */
  int64_t factor_nnz;              /* nonzeros of the scalar factor (shared by x, y, z) */
} pd_solver_stats;

int pd_solver_create(pd_solver** out);
int pd_solver_destroy(pd_solver* s);
/* IGlobalSolver::analyze(n, patternMatrix) (:57): symbolic work on the CSC pattern of the
 * n × n matrix (Eigen's compressed column layout; both triangles or the lower one). */
int pd_solver_analyze(pd_solver* s, int32_t n, const int32_t* col_ptr, const int32_t* row_idx);
/* IGlobalSolver::factorize(L) (:60): numeric LDLᵀ on the host, factor uploaded to the GPU.
 * The structure must equal the analysed one. Requires L = Ã ⊗ I₃ (every 3 × 3 block a scalar
 * times I₃), which holds for every energy term of this path; otherwise PD_ERR_UNSUPPORTED. */
int pd_solver_factorize(pd_solver* s, int32_t n, const int32_t* col_ptr, const int32_t* row_idx,
                        const double* values);
/* IGlobalSolver::analyzed() (:63): 1 after a successful analyze. */
int pd_solver_analyzed(const pd_solver* s);
/* IGlobalSolver::solve(b, x) (:66): host vectors of length n; blocks until x is written. */
int pd_solver_solve(pd_solver* s, const double* b, double* x);
/* IGlobalSolver::parallelComponents() (:85): 3 once analysed (L = Ã ⊗ I₃), else 1. */
int pd_solver_parallel_components(const pd_solver* s);
/* IGlobalSolver::solveComponent(c, b, x) (:94-97): solves column c alone — reads entries 3v+c of
 * b, writes only entries 3v+c of x — on the component's own device buffers and stream, so the
 * three components may be solved from three host threads at once, as the reference's Integrator
 * does (core/sim/Integrator.cpp:558-565). Calls for one component must not overlap. Each column
 * is bit-identical to that column of pd_solver_solve. */
int pd_solver_solve_component(pd_solver* s, int32_t c, const double* b, double* x);
/* IGlobalSolver::noteSolveStage(seconds) (:111). */
int pd_solver_note_solve_stage(pd_solver* s, double seconds);
/* IGlobalSolver::stats() (:126). */
int pd_solver_stats_get(const pd_solver* s, pd_solver_stats* out);

/* ---- Fused substep: stepOnce (core/sim/Integrator.cpp:312-797) ---- */
typedef struct pd_sim pd_sim;

typedef struct pd_sim_info {
  int32_t n_vertices, n_edges, n_bends;
  int32_t color_count;
  int64_t matrix_nnz;            /* scalar Ã (n × n) */
  int64_t factor_nnz;            /* strictly lower scalar factor */
  int32_t forward_levels, backward_levels;
  int32_t factorize_count;       /* SimContext::factorizeCount */
  int32_t analyze_count;
  int64_t device_bytes;          /* device memory held by this instance */
  int32_t cluster_ctas;          /* CTAs running each cloth */
  int32_t solve_kind;            /* PD_SOLVE_* */
  int32_t host_state;            /* PD_HOST_STATE_*: how pd_sim_step_host moves the bound arrays */
  int32_t device_factorize_count; /* of factorize_count: numeric refactorizations run on the GPU
                                     (same pattern, new values; every mode but FP64_EXACT) */
} pd_sim_info;

#define PD_HOST_STATE_NONE 0     /* no host arrays bound */
#define PD_HOST_STATE_COPIES 1   /* one cudaMemcpyAsync per array each way (pageable memory) */
#define PD_HOST_STATE_GRAPH 2    /* gather / scatter kernels over the host link, one CUDA graph per call */

/* How the substep kernel solves L·x = b. */
#define PD_SOLVE_LEVELS 0        /* FP64 level-scheduled rows in the reference's order */
#define PD_SOLVE_SUPERNODAL 1    /* FP64 nested-dissection supernodes */
#define PD_SOLVE_SUPERNODAL32 2  /* FP32 supernodes + one FP64 refinement step */
#define PD_SOLVE_DENSE32 3       /* explicit FP32 inverse + one FP64 refinement step */
#define PD_SOLVE_DENSE32_TEAM 4  /* MIXED: explicit FP32 inverse applied to the correction b − Ã·x
                                    by a team of co-resident CTAs per cloth */
#define PD_SOLVE_SUPERNODAL32_CORRECTION 5 /* MIXED: FP32 supernodes applied to the correction
                                              b − Ã·x, one CTA per cloth */
#define PD_SOLVE_DENSE64_TEAM 6  /* FP64 and FP32_PROJECTION (small cloths, no over-relaxation): the
                                    explicit inverse applied to the FP64 correction b − Ã·x in
                                    double-float arithmetic (FP32 pairs, error-free products and sums)
                                    by a team of co-resident CTAs per cloth; FP64-accurate positions,
                                    residual and gate (FP32_PROJECTION: the projection d_e in FP32). A
                                    requested cluster of 1-16 CTAs (cluster_ctas, pd_plan) or
                                    dense_max_vertices < 0 keeps PD_SOLVE_SUPERNODAL */

typedef struct pd_sim_stats {    /* SimContext counters (core/sim/Scene.h:161-169) */
  int32_t iterations_used;       /* of the last substep */
  int32_t converged;             /* last substep met the gate */
  int32_t early_exit_count;      /* accumulated */
  double last_residual;          /* m/s², -1 when the residual gate is disabled */
} pd_sim_stats;

/* Builds one cloth: validates and copies the arrays, colours the edges, assembles L, orders,
 * factorizes (one numeric factorization) and uploads everything to the GPU. */
int pd_sim_create(const pd_mesh* mesh, const pd_scene_config* cfg, pd_sim** out);
/* Builds a batch of independent cloths (per-instance meshes and configs) run in one launch. */
int pd_sim_create_batch(int32_t count, const pd_mesh* meshes, const pd_scene_config* cfgs, pd_sim** out);
int pd_sim_destroy(pd_sim* s);
int pd_sim_instance_count(const pd_sim* s);
/* Enqueues `substeps` substeps of every instance on the handle's stream and returns. */
int pd_sim_step(pd_sim* s, int32_t substeps);
int pd_sim_synchronize(pd_sim* s);
/* Uses a caller-owned cudaStream_t (passed as void*) for all later work; NULL = default stream. */
int pd_sim_set_stream(pd_sim* s, void* cuda_stream);
/* Copies positions / velocities (3n, nullable) of one instance to / from the host; the get
 * waits for the handle's queued work. */
int pd_sim_get_state(pd_sim* s, int32_t instance, double* positions, double* velocities);
int pd_sim_set_state(pd_sim* s, int32_t instance, const double* positions, const double* velocities);
/* Device addresses of an instance's position / velocity arrays (3n doubles each). */
int pd_sim_device_state(pd_sim* s, int32_t instance, double** positions, double** velocities);
/* Host-state stepping: the reference's stepOnce on SimContext::mesh.positions / velocities, which
 * live in host memory (core/sim/Integrator.cpp:312-797, core/sim/Scene.h:154-178), for a whole batch.
 * pd_sim_bind_host registers one positions and one velocities array (3n doubles, [x,y,z] per
 * vertex) per instance; they must stay allocated while bound (NULL, NULL unbinds). Each
 * pd_sim_step_host call copies every bound array in, runs `substeps` substeps (0: the copies
 * only) and copies them back, and returns when the results are in host memory.
 * - Arrays that all lie in page-locked memory (cudaHostAlloc, cudaMallocHost, cudaHostRegister)
 *   are read and written by one gather and one scatter kernel for the whole batch over the host
 *   link, and gather → substeps → scatter is captured once as a CUDA graph and replayed on every
 *   later call with the same substep count (recaptured after a refactorization, a pin-mask, dt or
 *   trace change, or a new binding). pd_sim_get_info reports PD_HOST_STATE_GRAPH.
 * - Otherwise each array is copied with its own cudaMemcpyAsync (PD_HOST_STATE_COPIES).
 * - A non-finite position fails the call with PD_ERR_INVALID_ARGUMENT: before any work for
 *   pageable arrays, after the step (whose results are then undefined) for page-locked ones.
 * The handle's stream orders the work; on the default stream a private stream carries the graph. */
int pd_sim_bind_host(pd_sim* s, double* const* positions, double* const* velocities);
int pd_sim_step_host(pd_sim* s, int32_t substeps);

/* ---- Stage times: StageTimes (core/sim/Scene.h:140-149) and resetStageTimes (core/sim/Integrator.h:20) ----
 * Seconds accumulated over the substeps stepped while timing is on (off by default). The device
 * stages are timed by one thread of the cloth's first CTA with the GPU's global timer at the
 * barriers that close each stage, so they sum to `total`: predict; local_step (projections — the
 * MIXED kernels' fused correction pass, which also scatters); scatter (the colour-ordered gather
 * of b; 0 where fused); solve (the triangular solves, or the team kernel's exchange of the
 * correction and its rows of Ã⁻¹); unpack_scan (unpack, the displacement / residual scan and the
 * gate; the team kernel's update and position exchange); velocity. `assemble` is host wall time
 * of the (re)factorizations of this instance, device refactorizations and re-uploads included.
 * While timing is on the kernels run as separately compiled timed variants (the untimed ones carry
 * no timing code); the FP32_SOLVE kernels are not timed (their device stages stay 0). */
typedef struct pd_stage_times {
  double predict, local_step, scatter, assemble, solve, unpack_scan, velocity, total;
} pd_stage_times;
int pd_sim_set_stage_timing(pd_sim* s, int32_t enable);
int pd_sim_get_stage_times(pd_sim* s, int32_t instance, pd_stage_times* out);
int pd_sim_reset_stage_times(pd_sim* s);

/* ---- Spectrum of the linearised PD iteration (the reference's _verify/iteration_spectrum.cpp) ----
 * At instance i's current positions: T = I − A⁻¹(M/h² + N + K_b), N = Σ_e κ_e A_eᵀ(n_e n_eᵀ)A_e with
 * n_e = unit(x_a − x_b), K_b = Σ_s k·A_sᵀA_s (bending stencils, whose projection is constant; the
 * reference's tool refuses them), pinned rows zeroed; B = I − T. `power_iterations` steps of power
 * iteration from the reference's start vector (std::mt19937(12345), (rng() % 2000)/1000 − 1 per
 * free component in vertex order), on the GPU with the FP64 supernodal solve. Returns the last
 * ‖y‖/‖x‖ estimates and the ones before them (their gap shows whether the iteration has
 * settled), λ_min(B) = 1 − ρ(T) and the Chebyshev rate (1 − √(λ_min/λ_max)) / (1 + √(λ_min/λ_max)).
 * Blocks until done; the state is unchanged. */
typedef struct pd_spectrum {
  double rho_plain;        /* ρ(T): predicted contraction per plain PD iteration */
  double rho_plain_prev;
  double lambda_max;       /* λ_max(B) */
  double lambda_max_prev;
  double lambda_min;       /* 1 − ρ(T) */
  double rho_cheb;         /* Chebyshev semi-iteration rate over [λ_min, λ_max] */
} pd_spectrum;
int pd_sim_spectrum(pd_sim* s, int32_t instance, int32_t power_iterations, pd_spectrum* out);

/* ---- Launch plan and autotuner (the north star's "level-group and tile sizes chosen by an
 * autotuner"; no counterpart in the reference, whose solve runs on host threads) ----
 * A plan overrides the planner's built-in choices; 0 keeps the built-in choice of a field. */
typedef struct pd_plan {
  int32_t team_ctas;         /* CTAs per cloth: the team kernels' team (built-in: the SMs shared
                                out over the cloths; one cloth's team trimmed to the CTAs that own
                                rows, 146 for a 40×40 cloth on 152 SMs), or the thread-block
                                cluster of the supernodal kernels (takes precedence over
                                pd_scene_config.cluster_ctas) */
  int32_t big_min_vertices;  /* MIXED batches above the explicit-inverse limit: cloths of at least
                                this many vertices run as clusters on a second stream (built-in
                                8192; < 0: none) */
  int32_t big_cluster_ctas;  /* CTAs of each of those clusters (built-in 4) */
  int32_t work_threads;      /* MIXED batches above the explicit-inverse limit: 256 = one 256-thread
                                CTA per cloth, all launched at once (with the large cloths on
                                clusters as above; built-in); 512 or 1024 = the batch as a work table:
                                resident CTAs of this many threads take the cloths largest first from
                                a counter until none is left (no clusters) */
  double latency_scale;      /* weight of the dependent-latency term against the issue term in the
                                lanes-per-row model of every supernodal level (built-in 1) */
} pd_plan;

#define PD_TUNE_MAX_CANDIDATES 32
/* Times candidate plans for this handle's own workload and keeps the fastest: the team size of
 * the team kernel; the large-cloth threshold and cluster size of a batch; the CTAs per cloth of a
 * supernodal kernel; then the latency weight of the lane model for the best of those. Each
 * candidate is re-planned and re-uploaded, starts from the handle's current state, runs one
 * warm-up substep and then `substeps` timed substeps (CUDA events on the handle's stream). The
 * state, pin targets and counters are restored afterwards, so tuning does not advance the
 * simulation; the per-substep iteration logs and residual trace are cleared. FP64_EXACT keeps its
 * reference order: one candidate. Results of different plans differ only in rounding (the sums
 * of a row are split over other lane counts), each plan bit-reproducible. tried / ms_per_substep
 * receive up to PD_TUNE_MAX_CANDIDATES entries (nullable): the effective plan of each candidate
 * (the planner's choices filled in) and its time; *chosen indexes the kept one (candidate 0 is
 * the built-in plan). */
int pd_sim_autotune(pd_sim* s, int32_t substeps, pd_plan* tried, double* ms_per_substep, int32_t* n_tried,
                    int32_t* chosen);
/* Applies a plan (re-plans and re-uploads; the state is kept) / reads the effective plan. */
int pd_sim_set_plan(pd_sim* s, const pd_plan* plan);
int pd_sim_get_plan(pd_sim* s, pd_plan* out);
/* Moves pin targets; only the RHS changes, no refactorization (core/assemble/Assembler.h:52-60). */
int pd_sim_set_pin_positions(pd_sim* s, int32_t instance, const double* pin_positions);
/* Changes edge stiffnesses; refactorizes (the stamp changes, Assembler.cpp:111-147). */
int pd_sim_set_edge_stiffness(pd_sim* s, int32_t instance, const double* edge_stiffness);
/* Changes the pin mask; re-analyzes and refactorizes (Assembler.cpp:149-174). */
int pd_sim_set_pinned(pd_sim* s, int32_t instance, const uint8_t* pinned, const double* pin_positions);
/* Replaces the stepping knobs of every instance (SceneConfig edits between frames). The state is
 * kept. A dt change refactorizes (dt is part of L). A precision change refactorizes on the host,
 * drops the launch plan (pd_sim_set_plan / pd_sim_autotune) and re-plans, so the handle then
 * steps exactly as one created in the new mode from the same state. A cluster_ctas or
 * dense_max_vertices change re-plans and lays the device arena out again. Other fields (iteration
 * budget, tolerances, damping, Chebyshev knobs) take effect at the next step. */
int pd_sim_set_config(pd_sim* s, const pd_scene_config* cfg);
int pd_sim_get_info(pd_sim* s, int32_t instance, pd_sim_info* out);
int pd_sim_get_stats(pd_sim* s, int32_t instance, pd_sim_stats* out);
/* Per-iteration residual trace, for convergence studies like the reference's
 * _verify/residual_trace.cpp (r_k within one substep): while enabled, every launch records for each
 * substep and iteration k = 1..max_iterations the residual the gate saw after iteration k
 * (Integrator.cpp:230-263: max over free vertices of |unbalanced force| / m), NaN where the substep
 * stopped earlier. Recorded only with the residual gate (residual_tolerance > 0; a tiny tolerance
 * traces without early exits). out: substeps × max_iterations doubles of instance i from the last
 * pd_sim_step, substeps ≤ that call's count. */
int pd_sim_set_residual_trace(pd_sim* s, int32_t enable);
int pd_sim_get_residual_trace(pd_sim* s, int32_t i, double* out, int32_t substeps);

/* Per-substep iteration counts / gate flags of the last pd_sim_step (count = its substeps). */
int pd_sim_iteration_log(pd_sim* s, int32_t instance, int32_t* iterations, uint8_t* converged, int32_t count);
/* Exports the factor (perm[n], colptr[n+1], rowidx[nnz], val[nnz], dinv[n]; NULL parts skipped);
 * *nnz receives the nonzero count. */
int pd_sim_get_factor(pd_sim* s, int32_t instance, int32_t* perm, int32_t* colptr, int32_t* rowidx,
                      double* val, double* dinv, int64_t* nnz);
/* Runs one 3-column solve with the instance's factor: b, x host arrays of 3n. */
int pd_sim_solve(pd_sim* s, int32_t instance, const double* b, double* x);

/* ---- Differentiation (no counterpart in the reference) ----
 * For every instance i: the loss L_i = mean over free vertices of |x − targets[i]|² after
 * `substeps` substeps from the current state, with the iteration count fixed at max_iterations
 * (the convergence gate is not differentiated) and an external per-vertex force forces[i] (3n,
 * NULL = 0) entering the prediction as x̂ = x + h·v + h²·g + h²·f/m; and, by the adjoint method in
 * FP64 with per-substep checkpoints, its gradient w.r.t. the per-edge stiffness (dkappa[i], n_edges),
 * the current velocities (dv0[i], 3n) and the force (dforce[i], 3n). All arrays are host memory,
 * one pointer per instance; loss may be NULL, and an instance whose three gradient pointers are
 * NULL gets its loss only. The state is left unchanged. One CTA per instance; a batch of problems
 * runs in one launch. Blocks until the results are copied back. */
int pd_sim_gradient(pd_sim* s, int32_t substeps, const double* const* targets, const double* const* forces,
                    double* loss, double* const* dkappa, double* const* dv0, double* const* dforce);

/* ---- Host-only inspection (no GPU work): the preparation pd_sim_create performs ---- */
/* Assembles L, orders and factorizes as pd_sim_create does; exports the factor like
 * pd_sim_get_factor (call once with NULL arrays to read *nnz) and fills *info (nullable). */
int pd_scene_factor(const pd_mesh* mesh, const pd_scene_config* cfg, int32_t* perm, int32_t* colptr,
                    int32_t* rowidx, double* val, double* dinv, int64_t* nnz, pd_sim_info* info);
/* Edge colouring (color_of[n_edges]) of the scene; returns the colour count in *colors. */
int pd_scene_coloring(const pd_mesh* mesh, uint32_t* color_of, int32_t* colors);

/* ---- Allocation-free solve (no counterpart in the reference) ----
 * For callers that cannot call cudaMalloc where they solve: a host engine that only hands out
 * device memory from its own pool, a real-time loop where allocation is banned, a plugin host
 * that owns the device heap. It solves L x = b for the three x/y/z columns and allocates
 * nothing: every argument is a DEVICE pointer owned by the caller — the factor exactly as
 * pd_sim_get_factor / pd_scene_factor export it (perm[n], colptr[n+1], rowidx[nnz], val[nnz],
 * dinv[n]) and b, x of 3n doubles ([x,y,z] per vertex) — and the only workspace is a fixed
 * device array built into the library (3 doubles per vertex, PD_NOALLOC_MAX_VERTICES vertices,
 * 1.5 MiB) that every GPU which loads the library holds until the process exits.
 * - n > PD_NOALLOC_MAX_VERTICES is rejected with PD_ERR_INVALID_ARGUMENT.
 * - The first call on a device looks up the workspace's device address for that device; make
 *   that first call before any stream capture on the device.
 * - Every call shares the one workspace: calls whose work overlaps on the GPU (different
 *   streams, or different host threads on one device) race; serialise them on one stream.
 *   The workspace needs no clearing: each call overwrites all of it that it reads.
 * - The arithmetic follows the reference's solve order, so x is bit-identical to pd_sim_solve on
 *   an FP64_EXACT handle; other precision modes' pd_sim_solve uses the supernodal FP64 solve and
 *   agrees with it to about 1e-10 relative.
 * - rowidx and val may be NULL only for n = 1 (a factor without off-diagonal entries otherwise
 *   still needs two non-null device pointers).
 * - The workspace address is cached per device for the process; after cudaDeviceReset (or any
 *   other reset of the device's primary context) reload the library before calling again.
 * The work is queued on `stream` (a cudaStream_t; NULL = default stream) and the call returns
 * without waiting. */
#define PD_NOALLOC_MAX_VERTICES 65536
int pd_solve_noalloc(int32_t n, const int32_t* perm, const int32_t* colptr, const int32_t* rowidx,
                     const double* val, const double* dinv, const double* b, double* x, void* stream);

#ifdef __cplusplus
}
#endif

#endif
