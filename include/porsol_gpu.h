/*
 * porsol_gpu.h -- C ABI of the GB300 (sm_103a) mimetic pressure / upstream transport library.
 *
 * This is the drop-in boundary for OPM/opm-porsol's incompressible hot path.  The
 * reference is header-only C++ templates with no FFI; the C++ shim in
 * opm-porsol_gb300/host/opm/porsol/gpu/ keeps the reference's template names and
 * method signatures and forwards to the functions below.  Each entry point names the
 * reference member function it replaces (path:line inside the opm-porsol project).
 *
 * Conventions
 *   - Plain pointers and sizes only.  Functions without a `_device` suffix take host
 *     pointers; `_device` variants take device pointers (CUDA global memory of the
 *     device that was current when the handle was created).
 *   - Every call returns a porsol_status; on failure porsol_last_error() holds a
 *     message.  The C++ shim turns non-zero codes into std::runtime_error with the
 *     reference's message text.
 *   - A handle owns one CUDA stream and all device buffers.  A handle is not
 *     thread-safe; distinct handles are independent.
 *   - Cells are numbered in the grid's iteration order; half-faces are grouped by cell
 *     in the cell's local face order (the layout of the reference's SparseTable
 *     `cellFaces_` / `outflux_`, IncompFlowSolverHybrid.hpp:435-438).
 */
#ifndef PORSOL_GPU_H
#define PORSOL_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
typedef enum porsol_status {
    PORSOL_OK = 0,
    PORSOL_ERR_NOT_CONVERGED = 1,  /* linear solver hit maxit (IncompFlowSolverHybrid.hpp:1416-1419) */
    PORSOL_ERR_BAD_ARG = 2,        /* invalid argument or inconsistent grid/BC data */
    PORSOL_ERR_NONFINITE = 3,      /* NaN/Inf detected in an input or an intermediate */
    PORSOL_ERR_SAT_RANGE = 4,      /* transport retries exhausted (EulerUpstream_impl.hpp:203-207) */
    PORSOL_ERR_CUDA = 5,           /* CUDA runtime error */
    PORSOL_ERR_TIMEOUT = 6,        /* a bounded device-side wait gave up */
    PORSOL_ERR_STATE = 7,          /* call out of order (e.g. solve before init) */
    PORSOL_ERR_UNKNOWN_SOLVER = 8, /* linsolver_type not in 0..3 (IncompFlowSolverHybrid.hpp:698-700) */
    PORSOL_ERR_CFL = 9             /* CFL computation gave dt = 0 (CflCalculator.hpp:75-77) */
} porsol_status;

/* FlowBC / SatBC type tags, same order as BCBase::BCType (BoundaryConditions.hpp:55).
 * Interior half-faces carry any value (ignored). */
enum { PORSOL_BC_DIRICHLET = 0, PORSOL_BC_NEUMANN = 1, PORSOL_BC_PERIODIC = 2 };

/* --------------------------------------------------------------- grid */
/* Flattened GridInterface (GridInterfaceEuler.hpp:126-214, 346-360, 441-470). */
typedef struct porsol_grid {
    int num_cells;
    const int* cell_facepos;      /* [nc+1] half-face offsets per cell */
    const int* hf_neighbour;      /* [nhf] Face::neighbourCellIndex(), -1 on the boundary */
    const int* hf_bid;            /* [nhf] Face::boundaryId(), 0 for interior */
    const double* hf_area;        /* [nhf] Face::area() */
    const double* hf_centroid;    /* [3*nhf] Face::centroid() */
    const double* hf_normal;      /* [3*nhf] Face::normal(), unit outward */
    const double* cell_volume;    /* [nc] Cell::volume() */
    const double* cell_centroid;  /* [3*nc] Cell::centroid() */
} porsol_grid;

/* --------------------------------------------------------------- fluid */
/* FluidInterface of IncompFlowSolverHybrid::solve (MimeticIPEvaluator.hpp:297-311).
 * PORSOL_FLUID_CELLWISE: the caller passes total mobility and sum(rho_i * mob_i) per cell.
 * PORSOL_FLUID_COREY2: two phases, kr1 = s^2, kr2 = (1-s)^2 (ReservoirPropertyCapillary
 *   without rock tables, ReservoirPropertyCapillary_impl.hpp:118-170), mob_i = kr_i/visc_i,
 *   evaluated on the GPU from the saturation.
 * PORSOL_FLUID_TENSOR: the inner product of MimeticIPAnisoRelpermEvaluator
 *   (mimetic/MimeticIPAnisoRelpermEvaluator.hpp:207-400): the caller passes per cell the total
 *   mobility tensor lambda_t = sum_i lambda_i (9 doubles, row-major) as `sat` and
 *   sum_i rho_i lambda_i (9 doubles, may be NULL) as `mobdens`; every solve rebuilds
 *   W = (N (lambda_t K) N^T + 2 tr(lambda_t K) A (I - Q Q^T) A) / |c| and the gravity flux
 *   N (sum_i rho_i lambda_i) K g per cell on the GPU. */
enum { PORSOL_FLUID_CELLWISE = 0, PORSOL_FLUID_COREY2 = 1, PORSOL_FLUID_TENSOR = 2 };
typedef struct porsol_fluid {
    int model;
    double viscosity1, viscosity2;
    double density1, density2;
} porsol_fluid;

/* ------------------------------------------------------ pressure solver */
typedef struct porsol_solver porsol_solver;

/* linsolver_type: 0 = ILU0-preconditioned CG, 1 = AMG-preconditioned CG (default),
 * 2 = KAMG: CG preconditioned by the Krylov-accelerated cycle (the first coarse level's
 * correction is two flexible-CG steps preconditioned by that level's cycle; batched solves run the
 * V-cycle), 3 = FastAMG (runs the type-1 AMG-CG; the reference itself falls back to AMG-CG where
 * FastAMG is unavailable, IncompFlowSolverHybrid.hpp:687-697).
 * precision: PORSOL_FP64 = the plain drop-in; PORSOL_MIXED = FP32 AMG hierarchy (FP16
 * smoother matrices); single solves run FP32 CG recurrences with an FP64 solution and FP64
 * residual replacements, batched upscaling runs FP64 CG around the FP32 hierarchy. */
enum { PORSOL_FP64 = 0, PORSOL_MIXED = 1 };
typedef struct porsol_solve_opts {
    double residual_tolerance;  /* 1e-8   (IncompFlowSolverHybrid.hpp:662) */
    int linsolver_verbosity;    /* 1      (:663) */
    int linsolver_type;         /* 1      (:664) */
    int same_matrix;            /* 0      (:665) reuse the AMG hierarchy of the previous solve */
    int linsolver_maxit;        /* 0      (:666) 0 = number of unknowns */
    double prolongate_factor;   /* 1.6    (:667) coarse-correction damping */
    int smooth_steps;           /* 1      (:668) pre/post smoothing sweeps */
    int precision;              /* PORSOL_FP64 */
    double inner_tolerance;     /* mixed only: residual drop that triggers an FP64 residual replacement (3e-3) */
    int max_outer;              /* reserved (ignored; kept for layout compatibility) */
} porsol_solve_opts;

typedef struct porsol_solve_stats {
    int iterations;          /* CG iterations (sum of inner iterations in mixed mode) */
    int outer_iterations;    /* FP64 residual replacements (mixed single solves), 1 otherwise */
    double reduction;        /* final ||r||/||r0|| */
    int amg_levels;          /* levels of the AMG hierarchy (0 for ILU0) */
    double mass_balance;     /* max_c |sum_f v - q_c| / max(max_c |q_c|, max_f |v_f|), FP64 */
    double ms_assemble;      /* wall time of the phases of this solve (host clock, stream synchronised) */
    double ms_precond_setup;
    double ms_krylov;
    double ms_recover;
} porsol_solve_stats;

void porsol_solve_opts_default(porsol_solve_opts* opts);

int porsol_create(porsol_solver** out);
void porsol_destroy(porsol_solver* h);
const char* porsol_last_error(const porsol_solver* h);

/* IncompFlowSolverHybrid::clear (IncompFlowSolverHybrid.hpp:498-516). */
int porsol_clear(porsol_solver* h);

/* IncompFlowSolverHybrid::initSystemStructure (IncompFlowSolverHybrid.hpp:534-545):
 * enumerate face DOFs (:956-1110) and build the sparsity of S incl. periodic couplings
 * (:1115-1319).  hf_flow_type is FlowBC::type of each boundary half-face, used only to
 * find periodic faces; hf_partner_bid is getPeriodicPartner(boundaryId) (may be NULL
 * when nothing is periodic). */
int porsol_init_system_structure(porsol_solver* h, const porsol_grid* grid,
                                 const int* hf_flow_type, const int* hf_partner_bid);

/* IncompFlowSolverHybrid::computeInnerProducts (IncompFlowSolverHybrid.hpp:565-578) with
 * MimeticIPEvaluator::buildStaticContrib (MimeticIPEvaluator.hpp:201-270).
 * perm: 9 doubles per cell, row-major permeability tensor (host).  grav: 3 doubles. */
int porsol_compute_inner_products(porsol_solver* h, const double* perm, const double* grav);
/* Same as porsol_compute_inner_products; the name `assembleStatic` survives only in
 * commented calls of the reference (common/SimulatorBase.hpp:211). */
int porsol_assemble_static(porsol_solver* h, const double* perm, const double* grav);

/* IncompFlowSolverHybrid::init (IncompFlowSolverHybrid.hpp:477-488): clear +
 * initSystemStructure + computeInnerProducts. */
int porsol_init(porsol_solver* h, const porsol_grid* grid, const double* perm, const double* grav,
                const int* hf_flow_type, const int* hf_partner_bid);

/* IncompFlowSolverHybrid::solve (IncompFlowSolverHybrid.hpp:658-703): assembleDynamic,
 * linear solve of the face-pressure system, computePressureAndFluxes.
 *   sat        [nc]  saturation (COREY2) or total mobility (CELLWISE); [9 nc] TENSOR: lambda_t
 *   mobdens    [nc]  CELLWISE: sum_i rho_i mob_i; [9 nc] TENSOR: sum_i rho_i lambda_i (may be NULL: zero)
 *   hf_flow_type/hf_flow_value [nhf]  FlowBC of each boundary half-face
 *   src        [nc]  source rates
 * opts may be NULL (defaults); stats may be NULL. */
int porsol_solve(porsol_solver* h, const porsol_fluid* fluid, const double* sat, const double* mobdens,
                 const int* hf_flow_type, const double* hf_flow_value, const double* src,
                 const porsol_solve_opts* opts, porsol_solve_stats* stats);
/* As porsol_solve with all array arguments in device memory. */
int porsol_solve_device(porsol_solver* h, const porsol_fluid* fluid, const double* sat,
                        const double* mobdens, const int* hf_flow_type, const double* hf_flow_value,
                        const double* src, const porsol_solve_opts* opts, porsol_solve_stats* stats);

/* IncompFlowSolverHybrid::postProcessFluxes (IncompFlowSolverHybrid.hpp:754-807). */
int porsol_post_process_fluxes(porsol_solver* h, double* max_modification);

/* IncompFlowSolverHybrid::getSolution (IncompFlowSolverHybrid.hpp:818-831), FlowSolution
 * (:382-447): cell pressure [nc], half-face outflux [nhf], face pressures [ndof].
 * Any pointer may be NULL. */
int porsol_get_solution(porsol_solver* h, double* pressure, double* outflux, double* face_pressure);
int porsol_get_solution_device(porsol_solver* h, const double** pressure, const double** outflux,
                               const double** face_pressure);

/* Introspection (printStats, IncompFlowSolverHybrid.hpp:849-871; printSystem :895-905). */
/* No counterpart in the reference (measurement).  Algorithmic bytes of the last solve:
 * out4[0] assembly, [1] linear solve (every CG iteration with its preconditioner application,
 * residual replacements and the start), [2] recovery, [3] the postProcessFluxes that followed
 * it (0 if none); and, for AMG solves, the bytes of one V-cycle per level (up to max_levels
 * values; vcycle_level_bytes may be NULL).  Each kernel is counted as its stored matrix entries
 * (values and column indices) read once plus every vector it gathers, reads or writes once. */
int porsol_solve_bytes(porsol_solver* h, double* out4, int max_levels, double* vcycle_level_bytes);
/* AMG hierarchy of the last type-1..3 solve: rows and stored entries per level (finest
 * first, at most max_levels written); returns the level count in *levels. */
int porsol_amg_info(porsol_solver* h, int max_levels, int* levels, int* rows, long long* entries);
int porsol_num_dofs(porsol_solver* h, int* num_dofs, int* nnz, int* max_ncf, int* num_internal_faces);
/* cellfaces [nhf], rowptr [ndof+1], colind [nnz] (CSR, sorted), ppartner [ndof] (-1 = none). */
int porsol_get_structure(porsol_solver* h, int* cellfaces, int* rowptr, int* colind, int* ppartner);
/* Static inner products: W column-major per cell (sum nf^2), gravity flux per half-face. */
int porsol_get_inner_products(porsol_solver* h, double* binv, double* gflux);
/* The assembled system of the last solve before regularisation: S values in the CSR
 * order of porsol_get_structure, rhs [ndof]. */
int porsol_get_system(porsol_solver* h, double* values, double* rhs);

/* ------------------------------------------------------ batched periodic upscaling */
/* Effective permeability of many independent sub-grids (no single-call counterpart in the
 * reference: each sub-grid and direction is what setupUpscalingConditions(Periodic)
 * (common/setupBoundaryConditions.hpp:136-157) + IncompFlowSolverHybrid::solve compute).
 * `grid` is the disjoint union of num_grids sub-grids, sub-grid g owning cells
 * [grid_cellpos[g], grid_cellpos[g+1]); every boundary half-face is periodic with partner
 * boundary id hf_partner_bid and canonical side hf_side (1..6 = x-, x+, y-, y+, z-, z+, 0 for
 * interior).  For d = x, y, z the library solves with a unit pressure drop across d (periodic
 * jump +1 on side 2d+1, -1 on side 2d+2), unit mobility, each sub-grid regularised as its own
 * pure-periodic solve, and returns k_eff[9 g + 3 i + d] = L_d * (Q_i / A_i), with Q_i the net
 * flux through the sub-grid's side 2i+2, A_i that side's area and L_d the sub-grid's extent in d.
 * The three directions share one AMG hierarchy.  opts may be NULL (AMG-CG, FP64, 1e-8). */
int porsol_upscale_periodic(porsol_solver* h, const porsol_grid* grid, int num_grids, const int* grid_cellpos,
                            const int* hf_partner_bid, const int* hf_side, const double* perm,
                            const porsol_solve_opts* opts, double* k_eff, porsol_solve_stats* stats);

/* How porsol_upscale_periodic solves the batch (a choice of this library, no counterpart in the
 * reference; every schedule solves the same systems to the same per-sub-grid test
 * ||r_g|| < residual_tolerance ||r_g^0||):
 *   PORSOL_UPSCALE_AMG         CG per sub-grid over the union with one AMG hierarchy for the
 *                              three directions (opts->linsolver_type and precision apply); the default
 *   PORSOL_UPSCALE_PERSISTENT  one persistent kernel launch (captured into a CUDA graph) solves all
 *                              sub-grids and all three directions: each sub-grid is one work item, its
 *                              Jacobi-preconditioned CG runs the three right-hand sides together inside
 *                              a cluster of CTAs, one CTA ("tile") or one warp, whatever opts->precision
 *                              says with FP32
 *                              recurrences, an FP64 solution and FP64 true residuals (replacing the FP32
 *                              one whenever it has dropped by opts->inner_tolerance) that alone decide
 *                              convergence; linsolver_maxit 0 = the largest sub-grid's face unknowns.
 * cta_threads (256, 512 or 1024), warp_max_unknowns (sub-grids with fewer face unknowns go to
 * single warps), vector_layout (0: the three directions of an unknown side by side, 1: one vector
 * per direction), cluster_ctas (1, 2 or 4) and cluster_min_unknowns (with cluster_ctas > 1,
 * sub-grids with at least this many face unknowns are solved by a cluster of that many CTAs on as
 * many SMs) fix the persistent schedule; cta_threads = 0 lets the autotuner time the candidates
 * (clusters of 1/2/4 CTAs for the sub-grids of at least half the largest one's unknowns x both
 * layouts x CTAs of 512/1024 threads x warp limits 0/4096) for a few iterations on the first batch
 * of each shape and keep the fastest. */
#define PORSOL_UPSCALE_AMG 0
#define PORSOL_UPSCALE_PERSISTENT 1
int porsol_upscale_set_schedule(porsol_solver* h, int schedule, int cta_threads, int warp_max_unknowns,
                                int vector_layout, int cluster_ctas, int cluster_min_unknowns);
/* The persistent schedule the last porsol_upscale_periodic call ran (zeros after an AMG-schedule
 * call); tuned = 1 when the autotuner chose it. */
int porsol_upscale_last_schedule(porsol_solver* h, int* cta_threads, int* warp_max_unknowns, int* vector_layout,
                                 int* cluster_ctas, int* cluster_min_unknowns, int* tuned);

/* ------------------------------------------------------ output fields */
/* The cell fields writeVtkOutput gathers (common/SimulatorUtilities.hpp:54-297), computed on the
 * GPU from the current solution (after postProcessFluxes when it was called):
 *   velocity [3 nc]  estimateCellVelocity: sum_f outflux_f (x_f - x_c) / |c|
 *   water_velocity, oil_velocity [3 nc]  computePhaseVelocities: f_w v, (1 - f_w) v
 *   fractional_flow [nc]  f_w = lambda_1 / (lambda_1 + lambda_2), Corey-2 model of `fluid`
 *   cap_pressure [nc]  computeCapPressure without rock tables: 1e5 (1 - s)
 * Host output arrays, each may be NULL; sat (host, [nc]) and fluid are needed only for the
 * saturation-dependent fields (fluid->model must then be PORSOL_FLUID_COREY2). */
int porsol_cell_fields(porsol_solver* h, const porsol_fluid* fluid, const double* sat, double* velocity,
                       double* water_velocity, double* oil_velocity, double* fractional_flow, double* cap_pressure);
/* writeField (SimulatorUtilities.hpp:290-297): the count on the first line, then one value per
 * line in the default ostream format (%g, 6 significant digits), as the reference writes it.
 * Host only; returns PORSOL_ERR_BAD_ARG if the file cannot be written. */
int porsol_write_field(const double* field, int n, const char* filename);

/* ------------------------------------------------------ adjoint permeability sensitivity */
/* No counterpart in the reference.  Objective of the last solve's solution
 *     J = sum_c w_c (p_c - p*_c)^2 + sum_hf u_hf v_hf
 * with p the cell pressures and v the half-face outfluxes of computePressureAndFluxes
 * (IncompFlowSolverHybrid.hpp:1672-1730, before postProcessFluxes).  Any array may be NULL
 * (read as zeros).  Supported for solves with zero gravity, no periodic faces and at least one
 * Dirichlet face (PORSOL_ERR_BAD_ARG otherwise). */
typedef struct porsol_objective {
    const double* cell_weight;   /* w_c, num_cells */
    const double* cell_target;   /* p*_c, num_cells */
    const double* hf_weight;     /* u_hf, num half-faces */
} porsol_objective;

/* Gradient modes: d J / d ln s_c for K_c -> s_c K_c (one value per cell, any tensor), or
 * d J / d ln k_{c,a} for a = x, y, z (three values per cell, grad[3 c + a]; diagonal tensors). */
enum { PORSOL_GRAD_LOGK = 0, PORSOL_GRAD_LOGK_AXES = 1 };

/* Forward half: J of the last solve (no linear solve). */
int porsol_objective_value(porsol_solver* h, const porsol_objective* obj, double* value);
/* Backward half: one adjoint solve with the assembled matrix of the last solve and its
 * preconditioner (no setup when the hierarchy matches opts->precision; the forward Krylov
 * iterates are not stored, only the forward solution), then the per-cell gradient.  opts NULL
 * = the options of the last solve.  grad is a host array of num_cells (mode 0) or
 * 3 num_cells (mode 1) doubles; value (may be NULL) receives J. */
int porsol_adjoint_gradient(porsol_solver* h, const porsol_objective* obj, int mode, const porsol_solve_opts* opts,
                            double* value, double* grad, porsol_solve_stats* stats);

/* ------------------------------------------------------ transport */
typedef struct porsol_transport porsol_transport;

/* EulerUpstream parameters (EulerUpstream_impl.hpp:60-72, 95-108). */
typedef struct porsol_transport_opts {
    double courant_number;      /* 0.5 */
    int method_viscous, method_gravity, method_capillary;    /* 1, 1, 1 */
    int use_cfl_viscous, use_cfl_gravity, use_cfl_capillary; /* 1, 1, 1 */
    int minimum_small_steps, maximum_small_steps;            /* 1, 10000 */
    int check_sat, clamp_sat;                                 /* 1, 0 */
} porsol_transport_opts;

typedef struct porsol_transport_stats {
    int small_steps;   /* sub-steps of the successful attempt */
    int repeats;       /* retries with doubled step count */
    double cfl_dt;     /* CFL time step (after the Courant factor) */
} porsol_transport_stats;

void porsol_transport_opts_default(porsol_transport_opts* opts);
int porsol_transport_create(porsol_transport** out);
void porsol_transport_destroy(porsol_transport* t);
const char* porsol_transport_last_error(const porsol_transport* t);

/* EulerUpstream::init(param, g, r, b) / initObj (EulerUpstream_impl.hpp:111-129) with
 * EulerUpstreamResidual::initFinal (EulerUpstreamResidual_impl.hpp:403-435).
 * perm 9/cell row-major, poro 1/cell, fluid must be PORSOL_FLUID_COREY2,
 * hf_sat_type/hf_sat_value = SatBC of boundary half-faces, hf_partner_bid as above. */
int porsol_transport_init(porsol_transport* t, const porsol_grid* grid, const double* perm,
                          const double* poro, const porsol_fluid* fluid,
                          const int* hf_sat_type, const double* hf_sat_value,
                          const int* hf_partner_bid, const porsol_transport_opts* opts);

/* EulerUpstream::init(param) / setCourantNumber on an initialised solver
 * (EulerUpstream_impl.hpp:95-108, 143-147): the parameters of later transportSolve calls. */
int porsol_transport_set_options(porsol_transport* t, const porsol_transport_opts* opts);

/* EulerUpstream::transportSolve (EulerUpstream_impl.hpp:153-218): sat [nc] in/out,
 * outflux [nhf] half-face fluxes of the pressure solution, injection [nc] (may be NULL). */
int porsol_transport_solve(porsol_transport* t, double* sat, double time, const double* grav,
                           const double* outflux, const double* injection,
                           porsol_transport_stats* stats);
int porsol_transport_solve_device(porsol_transport* t, double* sat, double time, const double* grav,
                                  const double* outflux, const double* injection,
                                  porsol_transport_stats* stats);

/* Rock tables (RockJfunc, common/RockJfunc.hpp:63-216, read by
 * ReservoirPropertyCommon::readRocks, ReservoirPropertyCommon_impl.hpp:785-805): rows
 * table_pos[r] .. table_pos[r+1]-1 of the columns (s, krw, kro, jfunc) are the table of rock
 * r, s non-decreasing and jfunc monotone within a rock; cell_rock[c] is the rock of cell c
 * (cell_to_rock_, 0-based).  As the reader does, krw is set to 0 at the first row and kro
 * to 0 at the last row of each table.  With use_jfunction_scaling the capillary pressure
 * is J(s) sigma_cos_theta / sqrt(tr K / (3 phi)), else the jfunc column itself.  The
 * tables are piecewise linear with the end value outside the table. */
typedef struct porsol_rock_tables {
    int num_rocks;
    const int* table_pos;       /* [num_rocks + 1] */
    const double* s;
    const double* krw;
    const double* kro;
    const double* jfunc;
    const int* cell_rock;       /* [num_cells] */
    int use_jfunction_scaling;  /* 1 */
    double sigma_cos_theta;     /* 1.0 (RockJfunc::setSigmaAndTheta: sigma cos(theta)) */
} porsol_rock_tables;

/* ReservoirPropertyCapillary with rock tables (ReservoirPropertyCapillary_impl.hpp:118-282,
 * ReservoirPropertyCommon_impl.hpp:466-528): from now on the transport solver's phase
 * mobilities are krw/visc1 and kro/visc2 from the tables, the capillary pressure is the
 * table's, and the CFL factors (incl. the capillary one) are recomputed per rock.
 * NULL returns to kr1 = s^2, kr2 = (1-s)^2, pc = 1e5 (1-s).  PORSOL_ERR_BAD_ARG for
 * malformed tables. */
int porsol_transport_set_rock_tables(porsol_transport* t, const porsol_rock_tables* rocks);

/* ImplicitCapillarity parameters (euler/ImplicitCapillarity_impl.hpp:57-68, 91-101). */
typedef struct porsol_capillary_opts {
    int method_viscous, method_gravity;   /* 1, 1 */
    int check_sat, clamp_sat;             /* 1, 0 */
    double residual_tolerance;            /* 1e-8 */
    int linsolver_verbosity;              /* 1 */
    int linsolver_type;                   /* 1 */
    double update_relaxation;             /* 1.0 */
    int precision;                        /* PORSOL_FP64 (PORSOL_MIXED for the capillary pressure solve) */
} porsol_capillary_opts;

typedef struct porsol_capillary_stats {
    double shift;                  /* constant added to the capillary pressure (mod_correct) */
    int root_iterations;           /* regula falsi iterations */
    int evaluations;               /* saturation-volume evaluations (bracket search included) */
    porsol_solve_stats pressure;   /* the capillary pressure solve */
} porsol_capillary_stats;

void porsol_capillary_opts_default(porsol_capillary_opts* opts);

/* ImplicitCapillarity::transportSolve (euler/ImplicitCapillarity_impl.hpp:138-226): capillary
 * mobilities lambda_1 lambda_2 / (lambda_1 + lambda_2) (at least 1e-10), the viscous/gravity
 * upstream residual of the transport solver t as source, a pressure solve on p with those
 * fixed mobilities and the flow BCs (periodic jumps set to 0) for the capillary pressure, then
 * the constant shift of the capillary pressure that keeps the pore-volume-weighted saturation
 * (MatchSaturatedVolumeFunctor.hpp:49-112), found by a bracket search from 0 with step
 * max(pc) - min(pc) and regula falsi (40 iterations, |residual| <= 1e-12); the new
 * saturation is the inverse capillary-pressure curve at the shifted pressure, relaxed by
 * update_relaxation, then checked/clamped as transportSolve does.
 * p: a pressure solver initialised on the same grid and flow-BC topology with zero gravity
 * (the reference's inner solver, :80-83).  t: a transport solver on that grid, normally with
 * rock tables (without them the inverse curve is 0 everywhere, as in the reference).
 * sat [nc] in/out (unchanged on failure), outflux [nhf] half-face fluxes of the pressure
 * solution, injection [nc] (may be NULL), hf_flow_type/value the flow BCs.
 * PORSOL_ERR_NOT_CONVERGED if no shift is bracketed or regula falsi runs out of iterations
 * (or the pressure solve fails); PORSOL_ERR_SAT_RANGE when the saturation leaves
 * [-0.001, 1.001] without clamp_sat. */
int porsol_capillary_solve(porsol_transport* t, porsol_solver* p, double* sat, const double* grav,
                           const double* outflux, const double* injection, const int* hf_flow_type,
                           const double* hf_flow_value, const porsol_capillary_opts* opts,
                           porsol_capillary_stats* stats);
/* As porsol_capillary_solve with device pointers for every array (grav stays a host [3]). */
int porsol_capillary_solve_device(porsol_transport* t, porsol_solver* p, double* sat, const double* grav,
                                  const double* outflux, const double* injection, const int* hf_flow_type,
                                  const double* hf_flow_value, const porsol_capillary_opts* opts,
                                  porsol_capillary_stats* stats);

/* No counterpart in the reference.  The viscous CFL time step of the transport solver
 * (the quantity findCFLtimeVelocity bounds, before the Courant factor), for callers that may
 * not allocate device memory when they need it -- e.g. a simulator whose device memory is
 * owned by its own pool allocator, where a cudaMalloc behind the pool's back would break the
 * budget the pool manages.
 * All arrays are device pointers of the current device (layout of porsol_grid; outflux per
 * half-face, porosity per cell); *dt is a host double, so the call waits for the stream.
 * No device memory is allocated: the scratch is a fixed array inside the library (256 KiB,
 * held by every GPU that loads the library until exit), so num_cells must be <= 4,194,304
 * (PORSOL_ERR_BAD_ARG beyond).  The first call on a device (and the first after that
 * device's context was reset) looks that array's address up, so make it before any stream
 * capture.  Calls that overlap on the GPU share the array and race.  stream may be NULL.
 * Returns PORSOL_ERR_CFL (with *dt = 0) when a cell's step is zero. */
int porsol_transport_cfl_noalloc(int num_cells, const int* cell_facepos, const double* outflux,
                                 const double* cell_volume, const double* porosity, double cfl_factor,
                                 double* dt, void* stream);

/* ------------------------------------------------------ profiling */
/* Per-kernel CUDA-event timing on the handle's stream (off by default). */
int porsol_profile_enable(porsol_solver* h, int enable);
/* Accumulated launches and milliseconds of one kernel class since the last reset.
 * kernel: 0 = CG SpMV (FP64), 1 = CG SpMV (FP32), 2 = assembly, 3 = recovery,
 * 4 = whole AMG V-cycle, 5 = finest-level Chebyshev smoothing step. */
int porsol_profile_get(porsol_solver* h, int kernel, int* launches, double* ms, double* bytes);
int porsol_profile_reset(porsol_solver* h);
/* The handle's CUDA stream (cudaStream_t) for callers that time around calls. */
void* porsol_stream(porsol_solver* h);
/* Number of kernel launches this library has issued in the process so far. */
long long porsol_launch_count(void);

/* ------------------------------------------------------ self-test (no counterpart in the reference) */
/* Runs the finest-level smoother step that stages its matrix slices by bulk copy once, on a fixed
 * 64-row system on the current device, and writes its 64 outputs r, d, x (arrays of 64 floats).
 * Row i holds the values 1/4, 1/2, 3/4, 1 at columns i, i+1, i+5, i+17 (mod 64); d_j = 1 + j/64,
 * r = 2, x = 0, c1 = 1/2, c2 = 1/4, so r' = 2 - row_i . d, d' = d/2 + r'/4, x' = d + d' exactly.
 * expire != 0 makes every wait for the copies run out (about 40 ms): the step then writes nothing
 * and the call returns PORSOL_ERR_TIMEOUT with the context still usable.  Returns PORSOL_OK after a
 * normal step. */
int porsol_selftest_bulk_wait(int expire, float* r, float* d, float* x);

#ifdef __cplusplus
}
#endif
#endif /* PORSOL_GPU_H */
