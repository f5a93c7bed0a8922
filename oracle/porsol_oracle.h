/*
 * porsol_oracle.h -- C interface of the FP64 CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a plain C++ restatement of the
 * reference algorithms (OPM/opm-porsol, mimetic/IncompFlowSolverHybrid.hpp,
 * mimetic/MimeticIPEvaluator.hpp, euler/EulerUpstream_impl.hpp,
 * euler/EulerUpstreamResidual_impl.hpp, euler/CflCalculator.hpp,
 * euler/ImplicitCapillarity_impl.hpp, common/RockJfunc.hpp).  It is the
 * checker that the GPU product path is compared against; only the test-suite,
 * the smoke check and the CPU-baseline leg of the benchmark may load it.  The
 * product library never links, loads or calls it.
 *
 * Parity pins: the oracle is checked against the reference's only quantitative
 * results for this path (examples/timing_results.txt:13-16, 35-37: known-answer
 * error norms of examples/known_answer_test.cpp) and the exactness of the
 * mimetic method for linear pressure fields (examples/known_answer_test.cpp:141-157).
 */
#ifndef PORSOL_ORACLE_H
#define PORSOL_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Flattened grid interface (cells in iteration order; half-faces grouped by
 * cell in local-face order).  Same layout as porsol_grid in the product ABI. */
typedef struct orc_grid {
    int num_cells;
    const int* cell_facepos;      /* [nc+1] */
    const int* hf_neighbour;      /* [nhf]  neighbour cell or -1 on the boundary */
    const int* hf_bid;            /* [nhf]  boundary id, 0 for interior */
    const double* hf_area;        /* [nhf]  */
    const double* hf_centroid;    /* [3*nhf] */
    const double* hf_normal;      /* [3*nhf] unit outward normal */
    const double* cell_volume;    /* [nc]  */
    const double* cell_centroid;  /* [3*nc] */
} orc_grid;

/* FlowBC/SatBC type tags, same order as BCBase::BCType (BoundaryConditions.hpp:55). */
enum { ORC_BC_DIRICHLET = 0, ORC_BC_NEUMANN = 1, ORC_BC_PERIODIC = 2 };

/* ---------------- pressure (IncompFlowSolverHybrid) ---------------- */
void* orc_create(const orc_grid* g, const int* hf_flow_type, const int* hf_partner_bid);
void  orc_destroy(void* h);
int   orc_num_dofs(void* h);
int   orc_nnz(void* h);
int   orc_max_ncf(void* h);
int   orc_num_internal_faces(void* h);
/* cellfaces[nhf] (half-face -> dof), rowptr[n+1], colind[nnz], ppartner[n] (or -1) */
void  orc_get_structure(void* h, int* cellfaces, int* rowptr, int* colind, int* ppartner);
void  orc_compute_inner_products(void* h, const double* K9, const double* grav);
/* Binv: sum_c nf_c^2 values (column-major per cell); gflux: nhf values */
void  orc_get_inner_products(void* h, double* Binv, double* gflux);
/* Assemble (assembleDynamic) only. totmob/mobdens per cell. */
void  orc_assemble(void* h, const double* totmob, const double* mobdens,
                   const int* hf_flow_type, const double* hf_flow_value, const double* src);
/* S values in the CSR order of orc_get_structure, rhs[n], F[nhf], L[nc], g[nc]; do_reg flag */
void  orc_get_system(void* h, double* Svals, double* rhs, double* F, double* L, double* g, int* do_reg);
/* Full solve: assemble + (regularise) + ILU0-CG + recover.
 * dirichlet_guess: 1 = initial guess with Dirichlet rows pre-solved (AMG/KAMG
 * path, IncompFlowSolverHybrid.hpp:1521-1532), 0 = zero guess (ILU0 path).
 * Returns 0 on convergence, 1 if not converged. */
int   orc_solve(void* h, const double* totmob, const double* mobdens,
                const int* hf_flow_type, const double* hf_flow_value, const double* src,
                double tol, int maxit, int dirichlet_guess, int* iterations, double* reduction);
/* As orc_solve; seconds3[0] = assembly + recovery, seconds3[1] = ILU0 factorisation,
 * seconds3[2] = CG iterations. */
int   orc_solve_timed(void* h, const double* totmob, const double* mobdens,
                      const int* hf_flow_type, const double* hf_flow_value, const double* src,
                      double tol, int maxit, int dirichlet_guess, int* iterations, double* reduction,
                      double* seconds3);
/* As orc_solve_timed; also the CG iteration and the seconds since the CG started at which the
 * residual reduction first fell below milestone_tol (-1 and 0 if it never did). */
int   orc_solve_milestone(void* h, const double* totmob, const double* mobdens,
                          const int* bct, const double* bcv, const double* src, double tol, int maxit,
                          int dirichlet_guess, int* iterations, double* reduction, double* seconds3,
                          double milestone_tol, int* milestone_iteration, double* milestone_seconds);
void  orc_get_solution(void* h, double* pressure, double* outflux, double* facepressure);
double orc_post_process_fluxes(void* h);
/* Solve with the tensor-mobility inner product of MimeticIPAnisoRelpermEvaluator: lam = total
 * mobility tensor, rlam = sum_i rho_i lambda_i (may be NULL), 9 doubles per cell row-major.
 * Later orc_assemble/orc_solve calls return to the static inner products. */
int orc_solve_tensor(void* h, const double* lam, const double* rlam, const int* bct, const double* bcv,
                     const double* src, double tol, int maxit, int* iterations, double* reduction);
/* Adjoint gradient of J = sum_c w_c (p_c - p*_c)^2 + sum_hf u_hf v_hf of the last solve with
 * respect to ln k (mode 0: per cell; mode 1: per cell and axis, diagonal tensors).  0 = ok,
 * 1 = adjoint CG did not converge, 2 = unsupported problem (periodic, pure Neumann). */
int orc_adjoint_gradient(void* h, const double* cell_weight, const double* cell_target, const double* hf_weight,
                         int mode, double tol, double* grad, double* objective, int* iterations);

/* -------- plain CG with ILU0 on a CSR matrix (for solver unit tests) -------- */
int   orc_ilu0_cg(int n, const int* rowptr, const int* colind, const double* vals,
                  const double* b, double* x, double tol, int maxit, int* iterations, double* reduction);

/* ---------------- transport (EulerUpstream) ---------------- */
typedef struct orc_transport_opts {
    double courant_number;      /* 0.5 */
    int method_viscous, method_gravity, method_capillary;   /* 1,1,1 */
    int use_cfl_viscous, use_cfl_gravity, use_cfl_capillary; /* 1,1,1 */
    int minimum_small_steps, maximum_small_steps;           /* 1, 10000 */
    int check_sat, clamp_sat;                                /* 1, 0 */
} orc_transport_opts;

/* Rock tables of RockJfunc (common/RockJfunc.hpp:63-216): rows table_pos[r] ..
 * table_pos[r+1]-1 of (s, krw, kro, jfunc) belong to rock r; cell_rock[c] is the rock of
 * cell c (cell_to_rock_, ReservoirPropertyCommon_impl.hpp:740-781).  With J scaling the
 * capillary pressure is J(s) sigma_cos_theta / sqrt(tr K / (3 phi)). */
typedef struct orc_rock_tables {
    int num_rocks;
    const int* table_pos;
    const double* s;
    const double* krw;
    const double* kro;
    const double* jfunc;
    const int* cell_rock;
    int use_jfunction_scaling;
    double sigma_cos_theta;
} orc_rock_tables;

typedef struct orc_fluid {
    double viscosity1, viscosity2;   /* mobility_i = kr_i / viscosity_i */
    double density1, density2;
    const orc_rock_tables* rocks;    /* NULL: kr1 = s^2, kr2 = (1-s)^2, pc = 1e5 (1-s) */
} orc_fluid;

/* CFL factors of ReservoirPropertyCapillary::computeCflFactors
 * (ReservoirPropertyCapillary_impl.hpp:213-282): out[0]=cfl_factor,
 * out[1]=cfl_factor_gravity, out[2]=cfl_factor_capillary.  K9/poro are used with rock
 * tables only (may be NULL otherwise). */
void orc_cfl_factors(const orc_fluid* fl, int num_cells, const double* K9, const double* poro, double* out3);

/* EulerUpstream::transportSolve.  Returns 0 on success, 2 if the retry loop gave up,
 * 3 if a CFL step is zero, 6 for malformed rock tables.
 * sat is updated in place.  nsteps/repeats report the small-step count used. */
int orc_transport_solve(const orc_grid* g, const double* K9, const double* poro,
                        const orc_fluid* fl, const orc_transport_opts* opts,
                        const int* hf_sat_type, const double* hf_sat_value, const int* hf_partner_bid,
                        const double* outflux_hf, const double* injection,
                        double* sat, double time, const double* grav,
                        int* nsteps, int* repeats);
/* One computeResidual (EulerUpstreamResidual_impl.hpp:475-505), for kernel unit tests. */
void orc_transport_residual(const orc_grid* g, const double* K9, const double* poro, const orc_fluid* fl,
                            const orc_transport_opts* opts,
                            const int* hf_sat_type, const double* hf_sat_value, const int* hf_partner_bid,
                            const double* outflux_hf, const double* injection,
                            const double* sat, const double* grav, double* residual);
/* computeCflTime (EulerUpstream_impl.hpp:265-331) */
double orc_transport_cfl(const orc_grid* g, const double* K9, const double* poro,
                         const orc_fluid* fl, const orc_transport_opts* opts,
                         const double* outflux_hf, const double* grav);

/* ---------------- ImplicitCapillarity ---------------- */
typedef struct orc_capillary_opts {
    int method_viscous, method_gravity;   /* 1, 1 */
    int check_sat, clamp_sat;             /* 1, 0 */
    double residual_tolerance;            /* 1e-8 */
    int linsolver_type;                   /* 1: Dirichlet rows pre-solved in the initial guess */
    double update_relaxation;             /* 1.0 */
} orc_capillary_opts;

/* ImplicitCapillarity::transportSolve (euler/ImplicitCapillarity_impl.hpp:138-226).
 * pressure: an orc_create handle for the same grid and flow-BC topology whose inner products
 * were computed with zero gravity.  hf_flow_type/value: the flow BCs (periodic values are
 * replaced by 0).  sat is updated in place.  Returns 0 = ok, 1 = pressure CG did not
 * converge, 2 = saturation out of range, 4 = no bracket of the volume-matching shift,
 * 5 = root iterations exhausted (40), 6 = malformed rock tables. */
int orc_capillary_solve(void* pressure, const orc_grid* g, const double* K9, const double* poro,
                        const orc_fluid* fl, const orc_capillary_opts* opts,
                        const int* hf_sat_type, const double* hf_sat_value, const int* hf_partner_bid,
                        const int* hf_flow_type, const double* hf_flow_value,
                        const double* outflux_hf, const double* injection, double* sat, const double* grav,
                        double* shift, int* root_iterations, int* cg_iterations);

#ifdef __cplusplus
}
#endif
#endif
