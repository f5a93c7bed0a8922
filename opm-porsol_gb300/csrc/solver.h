// solver.h -- the pressure-solver handle behind the C ABI.
#pragma once

#include <memory>

#include "amg.h"
#include "batch.h"
#include "kernels.h"
#include "krylov.h"
#include "structure.h"
#include "upscale.h"

struct porsol_solver {
    cudaStream_t stream = nullptr;
    int device = 0;
    std::string err;

    bool structure_valid = false, ip_valid = false, solved = false;
    porsol::Structure S;
    int maxnf = 6, npk = 21;

    // geometry / topology on the device
    porsol::DBuf<int> facepos, cf, pairs;
    porsol::DBuf<double> area, fcent, fnormal, cvol, ccent;
    // static inner products
    porsol::DBuf<double> perm, W, gflux;
    bool gravity_zero = true;
    double grav_[3] = {0.0, 0.0, 0.0};
    // tensor mobilities (PORSOL_FLUID_TENSOR): per-solve inner products and gravity fluxes
    porsol::DBuf<double> Wdyn, gflux_dyn, ones;
    const double* W_last = nullptr;   // inner products of the last assembly
    const double* gflux_last = nullptr;   // ... its gravity fluxes
    bool gzero_last = true;               // ... and whether gravity entered it
    bool tensor_last = false;
    porsol::DBuf<int> status;
    porsol::DBuf<unsigned long long> redbits;

    // assembly
    porsol::Recipe R;
    std::vector<int> recipe_types;   // boundary FlowBC types the recipe was built for
    porsol::DBuf<int> recipe_types_d, boundary_hf_d;
    porsol::DBuf<double> sloc, F, L, g, rrow, pb, totmob, mobdens, rhs, x;
    porsol::DBuf<double> val;
    porsol::DBuf<float> val32;
    bool reg_applied = false;

    // host-API staging
    porsol::DBuf<double> in_sat, in_mobdens, in_bcval, in_src;
    porsol::DBuf<int> in_bctype;

    // results
    porsol::DBuf<double> pressure, outflux;
    const double* last_src = nullptr;

    // linear solvers
    porsol::PcgSolver<double, double> cg64;
    porsol::ReliableCg rcg;
    porsol::Ilu0 ilu;
    bool ilu_levels = false;
    porsol::Amg<double> amg64;
    porsol::Amg<float> amg32;
    bool amg_ready = false;
    int amg_precision = -1;
    int amg_kcycle = -1;   // the K-cycle levels the hierarchy was set up with
    porsol::DBuf<double> ir_r;   // batched residual
    // the reference numbering's system for the ILU0 path of a renumbered structure:
    // dof permutation, slot sources, values, right-hand side and solution
    porsol::DBuf<int> dof_perm_d, ref_slot_src_d;
    porsol::DBuf<double> val_ref, rhs_ref, x_ref, pi_ref;
    void ilu_solve_reference_order(const porsol_solve_opts& o, porsol_solve_stats& st, int maxit);
    porsol::RedScratch red;

    porsol::Profiler prof;

    // batched periodic upscaling: the pinned row of each sub-grid (its first DOF, the row the
    // single-grid regularisation acts on), and whether the AMG hierarchy of the previous solve
    // is reused
    std::vector<int> reg_rows;
    porsol::DBuf<int> reg_rows_d;
    bool reuse_amg = false;
    // ... and solved with one CG per sub-grid (empty: one CG over the whole system)
    porsol::BatchRanges batch;
    porsol::BatchedPcg<double, double> bcg64;
    porsol::BatchCastPrecond cast_pre;   // mixed: FP32 AMG inside the FP64 batched CG
    porsol::DBuf<double> btol, bscale, bnorm;
    void batched_solve(const porsol_solve_opts& o, porsol_solve_stats& st, int maxit);
    // ... or all three directions of every sub-grid in one persistent launch
    int upscale_schedule = PORSOL_UPSCALE_AMG;
    porsol::UpscaleSchedule upscale_fixed;   // cta_threads 0: the autotuner's choice
    porsol::UpscaleSchedule up_last;         // the schedule of the last call (zeros: AMG)
    porsol::PersistentUpscale pup;
    porsol::DBuf<double> up_b3, up_x3;
    porsol::DBuf<double> up_ones, up_zeros, up_bcv;   // device inputs of the three upscaling solves
    bool assemble_only = false;   // solve() stops after the assembly (and the pinned rows)

    // adjoint (permeability sensitivity) of the last solve
    porsol_solve_opts last_opts{};
    // algorithmic bytes of the last solve: assembly, linear solve (every CG iteration with its
    // preconditioner application, residual replacements, start), recovery, postProcessFluxes;
    // one V-cycle per level (AMG solves)
    double bytes_asm = 0, bytes_krylov = 0, bytes_rec = 0, bytes_post = 0;
    std::vector<double> vcycle_level_bytes;
    void count_krylov_bytes(const porsol_solve_opts& o, int iterations, int replacements);
    porsol::DBuf<double> adj_wp, adj_pstar, adj_wv, adj_y, adj_jc, adj_rhs, adj_x, adj_grad, adj_sum;

    void require_structure() const;
    bool same_topology(const porsol_grid* grid, const int* flow_type, const int* partner_bid) const;
    void init_structure(const porsol_grid* grid, const int* flow_type, const int* partner_bid);
    void upload_geometry(const porsol_grid* grid);
    void compute_inner_products(const double* perm_h, const double* grav);
    void solve(const porsol_fluid* fluid, const double* sat, const double* mobdens, const int* bct,
               const double* bcv, const double* src, const porsol_solve_opts* opts, porsol_solve_stats* stats,
               bool device_ptrs);
    double post_process();
    void check_status(const char* where);
    void ensure_recipe(const int* bct_host, const int* bct_dev);
    void linear_solve(const porsol_solve_opts& o, porsol_solve_stats& st);
    void recover_solution(porsol_solve_stats& st);
    // J of the last solution; leaves dJ/dpi per half-face in adj_y
    double objective(const porsol_objective* obj);
    void adjoint_gradient(const porsol_objective* obj, int mode, const porsol_solve_opts* opts, double* value,
                          double* grad, porsol_solve_stats* stats);
    void upscale(const porsol_grid* grid, int ngrids, const int* cellpos, const int* partner, const int* side,
                 const double* perm, const porsol_solve_opts* opts, double* keff, porsol_solve_stats* stats);
};
