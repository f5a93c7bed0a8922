// kernels.h -- host launchers of the device kernels (one translation unit per family).
#pragma once

#include "porsol_internal.h"

namespace porsol {

struct FluidParams {
    int model;
    double mu1, mu2, rho1, rho2;
};

// ---- k_mimetic.cu --------------------------------------------------------------------
// Static inner products W (packed symmetric, [npk][nc]) and gravity flux per half-face.
void launch_static_ip(int maxnf, cudaStream_t s, int nc, const int* facepos, const double* area,
                      const double* fcent, const double* fnormal, const double* cvol, const double* ccent,
                      const double* perm, const double grav[3], double* W, double* gflux, int* status);

// Per-solve inner products of the tensor-mobility evaluator (PORSOL_FLUID_TENSOR).
struct TensorIpArgs {
    int nc;
    const int* facepos;
    const double *area, *fcent, *fnormal, *cvol, *ccent, *perm;
    const double* lam;     // total mobility tensor per cell (9, row-major)
    const double* rlam;    // sum_i rho_i lambda_i per cell (9), used when gravity != 0
    int gravity;
    double g0, g1, g2;
    double* W;             // packed [npk][nc] out
    double* gflux;         // per half-face out (gravity only)
    int* status;
};
void launch_dynamic_ip_tensor(int maxnf, cudaStream_t s, const TensorIpArgs& a);

struct AssembleArgs {
    int nc;
    const int* facepos;
    const double* W;
    const double* gflux;
    bool gravity_zero;
    FluidParams fluid;
    const double* sat;       // saturation (COREY2) or total mobility (CELLWISE)
    const double* mobdens;   // CELLWISE only, may be null
    const int* kind;         // HfKind per half-face
    const double* bcval;     // FlowBC value per half-face
    const double* src;
    double* sloc;            // packed local Schur matrices [npk][nc]
    double* F;               // per half-face
    double* L;
    double* g;
    double* rrow;            // per half-face
    double* pb;              // per half-face
    double* totmob;          // per cell (out)
    double* mobdens_out;     // per cell (out)
    int* status;
};
void launch_assemble_cells(int maxnf, cudaStream_t s, const AssembleArgs& a);

// val[k] = sum of signed recipe entries of SELL slot k; val32 (optional) gets a float copy.
void launch_gather_slots(cudaStream_t s, long long nent, const int* slot_ptr, const int* slot_ent,
                         const double* sloc, double* val, float* val32);
void launch_gather_rhs(cudaStream_t s, int n, const int* rhs_ptr, const int* rhs_ent, const double* rrow,
                       const double* pb, double* rhs);
void launch_scale_entry(cudaStream_t s, double* val, const int* diag, int row, double factor, float* val32);
// Between the internal and the reference numbering of the face unknowns (perm[reference] =
// internal): y[r] = x[perm[r]] (gather = true) or y[perm[r]] = x[r] (gather = false), r < n.
void launch_permute(cudaStream_t s, int n, const int* perm, const double* x, double* y, bool gather);
// val_ref[k] = src[k] >= 0 ? val[src[k]] : 0 for k < nent (the system in the reference numbering)
void launch_gather_values(cudaStream_t s, long long nent, const int* src, const double* val, double* val_ref);

struct RecoverArgs {
    int nc;
    const int* facepos;
    const int* cf;
    const double* x;         // face pressures
    const double* W;
    const double* gflux;
    bool gravity_zero;
    const double* F;
    const double* L;
    const double* g;
    const double* totmob;
    const double* mobdens;
    double* pressure;
    double* outflux;
};
void launch_recover(int maxnf, cudaStream_t s, const RecoverArgs& a);

// postProcessFluxes over precomputed half-face pairs; max |modification| into *maxmod_bits
// (as the bit pattern of a non-negative double, reduced with atomicMax).
void launch_post_process(cudaStream_t s, int npairs, const int* pairs, double* outflux,
                         unsigned long long* maxmod_bits);
// max_c |sum_f v - src_c| -> out[0] bits, max |src| -> out[1], max |v| -> out[2]
void launch_mass_balance(cudaStream_t s, int nc, const int* facepos, const double* outflux, const double* src,
                         unsigned long long* out3);
void launch_check_finite(cudaStream_t s, long long n, const double* v, int* status);
// zero row and column rows[q] (diagonal kept), rhs[rows[q]] = 0, for q < nrows (and the FP32 copy)
void launch_pin_rows(cudaStream_t s, int nrows, const int* rows, const int* sp, const int* col, const int* rowlen,
                     double* val, float* val32, double* rhs);
// per sub-grid g: q[3 g + i] = sum of outflux over half-faces of side 2 i + 2 (1-based sides)
void launch_side_fluxes(cudaStream_t s, int ngrids, const int* cellpos, const int* facepos, const int* side,
                        const double* outflux, double* q);
// changed = 1 if bct[bhf[q]] != cached[q] for some boundary half-face q
void launch_compare_types(cudaStream_t s, int nb, const int* bhf, const int* bct, const int* cached, int* changed);

// Output fields (cell velocity, phase velocities, fractional flow, capillary pressure); any
// output pointer may be null; sat null: velocity only.
struct CellFieldArgs {
    int nc;
    const int* facepos;
    const double *fcent, *ccent, *cvol, *outflux;
    const double* sat;
    double mu1, mu2;
    double *vel, *vw, *vo, *fw, *pc;
};
void launch_cell_fields(cudaStream_t s, const CellFieldArgs& a);

// ---- k_adjoint.cu --------------------------------------------------------------------
struct AdjointArgs {
    int nc;
    int mode;                // 0: d/d ln k (one value per cell); 1: d/d ln k_{x,y,z} (three)
    const int* facepos;
    const int* cf;
    const int* kind;         // HfKind per half-face (Dirichlet faces have zero adjoint)
    const double* sloc;      // local Schur complements of the last assembly
    const double* W;
    const double* F;
    const double* L;
    const double* g;
    const double* totmob;
    const double* pressure;
    const double* x;         // forward face pressures
    const double* mu;        // adjoint face values (gradient kernel only)
    const double* wp;        // objective: cell weights, targets, half-face flux weights (may be null)
    const double* pstar;
    const double* wv;
    const double* area;      // geometry and permeability (mode 1 only)
    const double* fcent;
    const double* fnormal;
    const double* cvol;
    const double* ccent;
    const double* perm;
    double* y;               // dJ/dpi per half-face (source kernel)
    double* jc;              // J per cell (source kernel)
    double* grad;            // gradient (gradient kernel)
    int* status;
};
void launch_adjoint_source(int maxnf, cudaStream_t s, const AdjointArgs& a);
void launch_adjoint_rhs(cudaStream_t s, int n, const int* rhs_ptr, const int* rhs_ent, const int* kind,
                        const double* y, double* rhs);
void launch_adjoint_grad(int maxnf, cudaStream_t s, const AdjointArgs& a);
// Deterministic sum of x[0..n): scratch needs sum_scratch_size() doubles; the result lands
// in scratch[sum_result_index(n)].
int sum_scratch_size();
int sum_result_index(int n);
void launch_sum(cudaStream_t s, int n, const double* x, double* scratch);

}  // namespace porsol
