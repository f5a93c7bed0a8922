// batch.h -- preconditioned CG over block-diagonal systems, one independent CG per block.
//
// Batched periodic upscaling solves the disjoint union of many sub-grids as one system.  One
// CG over the union converges at the rate of its whole spectrum: every sub-grid contributes
// its own smallest eigenvalue (its regularised constant mode), so the union needs several times
// the iterations of its hardest sub-grid.  BatchedPcg runs the CG recurrences per block instead
// (per-block alpha, beta, residual norm and stopping test) while every kernel still sweeps the
// whole union: the iteration count is that of the slowest sub-grid.  The preconditioner must be
// block diagonal too (an AMG hierarchy of the union is: aggregates never cross sub-grids).
#pragma once

#include "krylov.h"

namespace porsol {

// Block g owns the unknowns [r[4g], r[4g+1]) and [r[4g+2], r[4g+3]) (the internal and the
// boundary face unknowns of a sub-grid are each numbered contiguously).
struct BatchRanges {
    int nblk = 0, n = 0;
    std::vector<int> h;
    DBuf<int> ranges, blk;
    void build(const std::vector<int>& four_per_block, int n_unknowns, cudaStream_t s);
};

// Global state of a batched solve (device), mirrored for the host in mapped memory.
struct BatchDev {
    int iter, maxit, stop, active, breakdown, pad;
};
struct BatchHostView {
    volatile int iter, stop, active, breakdown;
};

template <class TV, class T>
class BatchedPcg {
public:
    // x holds the initial guess.  tol[g] (device, per block): stop block g when
    // ||r_g|| < tol[g] ||r_g^0|| or ||r_g|| < 1e-30.  On return def0/def (device, per block)
    // hold the initial and final residual norms.
    CgResult solve(cudaStream_t s, const SellPattern& P, const TV* val, Precond<T>& M, const BatchRanges& B,
                   const T* b, T* x, const double* tol, int maxit);
    const double* def0() const { return def0_.p; }
    const double* def() const { return def_.p; }
    ~BatchedPcg();

private:
    int n_ = 0, nblk_ = 0;
    DBuf<T> r_, z_, p_, q_;
    DBuf<double> rho_, rholast_, lambda_, beta_, def0_, def_;
    DBuf<int> conv_;   // per block: 0 active, 1 converged, 2 breakdown
    DBuf<BatchDev> st_;
    DBuf<unsigned int> counter_;
    BatchHostView* hview_ = nullptr;
    BatchHostView* dview_ = nullptr;
    std::vector<cudaEvent_t> ev_;
    cudaGraphExec_t exec_ = nullptr;
    const void* key_[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    long long key_gen_ = -1;
    long long nodes_ = 0;
    void setup(int n, int nblk, cudaStream_t s);
    void iteration(cudaStream_t s, const SellPattern& P, const TV* val, Precond<T>& M, const BatchRanges& B, T* x,
                   const double* tol);
};

// FP64 Krylov with an FP32 block-diagonal preconditioner: z = isc_g * double(M32(float(sc_g r)))
// per block g.  The preconditioner is linear and block diagonal, so the per-block scaling
// (sc = 1 / ||r0_g||, isc = ||r0_g||) only keeps the FP32 vectors in range; the CG recurrences,
// the solution and the stopping test stay FP64, so no restart is ever needed.
class BatchCastPrecond : public Precond<double> {
public:
    void bind(Precond<float>* inner, const BatchRanges* B, const double* sc, const double* isc);
    void apply(cudaStream_t s, const double* r, double* z, const int* stop) override;
    void set_block_state(const int* conv) override;   // passed to the inner preconditioner

private:
    Precond<float>* m_ = nullptr;
    const BatchRanges* B_ = nullptr;
    const double *sc_ = nullptr, *isc_ = nullptr;
    long long inner_gen_ = -1;
    DBuf<float> r32_, z32_;
};

// Per-block helper of the batched solve.
// out[g] = ||a_g||_2 (deterministic order)
template <class T>
void batch_norms(cudaStream_t s, const BatchRanges& B, const T* a, double* out);
}  // namespace porsol
