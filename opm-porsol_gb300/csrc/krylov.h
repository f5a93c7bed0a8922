// krylov.h -- SELL SpMV, preconditioned CG with device-side scalars, ILU(0).
#pragma once

#include "porsol_internal.h"

namespace porsol {

// Device-resident CG scalars.  Written by the last block of each reduction kernel; read by
// the next kernel in stream order, so no host round trip is needed per iteration.
struct CgDev {
    double rho, rholast, alpha, def0, def, tol, lambda, beta;
    int iter, maxit, converged, stop, breakdown, pad;
};

// Mirror of CgDev in mapped pinned host memory, written at the end of every iteration.
struct CgHostView {
    volatile double def0, def;
    volatile int iter, converged, stop, breakdown;
};

// Reduction scratch: partial sums per block + arrival counter (reset by the last block).
struct RedScratch {
    DBuf<double> partial;
    DBuf<unsigned int> counter;
    int max_blocks = 0;
    void ensure(int blocks, cudaStream_t s);
};

template <class T>
struct Precond {
    virtual ~Precond() = default;
    // z = M^{-1} r; kernels must do nothing when *stop != 0.  apply() must not synchronise
    // or allocate: it is captured into a CUDA graph.
    virtual void apply(cudaStream_t s, const T* r, T* z, const int* stop) = 0;
    // Batched solves: the per-block convergence flags (device, 0: block still iterating), so a
    // block-diagonal preconditioner may skip the rows of converged blocks; null for one system.
    virtual void set_block_state(const int*) {}
    // Changes whenever the kernels apply() launches change (new setup/factorisation).
    long long generation() const { return gen_; }
    void bump_generation() { ++gen_; }

private:
    long long gen_ = 0;
};

template <class TV, class TX>
void spmv(cudaStream_t s, const SellPattern& P, const TV* val, const TX* x, TX* y);

// y = b - A x  (residual)
template <class TV, class TX>
void residual(cudaStream_t s, const SellPattern& P, const TV* val, const TX* x, const TX* b, TX* y);

struct CgResult {
    int iterations = 0;
    double reduction = 0.0, def0 = 0.0, def = 0.0;
    bool converged = false, breakdown = false;
};

// Preconditioned CG, the algorithm of dune-istl's CGSolver::apply: stop when
// ||b - A x||_2 < tol ||b - A x0||_2 (or < 1e-30) or after maxit iterations.
// x holds the initial guess on entry.  TV = matrix value type, T = vector type.
template <class TV, class T>
class PcgSolver {
public:
    void setup(int n, cudaStream_t s);
    CgResult solve(cudaStream_t s, const SellPattern& P, const TV* val, Precond<T>& M, const T* b, T* x,
                   double tol, int maxit, Profiler* prof = nullptr, int prof_kernel = -1);
    // Replay one CG iteration (SpMV, updates, preconditioner) as a CUDA graph.
    void set_graphs(bool on) { use_graphs_ = on; }
    ~PcgSolver();

private:
    int n_ = 0;
    DBuf<T> r_, z_, p_, q_;
    DBuf<CgDev> st_;
    RedScratch red_;
    CgHostView* hview_ = nullptr;
    CgHostView* dview_ = nullptr;
    std::vector<cudaEvent_t> ev_;
    bool use_graphs_ = true;
    cudaGraphExec_t exec_ = nullptr;
    const void* key_[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    long long key_gen_ = -1;
    long long nodes_ = 0;   // kernels in one captured iteration
    void iteration(cudaStream_t s, const SellPattern& P, const TV* val, Precond<T>& M, T* x, Profiler* prof,
                   int prof_kernel);
};

// Mixed-precision CG with reliable updates (residual replacement; Sleijpen and van der Vorst,
// "Reliable updated residuals in hybrid Bi-CG methods", Computing 56, 1996): one FP32 CG
// recurrence (FP32 matrix copy, FP32 preconditioner) on the system scaled by sigma, the
// solution accumulated in FP64 (x += sigma alpha p), and the iterated residual replaced by the
// true FP64 residual b - A x whenever it has dropped by `delta` since the last replacement or
// the estimate reaches the tolerance.  Unlike restarted iterative refinement the search
// direction is kept across replacements (rescaled), so no Krylov information and no extra
// preconditioner application is lost.  Stops when the true residual satisfies
// ||b - A x|| < tol ||b - A x0|| (or < 1e-30).
struct RcDev {
    double rho, alpha, beta, sigma, isig, factor, def0, defs, tol, delta, true_def;
    int iter, maxit, stop, converged, breakdown, replace, nrep, pad;
};

class ReliableCg {
public:
    // prof (may be null): when per-kernel event timing is on, iterations run uncaptured
    CgResult solve(cudaStream_t s, const SellPattern& P, const double* val64, const float* val32,
                   Precond<float>& M, const double* b, double* x, double tol, int maxit, double delta,
                   Profiler* prof = nullptr);
    int replacements() const { return nrep_; }
    ~ReliableCg();

private:
    int n_ = 0, nrep_ = 0;
    DBuf<float> r_, z_, p_, q_;
    DBuf<double> r64_;
    DBuf<RcDev> st_;
    RedScratch red_;
    CgHostView* hview_ = nullptr;
    CgHostView* dview_ = nullptr;
    std::vector<cudaEvent_t> ev_;
    cudaGraphExec_t exec_ = nullptr;
    const void* key_[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    long long key_gen_ = -1;
    long long nodes_ = 0;
    void setup(int n, cudaStream_t s);
    void iteration(cudaStream_t s, const SellPattern& P, const double* val64, const float* val32, Precond<float>& M,
                   const double* b, double* x, Profiler* prof);
};

// ILU(0) with the pivots stored inverted, factor and triangular solves level-scheduled
// (rows of one level are independent).  The algorithm of dune-istl's SeqILU0 with
// relaxation 1 (IncompFlowSolverHybrid.hpp:1404).
class Ilu0 : public Precond<double> {
public:
    void build_levels(const SellPattern& P, cudaStream_t s);   // structure only
    void factor(cudaStream_t s, const SellPattern& P, const double* val);
    void apply(cudaStream_t s, const double* r, double* z, const int* stop) override;
    int num_levels_lower() const { return int(h_lptr_.size()) - 1; }
    int num_levels_upper() const { return int(h_uptr_.size()) - 1; }

private:
    const SellPattern* P_ = nullptr;
    DBuf<double> lu_;
    std::vector<int> h_lptr_, h_uptr_;
    DBuf<int> lrows_, urows_;
    DBuf<int> status_;
};

// Helpers used by the solver front end.
void device_copy(cudaStream_t s, void* dst, const void* src, size_t bytes);
template <class TA, class TB>
void convert(cudaStream_t s, long long n, const TA* a, TB* b);
// x += y (FP64)
void axpy_add(cudaStream_t s, int n, const double* y, double* x);
// Dirichlet-row initial guess (IncompFlowSolverHybrid.hpp:1521-1532): x_i = b_i / a_ii
// where all off-diagonal entries of row i are zero, else 0.
void dirichlet_guess(cudaStream_t s, const SellPattern& P, const double* val, const double* b, double* x);
// 2-norm of a vector (synchronous, FP64 accumulation)
template <class T>
double norm2(cudaStream_t s, int n, const T* x, RedScratch& red);

}  // namespace porsol
