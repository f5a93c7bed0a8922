// amg.h -- aggregation AMG preconditioner on the GPU (replaces dune-istl Amg::AMG).
//
// The reference preconditions CG with dune-istl's aggregation AMG (unsmoothed
// piecewise-constant prolongation, prolongation damping factor `prolongate_factor`,
// `smooth_steps` pre/post sweeps; IncompFlowSolverHybrid.hpp:1481-1541).  This is a GPU
// design of the same method class: each level coarsens by two rounds of parallel pairwise
// matching on the symmetric strength |a_ij| / sqrt(a_ii a_jj) (aggregates of up to 4
// rows), Galerkin coarse matrices P^T A P computed row-by-row without atomics
// (deterministic), l1-Jacobi smoothing (symmetric, so the V-cycle is a symmetric
// preconditioner for CG), the coarse correction scaled by the prolongation damping
// factor, and an exact FP64 solve on the coarsest level (explicit inverse from a
// Cholesky factorisation).  The hierarchy values are type T (double or float); the
// coarsest level is always FP64.
#pragma once

#include "krylov.h"

namespace porsol {

struct AmgOpts {
    int smooth_steps = 1;
    double prolong = 1.6;
    int coarse_target = 128;
    int max_levels = 24;
    double strength = 0.08;
};

template <class T>
class Amg : public Precond<T> {
public:
    void setup(cudaStream_t s, const SellPattern& P0, const T* A0, const AmgOpts& o);
    void apply(cudaStream_t s, const T* r, T* z, const int* stop) override;
    int levels() const { return int(lv_.size()) + 1; }
    int coarse_n() const { return nc_; }
    const std::vector<int>& level_sizes() const { return sizes_; }
    // SELL entries per level (fine level first)
    const std::vector<long long>& level_nnz() const { return nnzs_; }
    ~Amg();

private:
    struct Level {
        int n = 0;                       // rows of this level
        const SellPattern* P = nullptr;  // this level's matrix
        const T* A = nullptr;
        SellPattern own;                 // storage for levels > 0
        DBuf<T> own_val;
        DBuf<T> dinv;                    // l1-Jacobi inverse diagonal
        DBuf<int> agg;                   // row -> coarse row of the next level
        DBuf<int4> children;             // next-level row -> up to 4 rows of this level
        DBuf<T> x, b, r;                 // work vectors (level 0 uses the caller's r/z)
    };
    void pairwise(cudaStream_t s, const SellPattern& P, const T* A, int n, double theta, DBuf<int>& agg,
                  DBuf<int2>& kids, int& ncoarse);
    void galerkin_pairs(cudaStream_t s, const SellPattern& P, const T* A, int n, const int* agg, const int2* kids,
                        int ncoarse, SellPattern& Pc, DBuf<T>& Ac);
    void build_coarse_solver(cudaStream_t s, const SellPattern& P, const T* A, int n);
    void vcycle(cudaStream_t s, int l, const T* b, T* x, const int* stop);

    AmgOpts o_;
    std::vector<std::unique_ptr<Level>> lv_;
    std::vector<int> sizes_;
    std::vector<long long> nnzs_;
    // coarsest level: dense FP64 inverse
    int nc_ = 0;
    const SellPattern* Pc_ = nullptr;
    const T* Ac_ = nullptr;
    DBuf<double> cinv_;
    DBuf<int> status_;
    // scratch
    DBuf<int> best_, state_, flag_, scan_;
    DBuf<int> tmp_agg_;
    DBuf<int2> tmp_kids_;
    SellPattern tmp_pat_;
    DBuf<T> tmp_val_;
    DBuf<int> scan_blocks_;
};

// Exclusive prefix sum of n ints on the device; total (if not null) written to *total_dev.
void exclusive_scan(cudaStream_t s, int n, const int* in, int* out, int* total_dev, DBuf<int>& scratch);

}  // namespace porsol
