// amg.h -- aggregation AMG preconditioner on the GPU (replaces dune-istl Amg::AMG).
//
// The reference preconditions CG with dune-istl's aggregation AMG (unsmoothed
// piecewise-constant prolongation, coarse correction scaled by `prolongate_factor`,
// `smooth_steps` pre/post smoothing steps; IncompFlowSolverHybrid.hpp:1481-1541).  This is
// a GPU design of the same method class:
//   * rows without off-diagonal couplings (Dirichlet rows) are not aggregated;
//   * each level coarsens by two rounds of parallel pairwise matching on the strength of
//     negative couplings -a_ij / sqrt(a_ii a_jj) >= 0.25; a round that stalls (keeps more
//     than 80% of its rows) is redone on |a_ij| and lets unmatched rows join the aggregate
//     of their strongest matched neighbour;
//   * Galerkin coarse matrices P^T A P are merged row by row without atomics
//     (deterministic, run-to-run reproducible);
//   * the smoother is a degree-2 Chebyshev polynomial in D^-1 A on [G/30, G], G the
//     Gershgorin bound of D^-1 A (symmetric, so the V-cycle is a valid CG preconditioner);
//   * the coarsest level is solved exactly in FP64 (explicit inverse from a Cholesky
//     factorisation), whatever the precision T of the hierarchy.
#pragma once

#include <cuda_fp16.h>

#include "krylov.h"

namespace porsol {

struct AmgOpts {
    int smooth_steps = 1;       // Chebyshev applications before and after the coarse correction
    double prolong = 1.6;       // coarse-correction damping (dune-istl prolongation damping factor)
    int coarse_target = 128;
    int max_levels = 24;
    int round3_below = 0;       // coarse levels with fewer rows pair a third time (aggregates of about
                                // eight rows): fewer of the small, launch-latency-bound levels
    double strength = 0.25;
    int cheb_degree = 2;
    bool round1_negative = true;   // first pairing round of a level on strong negative couplings
    bool round2_negative = false;  // second round likewise; off: directly |a_ij| with joins (the
                                   // negative attempt stalls on these systems and is discarded)
    bool half_smoother = true;     // FP32 hierarchies: smoother/residual read D^-1 A stored in FP16
    bool layout4 = true;           // ... from a SELL-32x4 copy on levels smoothed one thread per row
    bool bulk_stage = true;        // finest level: Chebyshev step with the slices bulk-copied to shared memory
    bool autotune = false;         // time the lane schedules of each new level shape once (the
                                   // choice then depends on timing: off where runs must be
                                   // bitwise reproducible)
    int kcycle_levels = 0;         // K-cycle: the coarse corrections of levels 1 .. kcycle_levels are
                                   // two flexible-CG steps preconditioned by the cycle of that level
                                   // (0: plain V-cycle)
};

// One finest-level bulk-staged Chebyshev step on a fixed 64-row system (expire: every wait for the
// bulk copies runs out); returns the kernel's status bits and the 64 values of r, d and x.
int bulk_step_selftest(bool expire, float* r, float* d, float* x);

// Device aggregation result: agg (row -> aggregate or -1), members CSR (aggregate -> rows).
struct Aggregates {
    int n = 0, nc = 0;
    DBuf<int> agg, ptr, idx;
};

template <class T>
class Amg : public Precond<T> {
public:
    void setup(cudaStream_t s, const SellPattern& P0, const T* A0, const AmgOpts& o);
    void apply(cudaStream_t s, const T* r, T* z, const int* stop) override;
    int levels() const { return nlev_; }
    void set_profiler(Profiler* p) { prof_ = p; }
    const std::vector<int>& level_sizes() const { return sizes_; }
    // Algorithmic bytes of one apply() (one V-cycle) of the current hierarchy, in total and per
    // level: every kernel's stored matrix entries (values + columns or 16-bit offsets) read once,
    // each vector it gathers read once, the vectors it streams read or written once.
    double apply_bytes(std::vector<double>* per_level = nullptr) const;
    const std::vector<long long>& level_nnz() const { return nnzs_; }
    // error bits set by the apply kernels (ST_TIMEOUT: a bounded wait for a bulk copy gave up);
    // synchronises the stream
    int solve_status(cudaStream_t s) const;
    // Block-diagonal systems (batched solves): blk0 maps each row of the system to its block
    // (device, null: one system).  Set before setup(); setup() carries the map down the levels.
    void set_row_blocks(const int* blk0) { blk0_ = blk0; }
    // Per-block convergence flags of the batched CG (device, 0: still iterating; null: none).
    // apply() then marks each level's slices that hold an iterating block, and its kernels leave
    // the other slices as they are: with a block-diagonal hierarchy the iterating blocks' values
    // are those of a full cycle.
    void set_block_state(const int* conv) override;

private:
    struct Level {
        int n = 0;
        const SellPattern* P = nullptr;
        const T* A = nullptr;
        SellPattern own;
        DBuf<T> own_val;
        DBuf<T> dinv;
        // FP16 copy of D^-1 A (row-scaled, so entries are O(1) whatever the units) and the
        // diagonal, read by the smoother and residual kernels of FP32 hierarchies
        DBuf<__half> ah;
        DBuf<T> diagv;
        bool half = false;
        // SELL-32x4 copy of ah (levels smoothed with one thread per row): slice offsets,
        // columns, FP16 values
        bool v4 = false;
        int bulk_groups = 0;         // > 0: the Chebyshev step stages the x4 slices by bulk copy
        DBuf<int> sp4, col4;
        DBuf<__half> ah4;
        // the x4 copy's columns as 16-bit offsets from the row (off4) when every coupling of the
        // level lies within 32767 rows of the diagonal (c16); col4 otherwise
        bool c16 = false;
        DBuf<short> off4;
        double lmax = 2.0;
        int lanes = 1;               // threads per row in the smoother/residual kernels
        Aggregates agg;              // to the next level
        DBuf<T> t, r, d0, d1, b, x;  // work vectors
        DBuf<T> kc1, kc2, kv1, kv2, kr2;   // K-cycle vectors (K-levels only)
        DBuf<int> blk;               // block of each row (levels below the first; batched solves)
        const int* blkp = nullptr;   // block of each row: blk0_ on the finest level, blk below it
        DBuf<unsigned char> act;     // per 32-row slice: 1 while a block in it iterates
    };
    const int* blk0_ = nullptr;
    const int* conv_ = nullptr;
    const unsigned char* level_act(const Level& L) const { return conv_ && L.blkp ? L.act.p : nullptr; }
    // plain-layout level smoothed one thread per row whose pattern carries 16-bit column offsets (the
    // system matrix of an FP64 or FP32-valued hierarchy): the row dots read 2 instead of 4 index bytes
    static bool plain16(const Level& L) { return !L.half && !L.v4 && L.lanes == 1 && L.P->has_off16(); }
    void aggregate_round(cudaStream_t s, const SellPattern& P, const T* A, int n, bool neg_first, Aggregates& out);
    void pairwise(cudaStream_t s, const SellPattern& P, const T* A, int n, bool neg, double theta, bool join,
                  Aggregates& out);
    void members(cudaStream_t s, Aggregates& a);
    void galerkin(cudaStream_t s, const SellPattern& P, const T* A, const Aggregates& a, SellPattern& Pc,
                  DBuf<T>& Ac);
    void smoother_setup(cudaStream_t s, Level& L, int level);
    void adopt_tmp(Level& next);
    int tune_lanes(cudaStream_t s, Level& L);
    DBuf<int> tune_stop_;
    DBuf<int> s_maxoff_;   // per level: largest |col - row| of the x4 copy (16-bit offset check)
    void build_coarse_solver(cudaStream_t s, const SellPattern& P, const T* A, int n);
    // started: the first Chebyshev start from zero (r = D^-1 b, d = r / theta) was already done by
    // the restriction that produced b (k_restrict_start0)
    void chebyshev(cudaStream_t s, Level& L, const T* b, T* x, bool from_zero, const T* xc, const int* agg,
                   const int* stop, bool started = false);
    void vcycle(cudaStream_t s, int l, const T* b, T* x, const int* stop, bool started = false);
    // coarse correction of level l - 1 solved on level l by two flexible-CG steps (K-cycle)
    void kcycle(cudaStream_t s, int l, const T* b, T* x, const int* stop, bool started = false);
    bool k_level(int l) const { return l >= 1 && l <= o_.kcycle_levels && l < nlev_ - 1; }
    double cycle_bytes(int l, std::vector<double>* per_level, bool started = false) const;
    // 1 / theta of the level's Chebyshev interval [lmax / 30, lmax]
    static double cheb_inv_theta(const Level& L) { return 1.0 / (0.5 * (L.lmax + L.lmax / 30.0)); }
    DBuf<double> kpart_, kcoef_;   // K-cycle dot partials and coefficients (8 per level)

    AmgOpts o_;
    Profiler* prof_ = nullptr;
    std::vector<std::unique_ptr<Level>> lv_;   // levels are kept and reused by later setups
    int nlev_ = 0;                              // levels in use
    // setup scratch (grow-only, reused by every setup)
    DBuf<double> s_D_, s_Linv_;
    DBuf<float> s_rs_;
    DBuf<int> s_state_, s_partner_, s_join_, s_best_, s_flag_, s_cidx_, s_cnt_, s_pos_, s_width_;
    DBuf<int> s_wl_[2], s_wlcnt_;   // matching worklists (the free rows of a sweep) and their lengths
    DBuf<unsigned long long> s_gmax_;
    DBuf<int> s_bnd_, s_goff_, s_tcol_, s_dpos_, s_woff_;   // Galerkin temporaries
    DBuf<T> s_tval_;
    Aggregates agg2_;
    std::vector<int> sizes_;
    std::vector<long long> nnzs_;
    int nc_ = 0;
    DBuf<double> cinv_;
    DBuf<int> status_;
    DBuf<int> scan_blocks_, iscratch_;
    DBuf<double> dscratch_;
    SellPattern tmp_pat_;
    DBuf<T> tmp_val_;
};

// Exclusive prefix sum of n ints on the device; the total is written to *total_dev.
void exclusive_scan(cudaStream_t s, int n, const int* in, int* out, int* total_dev, DBuf<int>& scratch);

}  // namespace porsol
