// upscale.h -- batched periodic upscaling in one persistent launch.
//
// The three unit pressure-jump problems of every sub-grid (setupUpscalingConditions' pattern,
// common/setupBoundaryConditions.hpp:136-157) share one matrix: the sub-grid's block of the
// assembled union system.  PersistentUpscale solves all of them in a single kernel launch
// (captured into a CUDA graph): each sub-grid is one work item of a device queue, and the group of
// threads that takes an item runs a Jacobi-preconditioned CG for the three right-hand sides at once
// (one matrix read feeds three products; per-direction alpha, beta and stopping test) with only
// group-local barriers and reductions.  The CG recurrences run in FP32 with reliable updates: the
// solution and the true residual, which alone decides convergence, are FP64.  Two schedules share the launch:
//   * cluster: 2 or 4 CTAs on as many SMs per sub-grid, for the largest sub-grids (those of at least
//     cluster_min_unknowns unknowns), whose single-SM solve would otherwise set the launch's time;
//   * tile: a whole CTA (256, 512 or 1024 threads) per sub-grid;
//   * warp: one warp per sub-grid, for sub-grids below warp_max_unknowns unknowns.
// Items are taken largest first (cluster, tile, then warp items), so the longest solves start first.
// The autotuner times every candidate schedule for a few iterations on the batch itself and
// keeps the fastest per batch shape.
#pragma once

#include <vector>

#include "krylov.h"

namespace porsol {

struct UpscaleSchedule {
    int cta_threads = 0;         // threads of the CTA that solves a tile item
    int warp_max_unknowns = 0;   // sub-grids with fewer unknowns are solved by one warp each
    int layout = 1;              // vectors: 0 side by side (3 i + d), 1 direction-major (d n + i)
    int cluster = 1;             // CTAs per cluster item (1: no cluster items)
    int cluster_min_unknowns = 0;   // with cluster > 1: sub-grids with at least this many unknowns
    bool tuned = false;          // chosen by the autotuner (false: fixed by the caller)
};

struct UpscaleResult {
    int iterations = 0;          // CG iterations of the slowest direction of the slowest sub-grid
    double reduction = 0.0;      // largest final ||r|| / ||r0|| over sub-grids and directions
    bool converged = false;
    bool breakdown = false;
    int worst_block = -1;        // a sub-grid that did not converge (or broke down), -1 if none
};

class PersistentUpscale {
public:
    // ranges: 4 per sub-grid, the unknowns [r0, r1) and [r2, r3) (host copy and device copy).
    // b3: three right-hand sides, direction d of unknown i at 3 i + d (device); x3: the three
    // solutions (3 n, device) in the schedule's layout, read with launch_get3.  The schedule is
    // `fixed` when its cta_threads is non-zero, else the autotuner's.
    // val / val32: the system's values and their FP32 copy; delta: the drop of the FP32 residual
    // that triggers a replacement by the true FP64 residual.
    UpscaleResult solve(cudaStream_t s, const SellPattern& P, const double* val, const float* val32,
                        const std::vector<int>& ranges, const int* ranges_d, const double* b3, double* x3, double tol,
                        double delta, int maxit, const UpscaleSchedule& fixed);
    const UpscaleSchedule& last_schedule() const { return sched_; }
    // algorithmic bytes of the last solve (matrix entries once per iteration, vectors per pass)
    double bytes() const { return bytes_; }
    ~PersistentUpscale();

private:
    int n_ = 0, nblk_ = 0;
    DBuf<double> r64_, red_;
    DBuf<float> r32_, p32_, q32_, dinv_;
    DBuf<int> order_, iters_, counters_, status_;
    std::vector<int> order_h_;
    UpscaleSchedule sched_;
    double bytes_ = 0.0;
    cudaGraphExec_t exec_ = nullptr;
    std::vector<unsigned char> exec_key_;
    void launch(cudaStream_t s, const SellPattern& P, const double* val, const float* val32, const int* ranges_d,
                const double* b3, double* x3, double tol, double delta, int maxit, const UpscaleSchedule& sc,
                bool graph);
    UpscaleSchedule tune(cudaStream_t s, const SellPattern& P, const double* val, const float* val32,
                         const std::vector<int>& ranges, const int* ranges_d, const double* b3, double* x3);
    // items solved by clusters and by single CTAs under a schedule (the rest go to warps)
    void item_classes(const std::vector<int>& ranges, const UpscaleSchedule& sc, int& ncl, int& ntile) const;
    std::vector<int> rg_h_;
};

// v3[3 i + d] = v[i], i < n (one direction into the side-by-side layout), and v[i] = direction d
// of unknown i in v3 of the given layout
void launch_put3(cudaStream_t s, int n, const double* v, double* v3, int d);
void launch_get3(cudaStream_t s, int n, const double* v3, double* v, int d, int layout);
// v[i] = value, i < n
void launch_fill(cudaStream_t s, int n, double value, double* v);
// The pressure jumps of direction d (setupUpscalingConditions' pattern,
// common/setupBoundaryConditions.hpp:136-157): +1 on half-faces of side 2d+1, -1 on side 2d+2,
// 0 elsewhere (side tags 1..6, 0 inside)
void launch_jump_values(cudaStream_t s, int nhf, const int* side, int d, double* bcv);

}  // namespace porsol
