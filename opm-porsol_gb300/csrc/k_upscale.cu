// k_upscale.cu -- PersistentUpscale: the three periodic solves of every sub-grid of a batch in one
// persistent kernel launch.
//
// Work items are sub-grids, taken from two device counters: first the tile items (a whole CTA per
// sub-grid, largest first), then the warp items (one warp per sub-grid).  The group that owns an
// item runs a Jacobi-preconditioned CG for the three unit pressure-jump right-hand sides together:
//   start   x = 0, r = b, p = D^-1 r, rho = r.D^-1 r
//   pass A  q = A p for the three directions from one read of the sub-grid's matrix rows; p.q
//   pass B  x += alpha p, r -= alpha q; r.D^-1 r and r.r; stopping test per direction
//   pass C  p = D^-1 r + beta p
// with group-local reductions only (warp shuffles, plus shared memory across the warps of a CTA),
// so no sub-grid ever waits for another.  A direction stops when ||r|| < tol ||r0|| or
// ||r|| < 1e-30 (the per-block test of the batched AMG solve); it is frozen from then on.
// Vectors hold the three directions of an unknown side by side (3 i + d), so the gathers of p in
// pass A touch one 24-byte run per column.  Every sum runs in a fixed order for a given schedule:
// results are run-to-run reproducible; another CTA size changes the summation order.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>
#include <numeric>
#include <unordered_map>

#include "upscale.h"

namespace porsol {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int UP_MAX_THREADS = 1024;
constexpr int UP_MAX_WARPS = UP_MAX_THREADS / 32;
constexpr int TUNE_ITERS = 8;   // CG iterations per sub-grid of one autotuner trial

struct UpArgs {
    int nitems, ntile, maxit;
    double tol;
    const int* order;    // sub-grid ids: tile items [0, ntile), then warp items
    const int* ranges;   // 4 per sub-grid
    const int* sp;       // SELL-32 union matrix
    const int* col;
    const double* val;
    const int* diag;
    const double* b3;
    double* x3;
    double* r3;
    double* p3;
    double* q3;
    double* dinv;
    int* iters;          // 3 per sub-grid: iteration at which the direction met its test, -1: never
    double* red;         // 3 per sub-grid: final ||r|| / ||r0||
    int* counters;       // [0]: next tile item, [1]: next warp item
    int* status;
};

// The unknowns of one sub-grid: local index k < n1 is row r0 + k, otherwise row r2 + (k - n1).
struct Rows {
    int r0, n1, r2, n;
    __device__ __forceinline__ int row(int k) const { return k < n1 ? r0 + k : r2 + (k - n1); }
};

// Sum of NV values over the group.  The warp butterfly leaves the bitwise-same total in every
// lane (each step adds two equal pairs in swapped order); a CTA then adds the per-warp totals in
// warp order, every thread reading them from shared memory, so all threads hold the same sums.
// Consecutive reductions must alternate between two buffers: a thread that has left one
// reduction's barrier may write the next one while others still read this one.
template <bool CTA, int NV>
__device__ __forceinline__ void group_sum(double (&v)[NV], double* sbuf)
{
#pragma unroll
    for (int i = 0; i < NV; ++i)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_xor_sync(FULL, v[i], o);
    if constexpr (CTA) {
        const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
        if ((threadIdx.x & 31) == 0)
#pragma unroll
            for (int i = 0; i < NV; ++i) sbuf[w * NV + i] = v[i];
        __syncthreads();
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double s = 0.0;
            for (int j = 0; j < nw; ++j) s += sbuf[j * NV + i];
            v[i] = s;
        }
    } else {
        __syncwarp();
    }
}

template <bool CTA>
__device__ __forceinline__ void group_sync()
{
    if constexpr (CTA) __syncthreads();
    else __syncwarp();
}

// q = (A p)_r for the three directions: the row's SELL-32 entries read once, four entries' loads
// in flight before their gathers; products added in entry order (padding adds exact zeros).
__device__ __forceinline__ void row_apply3(const int* __restrict__ sp, const int* __restrict__ col,
                                           const double* __restrict__ val, const double* __restrict__ p3, int r,
                                           double& q0, double& q1, double& q2)
{
    const int s = r >> 5;
    const int b = sp[s], w = (sp[s + 1] - b) >> 5;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    int k = b + (r & 31), t = 0;
    for (; t + 2 <= w; t += 2, k += 64) {
        const int c0 = col[k], c1 = col[k + 32];
        const double v0 = val[k], v1 = val[k + 32];
        const double* y0 = p3 + 3 * size_t(c0);
        const double* y1 = p3 + 3 * size_t(c1);
        const double y00 = y0[0], y01 = y0[1], y02 = y0[2];
        const double y10 = y1[0], y11 = y1[1], y12 = y1[2];
        a0 += v0 * y00;
        a1 += v0 * y01;
        a2 += v0 * y02;
        a0 += v1 * y10;
        a1 += v1 * y11;
        a2 += v1 * y12;
    }
    if (t < w) {
        const int c0 = col[k];
        const double v0 = val[k];
        const double* y0 = p3 + 3 * size_t(c0);
        a0 += v0 * y0[0];
        a1 += v0 * y0[1];
        a2 += v0 * y0[2];
    }
    q0 = a0;
    q1 = a1;
    q2 = a2;
}

// The CG of one sub-grid, three directions at once, by a group of nthr threads (tid = rank).
template <bool CTA>
__device__ void solve_one(const UpArgs& a, int g, int tid, int nthr, double* sb0, double* sb1)
{
    const int* rg = a.ranges + 4 * g;
    const Rows R{rg[0], rg[1] - rg[0], rg[2], (rg[1] - rg[0]) + (rg[3] - rg[2])};
    bool bad = false;
    double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int k = tid; k < R.n; k += nthr) {
        const int r = R.row(k);
        const double di = a.val[a.diag[r]];
        bad |= !(di > 0.0);
        const double dv = 1.0 / di;
        a.dinv[r] = dv;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double b = a.b3[3 * size_t(r) + d];
            const double z = dv * b;
            a.x3[3 * size_t(r) + d] = 0.0;
            a.r3[3 * size_t(r) + d] = b;
            a.p3[3 * size_t(r) + d] = z;
            v[d] += b * z;
            v[3 + d] += b * b;
        }
    }
    if (bad) atomicOr(a.status, ST_NONFINITE);
    group_sum<CTA, 6>(v, sb0);
    double rz[3], nr0[3], red[3];
    bool act[3];
    int itc[3];
    bool brk = false;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        rz[d] = v[d];
        nr0[d] = sqrt(v[3 + d]);
        red[d] = 0.0;
        const bool fin = isfinite(nr0[d]) && isfinite(rz[d]);
        brk |= !fin;
        act[d] = fin && !(nr0[d] < 1e-30);
        itc[d] = fin ? (act[d] ? -1 : 0) : -1;
    }
    int it = 0;
    while ((act[0] || act[1] || act[2]) && it < a.maxit) {
        ++it;
        // pass A
        double w[3] = {0.0, 0.0, 0.0};
        for (int k = tid; k < R.n; k += nthr) {
            const int r = R.row(k);
            double q0, q1, q2;
            row_apply3(a.sp, a.col, a.val, a.p3, r, q0, q1, q2);
            double* q = a.q3 + 3 * size_t(r);
            const double* p = a.p3 + 3 * size_t(r);
            q[0] = q0;
            q[1] = q1;
            q[2] = q2;
            w[0] += p[0] * q0;
            w[1] += p[1] * q1;
            w[2] += p[2] * q2;
        }
        group_sum<CTA, 3>(w, sb1);
        double al[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            if (act[d] && !(w[d] > 0.0 && isfinite(w[d]))) {   // non-positive curvature: stop
                act[d] = false;
                brk = true;
            }
            al[d] = act[d] ? rz[d] / w[d] : 0.0;
        }
        // pass B
        double u[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        for (int k = tid; k < R.n; k += nthr) {
            const int r = R.row(k);
            const double dv = a.dinv[r];
#pragma unroll
            for (int d = 0; d < 3; ++d)
                if (act[d]) {
                    const size_t i = 3 * size_t(r) + d;
                    a.x3[i] += al[d] * a.p3[i];
                    const double rn = a.r3[i] - al[d] * a.q3[i];
                    a.r3[i] = rn;
                    u[d] += rn * (dv * rn);
                    u[3 + d] += rn * rn;
                }
        }
        group_sum<CTA, 6>(u, sb0);
        double be[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            be[d] = 0.0;
            if (!act[d]) continue;
            const double nr = sqrt(u[3 + d]);
            red[d] = nr0[d] > 0.0 ? nr / nr0[d] : 0.0;
            if (!isfinite(nr) || !isfinite(u[d])) {
                act[d] = false;
                brk = true;
            } else if (nr < a.tol * nr0[d] || nr < 1e-30) {
                act[d] = false;
                itc[d] = it;
            } else {
                be[d] = u[d] / rz[d];
                rz[d] = u[d];
            }
        }
        if (!(act[0] || act[1] || act[2])) break;
        // pass C
        for (int k = tid; k < R.n; k += nthr) {
            const int r = R.row(k);
            const double dv = a.dinv[r];
#pragma unroll
            for (int d = 0; d < 3; ++d)
                if (act[d]) {
                    const size_t i = 3 * size_t(r) + d;
                    a.p3[i] = dv * a.r3[i] + be[d] * a.p3[i];
                }
        }
        group_sync<CTA>();
    }
    if (tid == 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            a.iters[3 * g + d] = itc[d];
            a.red[3 * g + d] = red[d];
        }
        if (brk) atomicOr(a.status, ST_BREAKDOWN);
    }
}

// The persistent kernel: tile items while any is left (the CTA takes the next one), then warp
// items (each warp on its own).  Every loop ends: the counters only grow, and each CG is bounded
// by maxit.
__global__ void __launch_bounds__(UP_MAX_THREADS, 1) k_upscale_persistent(const UpArgs a)
{
    __shared__ double sb[2][UP_MAX_WARPS * 6];
    __shared__ int s_item;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(a.counters, 1);
        __syncthreads();
        const int item = s_item;
        __syncthreads();   // every thread has read s_item before thread 0 writes it again
        if (item >= a.ntile) break;
        solve_one<true>(a, a.order[item], threadIdx.x, blockDim.x, sb[0], sb[1]);
    }
    const int lane = threadIdx.x & 31;
    const int nwarp = a.nitems - a.ntile;
    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(a.counters + 1, 1);
        item = __shfl_sync(FULL, item, 0);
        if (item >= nwarp) break;
        solve_one<false>(a, a.order[a.ntile + item], lane, 32, nullptr, nullptr);
    }
}

__global__ void k_put3(int n, const double* __restrict__ v, double* __restrict__ v3, int d)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v3[3 * size_t(i) + d] = v[i];
}

__global__ void k_get3(int n, const double* __restrict__ v3, double* __restrict__ v, int d)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = v3[3 * size_t(i) + d];
}

// Autotuner choices, per batch shape (sub-grid count, log2 of the unknowns, log2 of the largest
// sub-grid's unknowns), for the life of the process.
std::mutex& tune_mutex()
{
    static std::mutex m;
    return m;
}
std::unordered_map<long long, UpscaleSchedule>& tune_cache()
{
    static std::unordered_map<long long, UpscaleSchedule> c;
    return c;
}

int ilog2(long long v)
{
    int l = 0;
    while ((2LL << l) <= v) ++l;
    return l;
}

}  // namespace

void launch_put3(cudaStream_t s, int n, const double* v, double* v3, int d)
{
    if (n <= 0) return;
    PORSOL_LAUNCH(k_put3<<<div_up(n, 256), 256, 0, s>>>(n, v, v3, d));
    PORSOL_CUDA(cudaGetLastError());
}

void launch_get3(cudaStream_t s, int n, const double* v3, double* v, int d)
{
    if (n <= 0) return;
    PORSOL_LAUNCH(k_get3<<<div_up(n, 256), 256, 0, s>>>(n, v3, v, d));
    PORSOL_CUDA(cudaGetLastError());
}

PersistentUpscale::~PersistentUpscale()
{
    if (exec_) cudaGraphExecDestroy(exec_);
}

int PersistentUpscale::tile_items(const std::vector<int>& rg, int wmax) const
{
    int nt = 0;
    for (int g : order_h_) {
        const int n = (rg[4 * size_t(g) + 1] - rg[4 * size_t(g)]) + (rg[4 * size_t(g) + 3] - rg[4 * size_t(g) + 2]);
        if (n >= wmax) ++nt;
    }
    return nt;
}

void PersistentUpscale::launch(cudaStream_t s, const SellPattern& P, const double* val, const int* ranges_d,
                               const double* b3, double* x3, double tol, int maxit, const UpscaleSchedule& sc,
                               int ntile, bool graph)
{
    UpArgs a;
    std::memset(&a, 0, sizeof(a));
    a.nitems = nblk_;
    a.ntile = ntile;
    a.maxit = maxit;
    a.tol = tol;
    a.order = order_.p;
    a.ranges = ranges_d;
    a.sp = P.slice_ptr.p;
    a.col = P.col.p;
    a.val = val;
    a.diag = P.diag.p;
    a.b3 = b3;
    a.x3 = x3;
    a.r3 = r3_.p;
    a.p3 = p3_.p;
    a.q3 = q3_.p;
    a.dinv = dinv_.p;
    a.iters = iters_.p;
    a.red = red_.p;
    a.counters = counters_.p;
    a.status = status_.p;
    int dev = 0, sms = 0, per = 0;
    PORSOL_CUDA(cudaGetDevice(&dev));
    PORSOL_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PORSOL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_upscale_persistent, sc.cta_threads, 0));
    const int grid = std::max(1, sms * std::max(per, 1));
    auto enqueue = [&] {
        PORSOL_CUDA(cudaMemsetAsync(counters_.p, 0, 2 * sizeof(int), s));
        PORSOL_LAUNCH(k_upscale_persistent<<<grid, sc.cta_threads, 0, s>>>(a));
        PORSOL_CUDA(cudaGetLastError());
    };
    if (!graph) {
        enqueue();
        return;
    }
    // the launch (with the queue reset) as a captured graph, rebuilt when an argument changes
    std::vector<unsigned char> key(sizeof(a) + 2 * sizeof(int));
    std::memcpy(key.data(), &a, sizeof(a));
    std::memcpy(key.data() + sizeof(a), &grid, sizeof(int));
    std::memcpy(key.data() + sizeof(a) + sizeof(int), &sc.cta_threads, sizeof(int));
    if (!exec_ || key != exec_key_) {
        if (exec_) PORSOL_CUDA(cudaGraphExecDestroy(exec_));
        exec_ = nullptr;
        cudaGraph_t gr;
        const long long l0 = g_launches.load();
        PORSOL_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        enqueue();
        PORSOL_CUDA(cudaStreamEndCapture(s, &gr));
        g_launches.fetch_sub(g_launches.load() - l0);
        PORSOL_CUDA(cudaGraphInstantiate(&exec_, gr, 0));
        PORSOL_CUDA(cudaGraphDestroy(gr));
        exec_key_ = key;
    }
    PORSOL_CUDA(cudaGraphLaunch(exec_, s));
    PORSOL_COUNT_LAUNCH();
}

// Candidate schedules: CTAs of 256, 512 or 1024 threads for the tile items, and sub-grids below
// 0, 4096 or 16384 unknowns (sides up to about 11 and 17 in the unit-cube batches) left to single
// warps.  Each candidate runs TUNE_ITERS iterations of every sub-grid once, after one warm-up
// launch; the fastest is kept for the batch shape.
UpscaleSchedule PersistentUpscale::tune(cudaStream_t s, const SellPattern& P, const double* val,
                                        const std::vector<int>& rg, const int* ranges_d, const double* b3, double* x3)
{
    long long total = 0, largest = 0;
    for (int g = 0; g < nblk_; ++g) {
        const long long n = (rg[4 * size_t(g) + 1] - rg[4 * size_t(g)]) + (rg[4 * size_t(g) + 3] - rg[4 * size_t(g) + 2]);
        total += n;
        largest = std::max(largest, n);
    }
    const long long key = ((long long)nblk_ << 16) | ((long long)ilog2(std::max(total, 1LL)) << 8) |
                          (long long)ilog2(std::max(largest, 1LL));
    {
        std::lock_guard<std::mutex> lk(tune_mutex());
        auto it = tune_cache().find(key);
        if (it != tune_cache().end()) return it->second;
    }
    cudaEvent_t e0, e1;
    PORSOL_CUDA(cudaEventCreate(&e0));
    PORSOL_CUDA(cudaEventCreate(&e1));
    UpscaleSchedule best;
    float best_ms = 1e30f;
    bool warmed = false;
    try {
        for (int threads : {256, 512, 1024})
            for (int wmax : {0, 4096, 16384}) {
                UpscaleSchedule c;
                c.cta_threads = threads;
                c.warp_max_unknowns = wmax;
                c.tuned = true;
                const int nt = tile_items(rg, wmax);
                if (!warmed) {
                    launch(s, P, val, ranges_d, b3, x3, 0.0, TUNE_ITERS, c, nt, false);
                    warmed = true;
                }
                PORSOL_CUDA(cudaEventRecord(e0, s));
                launch(s, P, val, ranges_d, b3, x3, 0.0, TUNE_ITERS, c, nt, false);
                PORSOL_CUDA(cudaEventRecord(e1, s));
                PORSOL_CUDA(cudaEventSynchronize(e1));
                float ms = 0.f;
                PORSOL_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                if (ms < best_ms) {
                    best_ms = ms;
                    best = c;
                }
            }
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::lock_guard<std::mutex> lk(tune_mutex());
    tune_cache()[key] = best;
    return best;
}

UpscaleResult PersistentUpscale::solve(cudaStream_t s, const SellPattern& P, const double* val,
                                       const std::vector<int>& rg, const int* ranges_d, const double* b3, double* x3,
                                       double tol, int maxit, const UpscaleSchedule& fixed)
{
    PORSOL_REQUIRE(rg.size() % 4 == 0 && !rg.empty(), PORSOL_ERR_BAD_ARG, "persistent upscaling: no sub-grids");
    PORSOL_REQUIRE(P.n <= INT_MAX / 3, PORSOL_ERR_BAD_ARG, "persistent upscaling: too many unknowns");
    PORSOL_REQUIRE(fixed.cta_threads == 0 || fixed.cta_threads == 256 || fixed.cta_threads == 512 ||
                       fixed.cta_threads == 1024,
                   PORSOL_ERR_BAD_ARG, "persistent upscaling: CTA threads must be 256, 512 or 1024");
    n_ = P.n;
    nblk_ = int(rg.size() / 4);
    r3_.alloc(3 * size_t(n_));
    p3_.alloc(3 * size_t(n_));
    q3_.alloc(3 * size_t(n_));
    dinv_.alloc(size_t(n_));
    red_.alloc(3 * size_t(nblk_));
    iters_.alloc(3 * size_t(nblk_));
    counters_.alloc(2);
    status_.alloc(1);
    // largest sub-grids first (ties by index): the tile items, then the warp items, each in
    // decreasing size, so the longest solves start first
    std::vector<int> nrow(static_cast<size_t>(nblk_));
    for (int g = 0; g < nblk_; ++g)
        nrow[size_t(g)] = (rg[4 * size_t(g) + 1] - rg[4 * size_t(g)]) + (rg[4 * size_t(g) + 3] - rg[4 * size_t(g) + 2]);
    order_h_.resize(size_t(nblk_));
    std::iota(order_h_.begin(), order_h_.end(), 0);
    std::stable_sort(order_h_.begin(), order_h_.end(),
                     [&](int x, int y) { return nrow[size_t(x)] > nrow[size_t(y)]; });
    order_.upload(order_h_, s);
    status_.zero(s);
    sched_ = fixed.cta_threads ? fixed : tune(s, P, val, rg, ranges_d, b3, x3);
    if (fixed.cta_threads) sched_.tuned = false;
    const int nt = tile_items(rg, sched_.warp_max_unknowns);
    status_.zero(s);
    launch(s, P, val, ranges_d, b3, x3, tol, maxit, sched_, nt, true);
    std::vector<int> its(3 * size_t(nblk_));
    std::vector<double> red(3 * size_t(nblk_));
    int st = 0;
    iters_.download(its.data(), its.size(), s);
    red_.download(red.data(), red.size(), s);
    PORSOL_CUDA(cudaMemcpyAsync(&st, status_.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    PORSOL_CUDA(cudaStreamSynchronize(s));
    UpscaleResult res;
    res.converged = true;
    res.breakdown = (st & (ST_BREAKDOWN | ST_NONFINITE)) != 0;
    const double avg_entries = n_ > 0 ? double(P.nent) / n_ : 0.0;
    bytes_ = 0.0;
    for (int g = 0; g < nblk_; ++g) {
        int gi = 0;
        for (int d = 0; d < 3; ++d) {
            const int k = its[3 * size_t(g) + d];
            res.reduction = std::max(res.reduction, red[3 * size_t(g) + d]);
            if (k < 0) {
                res.converged = false;
                if (res.worst_block < 0) res.worst_block = g;
                gi = maxit;
            } else {
                gi = std::max(gi, k);
            }
        }
        res.iterations = std::max(res.iterations, gi);
        // start: diagonal, b, x, r, p (3 each); per iteration: stored entries (column 4 + value 8),
        // p gathered once and q written (24 + 24), pass B (D^-1, x, r twice, p, q) and pass C
        // (D^-1, r, p twice), three directions each
        const double n = nrow[size_t(g)];
        bytes_ += n * (12.0 + 8.0 + 4 * 24.0) + gi * n * (12.0 * avg_entries + 48.0 + 8.0 + 6 * 24.0 + 8.0 + 3 * 24.0);
    }
    return res;
}

}  // namespace porsol
