// k_upscale.cu -- PersistentUpscale: the three periodic solves of every sub-grid of a batch in one
// persistent kernel launch.
//
// Work items are sub-grids, taken from device counters, largest first: cluster items (a cluster of
// 2 or 4 CTAs per sub-grid, on as many SMs), then CTA items (a whole CTA per sub-grid), then warp
// items (one warp per sub-grid).  The group that owns an
// item runs a Jacobi-preconditioned CG for the three unit pressure-jump right-hand sides together,
// with FP32 recurrences (matrix copy, vectors and products in FP32: one matrix read feeds three
// products) and reliable updates in FP64 (solution, true residual, convergence test), with
// group-local reductions only (warp shuffles, plus shared memory across the warps of a CTA and
// distributed shared memory across the CTAs of a cluster), so no sub-grid ever waits for another.  A direction stops when its true residual meets
// ||b - A x|| < tol ||b|| or ||b - A x|| < 1e-30 (the per-block test of the batched AMG solve); it
// is frozen from then on.  FP32 matters on this GPU: one SM runs the largest sub-grid alone, and
// with FP64 products its FP64 pipe, not memory, set the time (ncu: 95 % busy).  Every sum runs in a
// fixed order for a given schedule: results are run-to-run reproducible; another CTA size changes
// the summation order.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <numeric>
#include <unordered_map>

#include <cooperative_groups.h>

#include "upscale.h"

namespace porsol {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int UP_MAX_THREADS = 1024;
constexpr int UP_MAX_WARPS = UP_MAX_THREADS / 32;
constexpr int TUNE_ITERS = 8;   // CG iterations per sub-grid of one autotuner trial
namespace cg = cooperative_groups;

// The group of threads that solves one sub-grid: a warp, a CTA, or a cluster of CTAs.
constexpr int G_WARP = 0, G_CTA = 1, G_CLUSTER = 2;
// One reduction buffer: the per-warp partials (up to 32 warps x 6 values), then the CTA's totals
// (6 values, read by the other CTAs of a cluster).  Two buffers alternate.
constexpr int SB_STRIDE = UP_MAX_WARPS * 6 + 6;

struct UpArgs {
    int nitems, ncl, ntile, maxit, n;   // items [0, ncl): clusters; then ntile CTA items; then warp items
    double tol, delta;
    const int* order;     // sub-grid ids: tile items [0, ntile), then warp items
    const int* ranges;    // 4 per sub-grid
    const int* sp;        // SELL-32 union matrix: FP64 values and their FP32 copy
    const int* col;
    const double* val;
    const float* val32;
    const int* diag;
    const double* b3;     // right-hand sides, side by side
    double* x3;           // solutions (FP64)
    double* r64;          // true residuals at replacements (FP64)
    float* r32;           // CG vectors (FP32, in units of the direction's sigma)
    float* p32;
    float* q32;
    float* dinv;          // 1 / a_ii
    int* iters;           // 3 per sub-grid: iteration at which the direction met its test, -1: never
    double* red;          // 3 per sub-grid: last true ||r|| / ||r0||
    int* counters;        // [0]: next cluster item, [1]: next CTA item, [2]: next warp item
    int* status;
};

// The unknowns of one sub-grid: local index k < n1 is row r0 + k, otherwise row r2 + (k - n1).
struct Rows {
    int r0, n1, r2, n;
    __device__ __forceinline__ int row(int k) const { return k < n1 ? r0 + k : r2 + (k - n1); }
};

// Sums over the group.  The warp butterfly leaves the bitwise-same total in every lane (each step
// adds two equal pairs in swapped order); a CTA then adds the per-warp totals in warp order in FP64,
// every thread reading them from shared memory; in a cluster every CTA forms its total that way, and
// after the cluster barrier each thread adds the CTAs' totals in CTA order, reading them from the
// other CTAs' shared memory (one remote load per CTA and value, not one per warp); so all threads
// of the group hold the same sums.  Two buffers alternate from one reduction to the
// next (rb): a thread that has left one reduction's barrier may write the next one while others
// still read this one.  FP32 partials (the CG's dot products) are summed in FP32 within a warp and in
// FP64 across warps.
template <int G, int NV, class T>
__device__ __forceinline__ void group_sum(const T (&v)[NV], double (&out)[NV], double* sb, int& rb)
{
    T w[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        w[i] = v[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) w[i] += __shfl_xor_sync(FULL, w[i], o);
    }
    if constexpr (G == G_CTA) {
        double* buf = sb + rb * SB_STRIDE;
        rb ^= 1;
        const int wi = threadIdx.x >> 5, nw = blockDim.x >> 5;
        if ((threadIdx.x & 31) == 0)
#pragma unroll
            for (int i = 0; i < NV; ++i) buf[wi * NV + i] = double(w[i]);
        __syncthreads();
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double s = 0.0;
            for (int j = 0; j < nw; ++j) s += buf[j * NV + i];
            out[i] = s;
        }
    } else if constexpr (G == G_CLUSTER) {
        cg::cluster_group cl = cg::this_cluster();
        double* buf = sb + rb * SB_STRIDE;
        double* ctot = buf + UP_MAX_WARPS * 6;
        rb ^= 1;
        const int wi = threadIdx.x >> 5, nw = blockDim.x >> 5;
        if ((threadIdx.x & 31) == 0)
#pragma unroll
            for (int i = 0; i < NV; ++i) buf[wi * NV + i] = double(w[i]);
        __syncthreads();
        if (threadIdx.x == 0)
#pragma unroll
            for (int i = 0; i < NV; ++i) {
                double s = 0.0;
                for (int j = 0; j < nw; ++j) s += buf[j * NV + i];
                ctot[i] = s;
            }
        cl.sync();
        const int nc = int(cl.num_blocks());
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double s = 0.0;
            for (int c = 0; c < nc; ++c) s += cl.map_shared_rank(ctot, c)[i];
            out[i] = s;
        }
    } else {
#pragma unroll
        for (int i = 0; i < NV; ++i) out[i] = double(w[i]);
        __syncwarp();
    }
}

template <int G>
__device__ __forceinline__ void group_sync()
{
    if constexpr (G == G_CLUSTER) cg::this_cluster().sync();
    else if constexpr (G == G_CTA) __syncthreads();
    else __syncwarp();
}

// Position of direction d of unknown i in the three-direction vectors: side by side (L = 0,
// 3 i + d: one run per gathered column) or direction-major (L = 1, d n + i: every streamed access
// of a warp is one contiguous run).  The autotuner tries both; they measured within a few per cent
// of each other, either ahead.  A third layout, side by side padded to four values and accessed as
// 16-byte vectors (fewer memory instructions), measured no faster and was removed.
template <int L>
__device__ __forceinline__ size_t vix(int i, int d, int n)
{
    return L == 0 ? 3 * size_t(i) + d : size_t(d) * size_t(n) + i;
}

// The three values of unknown i, per direction: masked-off directions are neither loaded (read as
// 0) nor stored.  The vectors are written by this kernel (by other CTAs of a cluster, too), so
// their pointers carry no __restrict__: the loads stay ordinary coherent loads, ordered by the
// group's barriers, never the read-only path.
template <int L, class T>
__device__ __forceinline__ void ld3(const T* v, int i, int n, const bool (&m)[3], T (&o)[3])
{
#pragma unroll
    for (int d = 0; d < 3; ++d) o[d] = m[d] ? v[vix<L>(i, d, n)] : T(0);
}
template <int L, class T>
__device__ __forceinline__ void st3(T* v, int i, int n, const bool (&m)[3], const T (&x)[3])
{
#pragma unroll
    for (int d = 0; d < 3; ++d)
        if (m[d]) v[vix<L>(i, d, n)] = x[d];
}

// q = (A y)_r for the three directions (values TV, vector TX, sums TA): the row's SELL-32
// entries read once, two entries' loads in flight before their gathers; products added in entry
// order (padding adds exact zeros).
template <int L, class TA, class TV, class TX>
__device__ __forceinline__ void row_apply3(const int* __restrict__ sp, const int* __restrict__ col,
                                           const TV* __restrict__ val, const TX* y, int n, int r,
                                           TA (&q)[3])
{
    constexpr bool all[3] = {true, true, true};
    const int s = r >> 5;
    const int b = sp[s], w = (sp[s + 1] - b) >> 5;
    TA a0 = TA(0), a1 = TA(0), a2 = TA(0);
    int k = b + (r & 31), t = 0;
    for (; t + 2 <= w; t += 2, k += 64) {
        const int c0 = col[k], c1 = col[k + 32];
        const TA v0 = TA(val[k]), v1 = TA(val[k + 32]);
        TX y0[3], y1[3];
        ld3<L>(y, c0, n, all, y0);
        ld3<L>(y, c1, n, all, y1);
        a0 += v0 * TA(y0[0]);
        a1 += v0 * TA(y0[1]);
        a2 += v0 * TA(y0[2]);
        a0 += v1 * TA(y1[0]);
        a1 += v1 * TA(y1[1]);
        a2 += v1 * TA(y1[2]);
    }
    if (t < w) {
        const int c0 = col[k];
        const TA v0 = TA(val[k]);
        TX y0[3];
        ld3<L>(y, c0, n, all, y0);
        a0 += v0 * TA(y0[0]);
        a1 += v0 * TA(y0[1]);
        a2 += v0 * TA(y0[2]);
    }
    q[0] = a0;
    q[1] = a1;
    q[2] = a2;
}

// The CG of one sub-grid, three directions at once, by a group of nthr threads (tid = rank), with
// FP32 recurrences and reliable updates (residual replacement, Sleijpen and van der Vorst):
//   start   x = 0, sigma = ||b||, r = b / sigma (FP32), p = D^-1 r, rho = r.D^-1 r
//   pass A  q = A32 p (FP32), p.q
//   pass B  x += sigma alpha p (FP64), r -= alpha q; r.D^-1 r, r.r
//   when ||r|| has dropped below delta since the last replacement, or sigma ||r|| reaches the
//   tolerance: pass R, the true residual b - A x in FP64, which alone decides convergence; then
//   pass S, r = (b - A x) / sigma' and p *= sigma / sigma' (the recurrence continues in units of
//   the new sigma), r.D^-1 r again
//   pass C  p = D^-1 r + beta p
// x stays FP64 every iteration: an FP32 increment of x flushed at each replacement (measured) let
// one sub-grid of the 512-sub-grid batch stall at 3.3e-11 against a 1e-11 tolerance, its rounding
// times the condition number bounding the residual each replacement can reach.
// Each pass loads all of a row's values before it stores any, and frozen directions keep their
// values.  Thread 0 keeps the per-direction iteration count and reduction in global memory.
template <int G, int L>
__device__ void solve_one(const UpArgs& a, int g, int tid, int nthr, double* sb)
{
    constexpr bool all[3] = {true, true, true};
    const int* rg = a.ranges + 4 * g;
    const Rows R{rg[0], rg[1] - rg[0], rg[2], (rg[1] - rg[0]) + (rg[3] - rg[2])};
    const int n = a.n;
    int rb = 0;
    bool bad = false;
    double v[3] = {0.0, 0.0, 0.0}, sum[3];
    for (int k = tid; k < R.n; k += nthr) {
        const int r = R.row(k);
        double b[3];
        ld3<0>(a.b3, r, n, all, b);   // right-hand sides: side by side
        const double di = a.val[a.diag[r]];
        bad |= !(di > 0.0);
        a.dinv[r] = float(1.0 / di);
        const double z3[3] = {0.0, 0.0, 0.0};
        st3<L>(a.x3, r, n, all, z3);
#pragma unroll
        for (int d = 0; d < 3; ++d) v[d] += b[d] * b[d];
    }
    if (bad) atomicOr(a.status, ST_NONFINITE);
    group_sum<G, 3>(v, sum, sb, rb);
    double sig[3], def0[3], rho[3];
    bool act[3];
    bool brk = false;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        def0[d] = sig[d] = sqrt(sum[d]);
        const bool fin = isfinite(def0[d]);
        brk |= !fin;
        act[d] = fin && !(def0[d] < 1e-30);
        if (tid == 0) {
            a.iters[3 * g + d] = fin ? (act[d] ? -1 : 0) : -1;
            a.red[3 * g + d] = act[d] ? 1.0 : 0.0;
        }
    }
    {
        float u[3] = {0.f, 0.f, 0.f};
        for (int k = tid; k < R.n; k += nthr) {
            const int r = R.row(k);
            double b[3];
            ld3<0>(a.b3, r, n, all, b);
            const float dv = a.dinv[r];
            float rr[3], pp[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                rr[d] = act[d] ? float(b[d] / sig[d]) : 0.f;
                pp[d] = dv * rr[d];
                u[d] += rr[d] * pp[d];
            }
            st3<L>(a.r32, r, n, all, rr);
            st3<L>(a.p32, r, n, all, pp);
        }
        group_sum<G, 3>(u, rho, sb, rb);
    }
    int it = 0;
    while ((act[0] || act[1] || act[2]) && it < a.maxit) {
        ++it;
        // pass A: q = A32 p, p.q
        {
            float w[3] = {0.f, 0.f, 0.f};
            for (int k = tid; k < R.n; k += nthr) {
                const int r = R.row(k);
                float p[3], q[3];
                ld3<L>(a.p32, r, n, all, p);
                row_apply3<L, float>(a.sp, a.col, a.val32, a.p32, n, r, q);
                st3<L>(a.q32, r, n, all, q);
#pragma unroll
                for (int d = 0; d < 3; ++d) w[d] += p[d] * q[d];
            }
            group_sum<G, 3>(w, sum, sb, rb);
        }
        double al[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            if (act[d] && !(sum[d] > 0.0 && isfinite(sum[d]))) {   // non-positive curvature: stop
                act[d] = false;
                brk = true;
            }
            al[d] = act[d] ? rho[d] / sum[d] : 0.0;
        }
        // pass B: x += sigma alpha p, r -= alpha q; r.D^-1 r, r.r
        double u[3], rr2[3];
        {
            float part[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            for (int k = tid; k < R.n; k += nthr) {
                const int r = R.row(k);
                const float dv = a.dinv[r];
                double x[3];
                float p[3], rr[3], q[3];
                ld3<L>(a.x3, r, n, act, x);
                ld3<L>(a.p32, r, n, act, p);
                ld3<L>(a.r32, r, n, act, rr);
                ld3<L>(a.q32, r, n, act, q);
#pragma unroll
                for (int d = 0; d < 3; ++d)
                    if (act[d]) {
                        const float rn = rr[d] - float(al[d]) * q[d];
                        x[d] += (sig[d] * al[d]) * double(p[d]);
                        rr[d] = rn;
                        part[d] += rn * (dv * rn);
                        part[3 + d] += rn * rn;
                    }
                st3<L>(a.x3, r, n, act, x);
                st3<L>(a.r32, r, n, act, rr);
            }
            double tot[6];
            group_sum<G, 6>(part, tot, sb, rb);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                u[d] = tot[d];
                rr2[d] = tot[3 + d];
            }
        }
        // reliable update: which directions replace their residual
        bool rep[3], any = false;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double defs = sqrt(rr2[d]), est = defs * sig[d];
            rep[d] = act[d] && (defs < a.delta || est < a.tol * def0[d] || est < 1e-30 || !isfinite(defs) ||
                                it >= a.maxit);
            any |= rep[d];
        }
        if (any) {
            // pass R: the true residual b - A x (FP64) of the replacing directions
            double t2[3] = {0.0, 0.0, 0.0};
            for (int k = tid; k < R.n; k += nthr) {
                const int r = R.row(k);
                double ax[3], b[3], t[3];
                row_apply3<L, double>(a.sp, a.col, a.val, a.x3, n, r, ax);
                ld3<0>(a.b3, r, n, all, b);
                ld3<L>(a.r64, r, n, rep, t);
#pragma unroll
                for (int d = 0; d < 3; ++d)
                    if (rep[d]) {
                        t[d] = b[d] - ax[d];
                        t2[d] += t[d] * t[d];
                    }
                st3<L>(a.r64, r, n, rep, t);
            }
            group_sum<G, 3>(t2, sum, sb, rb);
            bool resc[3], anyr = false;
            double fac[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                resc[d] = false;
                fac[d] = 1.0;
                if (!rep[d]) continue;
                const double dd = sqrt(sum[d]);
                if (tid == 0) a.red[3 * g + d] = dd / def0[d];
                if (!isfinite(dd)) {
                    act[d] = false;
                    brk = true;
                } else if (dd < a.tol * def0[d] || dd < 1e-30) {
                    act[d] = false;
                    if (tid == 0) a.iters[3 * g + d] = it;
                } else if (it >= a.maxit) {
                    act[d] = false;
                } else {
                    fac[d] = sig[d] / dd;
                    rho[d] *= fac[d] * fac[d];
                    sig[d] = dd;
                    resc[d] = true;
                    anyr = true;
                }
            }
            if (anyr) {
                // pass S: r = r_true / sigma, p in units of the new sigma; r.D^-1 r of the new r
                float uu[3] = {0.f, 0.f, 0.f};
                for (int k = tid; k < R.n; k += nthr) {
                    const int r = R.row(k);
                    const float dv = a.dinv[r];
                    double t[3];
                    float p[3], rr[3];
                    ld3<L>(a.r64, r, n, resc, t);
                    ld3<L>(a.p32, r, n, resc, p);
                    ld3<L>(a.r32, r, n, resc, rr);
#pragma unroll
                    for (int d = 0; d < 3; ++d)
                        if (resc[d]) {
                            rr[d] = float(t[d] / sig[d]);
                            p[d] *= float(fac[d]);
                            uu[d] += rr[d] * (dv * rr[d]);
                        }
                    st3<L>(a.r32, r, n, resc, rr);
                    st3<L>(a.p32, r, n, resc, p);
                }
                double un[3];
                group_sum<G, 3>(uu, un, sb, rb);
#pragma unroll
                for (int d = 0; d < 3; ++d)
                    if (resc[d]) u[d] = un[d];
            }
        }
        double be[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            be[d] = 0.0;
            if (!act[d]) continue;
            if (!isfinite(u[d])) {
                act[d] = false;
                brk = true;
                continue;
            }
            be[d] = u[d] / rho[d];
            rho[d] = u[d];
        }
        if (!(act[0] || act[1] || act[2])) break;
        // pass C: p = D^-1 r + beta p
        for (int k = tid; k < R.n; k += nthr) {
            const int r = R.row(k);
            const float dv = a.dinv[r];
            float p[3], rr[3];
            ld3<L>(a.p32, r, n, act, p);
            ld3<L>(a.r32, r, n, act, rr);
#pragma unroll
            for (int d = 0; d < 3; ++d)
                if (act[d]) p[d] = dv * rr[d] + float(be[d]) * p[d];
            st3<L>(a.p32, r, n, act, p);
        }
        group_sync<G>();
    }
    if (tid == 0 && brk) atomicOr(a.status, ST_BREAKDOWN);
}

// The persistent kernel: cluster items while any is left (rank 0 of the cluster takes the next
// one and the other CTAs read it from rank 0's shared memory), then CTA items (each CTA takes the
// next one), then warp items (each warp on its own).  Every loop ends: the counters only grow, and
// each CG is bounded by maxit.  Every cluster barrier is reached by all CTAs of the cluster: the
// item and every sum that steers the CG are the same in all of them.  After its last cluster
// item a CTA passes two more cluster barriers, so no CTA reads another's shared memory once any has
// moved on (or exited).
template <int L, bool CLUSTER>
__global__ void __launch_bounds__(UP_MAX_THREADS, 1) k_upscale_persistent(const UpArgs a)
{
    __shared__ double sb[2 * SB_STRIDE];
    __shared__ int s_item;
    if constexpr (CLUSTER) {
        cg::cluster_group cl = cg::this_cluster();
        const int crank = int(cl.block_rank()), csize = int(cl.num_blocks());
        for (;;) {
            if (crank == 0 && threadIdx.x == 0) s_item = atomicAdd(a.counters, 1);
            cl.sync();
            const int item = *cl.map_shared_rank(&s_item, 0);
            cl.sync();   // every CTA has read rank 0's s_item before it is written again
            if (item >= a.ncl) break;
            solve_one<G_CLUSTER, L>(a, a.order[item], crank * int(blockDim.x) + int(threadIdx.x),
                                    csize * int(blockDim.x), sb);
        }
    }
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(a.counters + 1, 1);
        __syncthreads();
        const int item = s_item;
        __syncthreads();   // every thread has read s_item before thread 0 writes it again
        if (item >= a.ntile) break;
        solve_one<G_CTA, L>(a, a.order[a.ncl + item], threadIdx.x, blockDim.x, sb);
    }
    const int lane = threadIdx.x & 31;
    const int first = a.ncl + a.ntile, nwarp = a.nitems - first;
    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(a.counters + 2, 1);
        item = __shfl_sync(FULL, item, 0);
        if (item >= nwarp) break;
        solve_one<G_WARP, L>(a, a.order[first + item], lane, 32, nullptr);
    }
}

__global__ void k_put3(int n, const double* __restrict__ v, double* __restrict__ v3, int d)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v3[3 * size_t(i) + d] = v[i];
}

__global__ void k_get3(int n, const double* __restrict__ v3, double* __restrict__ v, int d, int layout)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = layout == 0 ? v3[3 * size_t(i) + d] : v3[size_t(d) * size_t(n) + i];
}

__global__ void k_fill(int n, double value, double* __restrict__ v)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = value;
}

__global__ void k_jump_values(int nhf, const int* __restrict__ side, int d, double* __restrict__ bcv)
{
    const int hf = blockIdx.x * blockDim.x + threadIdx.x;
    if (hf >= nhf) return;
    const int sd = side[hf];
    bcv[hf] = sd == 2 * d + 1 ? 1.0 : (sd == 2 * d + 2 ? -1.0 : 0.0);
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

void launch_get3(cudaStream_t s, int n, const double* v3, double* v, int d, int layout)
{
    if (n <= 0) return;
    PORSOL_LAUNCH(k_get3<<<div_up(n, 256), 256, 0, s>>>(n, v3, v, d, layout));
    PORSOL_CUDA(cudaGetLastError());
}

void launch_fill(cudaStream_t s, int n, double value, double* v)
{
    if (n <= 0) return;
    PORSOL_LAUNCH(k_fill<<<div_up(n, 256), 256, 0, s>>>(n, value, v));
    PORSOL_CUDA(cudaGetLastError());
}

void launch_jump_values(cudaStream_t s, int nhf, const int* side, int d, double* bcv)
{
    if (nhf <= 0) return;
    PORSOL_LAUNCH(k_jump_values<<<div_up(nhf, 256), 256, 0, s>>>(nhf, side, d, bcv));
    PORSOL_CUDA(cudaGetLastError());
}

PersistentUpscale::~PersistentUpscale()
{
    if (exec_) cudaGraphExecDestroy(exec_);
}

void PersistentUpscale::item_classes(const std::vector<int>& rg, const UpscaleSchedule& sc, int& ncl, int& ntile) const
{
    ncl = ntile = 0;
    for (int g : order_h_) {
        const int n = (rg[4 * size_t(g) + 1] - rg[4 * size_t(g)]) + (rg[4 * size_t(g) + 3] - rg[4 * size_t(g) + 2]);
        if (sc.cluster > 1 && n >= sc.cluster_min_unknowns) ++ncl;
        else if (n >= sc.warp_max_unknowns) ++ntile;
    }
}

void PersistentUpscale::launch(cudaStream_t s, const SellPattern& P, const double* val, const float* val32,
                               const int* ranges_d, const double* b3, double* x3, double tol, double delta, int maxit,
                               const UpscaleSchedule& sc, bool graph)
{
    UpArgs a;
    std::memset(&a, 0, sizeof(a));
    a.nitems = nblk_;
    item_classes(rg_h_, sc, a.ncl, a.ntile);
    a.n = n_;
    a.maxit = maxit;
    a.tol = tol;
    a.delta = delta;
    a.order = order_.p;
    a.ranges = ranges_d;
    a.sp = P.slice_ptr.p;
    a.col = P.col.p;
    a.val = val;
    a.val32 = val32;
    a.diag = P.diag.p;
    a.b3 = b3;
    a.x3 = x3;
    a.r64 = r64_.p;
    a.r32 = r32_.p;
    a.p32 = p32_.p;
    a.q32 = q32_.p;
    a.dinv = dinv_.p;
    a.iters = iters_.p;
    a.red = red_.p;
    a.counters = counters_.p;
    a.status = status_.p;
    const bool cl = sc.cluster > 1;
    void (*kern)(const UpArgs) = sc.layout == 0 ? (cl ? k_upscale_persistent<0, true> : k_upscale_persistent<0, false>)
                                                : (cl ? k_upscale_persistent<1, true> : k_upscale_persistent<1, false>);
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    cfg.blockDim = dim3(unsigned(sc.cta_threads));
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    int grid = 1;
    if (cl) {
        // as many clusters as can be resident at once (each CTA fills its SM)
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = unsigned(sc.cluster);
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        cfg.gridDim = dim3(unsigned(sc.cluster));
        int nclusters = 0;
        PORSOL_CUDA(cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg));
        PORSOL_REQUIRE(nclusters > 0, PORSOL_ERR_BAD_ARG, "persistent upscaling: cluster schedule cannot be resident");
        grid = nclusters * sc.cluster;
    } else {
        int dev = 0, sms = 0, per = 0;
        PORSOL_CUDA(cudaGetDevice(&dev));
        PORSOL_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        PORSOL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, sc.cta_threads, 0));
        grid = std::max(1, sms * std::max(per, 1));
        cfg.attrs = nullptr;
        cfg.numAttrs = 0;
    }
    cfg.gridDim = dim3(unsigned(grid));
    auto enqueue = [&] {
        PORSOL_CUDA(cudaMemsetAsync(counters_.p, 0, 3 * sizeof(int), s));
        PORSOL_CUDA(cudaLaunchKernelEx(&cfg, kern, a));
        PORSOL_COUNT_LAUNCH();
        PORSOL_CUDA(cudaGetLastError());
    };
    if (!graph) {
        enqueue();
        return;
    }
    // the launch (with the queue reset) as a captured graph, rebuilt when an argument changes
    std::vector<unsigned char> key(sizeof(a) + 4 * sizeof(int));
    std::memcpy(key.data(), &a, sizeof(a));
    std::memcpy(key.data() + sizeof(a), &grid, sizeof(int));
    std::memcpy(key.data() + sizeof(a) + sizeof(int), &sc.cta_threads, sizeof(int));
    std::memcpy(key.data() + sizeof(a) + 2 * sizeof(int), &sc.layout, sizeof(int));
    std::memcpy(key.data() + sizeof(a) + 3 * sizeof(int), &sc.cluster, sizeof(int));
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

// Candidate schedules: both vector layouts; CTAs of 512 or 1024 threads for the CTA items
// (256-thread CTAs and a 16384-unknown warp limit always measured slower on the 512-sub-grid
// batch); sub-grids below 0 or 4096 unknowns (sides up to about 11 in the unit-cube batches) left
// to single warps; and the sub-grids of at least half the largest one's unknowns solved by clusters
// of 1 (none), 2 or 4 CTAs.  Each candidate runs TUNE_ITERS iterations of every sub-grid once, after
// one warm-up launch; the fastest is kept for the batch shape.  A cluster shape that cannot be
// resident on this GPU is skipped.
UpscaleSchedule PersistentUpscale::tune(cudaStream_t s, const SellPattern& P, const double* val, const float* val32,
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
    static const bool debug = std::getenv("PORSOL_DEBUG_UPSCALE") != nullptr;
    cudaEvent_t e0, e1;
    PORSOL_CUDA(cudaEventCreate(&e0));
    PORSOL_CUDA(cudaEventCreate(&e1));
    UpscaleSchedule best;
    float best_ms = 1e30f;
    bool warmed = false;
    try {
        for (int cluster : {1, 2, 4})
            for (int layout : {0, 1})
                for (int threads : {512, 1024})
                    for (int wmax : {0, 4096}) {
                        UpscaleSchedule c;
                        c.cta_threads = threads;
                        c.warp_max_unknowns = wmax;
                        c.layout = layout;
                        c.cluster = cluster;
                        c.cluster_min_unknowns = cluster > 1 ? int(largest / 2) : 0;
                        c.tuned = true;
                        try {
                            if (!warmed) {
                                launch(s, P, val, val32, ranges_d, b3, x3, 0.0, 0.0, TUNE_ITERS, c, false);
                                warmed = true;
                            }
                            PORSOL_CUDA(cudaEventRecord(e0, s));
                            launch(s, P, val, val32, ranges_d, b3, x3, 0.0, 0.0, TUNE_ITERS, c, false);
                        } catch (const Error& e) {
                            if (e.code != PORSOL_ERR_BAD_ARG) throw;
                            continue;   // cluster shape not resident here
                        }
                        PORSOL_CUDA(cudaEventRecord(e1, s));
                        PORSOL_CUDA(cudaEventSynchronize(e1));
                        float ms = 0.f;
                        PORSOL_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                        if (debug)
                            std::fprintf(stderr, "[upscale] trial cluster=%d layout=%d cta=%d warp_below=%d: %.3f ms\n",
                                         cluster, layout, threads, wmax, ms);
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
    PORSOL_REQUIRE(best_ms < 1e30f, PORSOL_ERR_CUDA, "persistent upscaling: no schedule could be launched");
    std::lock_guard<std::mutex> lk(tune_mutex());
    tune_cache()[key] = best;
    return best;
}

UpscaleResult PersistentUpscale::solve(cudaStream_t s, const SellPattern& P, const double* val, const float* val32,
                                       const std::vector<int>& rg, const int* ranges_d, const double* b3, double* x3,
                                       double tol, double delta, int maxit, const UpscaleSchedule& fixed)
{
    PORSOL_REQUIRE(rg.size() % 4 == 0 && !rg.empty(), PORSOL_ERR_BAD_ARG, "persistent upscaling: no sub-grids");
    PORSOL_REQUIRE(P.n <= INT_MAX / 3, PORSOL_ERR_BAD_ARG, "persistent upscaling: too many unknowns");
    PORSOL_REQUIRE(fixed.layout == 0 || fixed.layout == 1, PORSOL_ERR_BAD_ARG,
                   "persistent upscaling: vector layout must be 0 or 1");
    PORSOL_REQUIRE(fixed.cluster == 1 || fixed.cluster == 2 || fixed.cluster == 4, PORSOL_ERR_BAD_ARG,
                   "persistent upscaling: cluster size must be 1, 2 or 4");
    PORSOL_REQUIRE(fixed.cta_threads == 0 || fixed.cta_threads == 256 || fixed.cta_threads == 512 ||
                       fixed.cta_threads == 1024,
                   PORSOL_ERR_BAD_ARG, "persistent upscaling: CTA threads must be 256, 512 or 1024");
    n_ = P.n;
    nblk_ = int(rg.size() / 4);
    r64_.alloc(3 * size_t(n_));
    r32_.alloc(3 * size_t(n_));
    p32_.alloc(3 * size_t(n_));
    q32_.alloc(3 * size_t(n_));
    dinv_.alloc(size_t(n_));
    red_.alloc(3 * size_t(nblk_));
    iters_.alloc(3 * size_t(nblk_));
    counters_.alloc(3);
    rg_h_ = rg;
    status_.alloc(1);
    // largest sub-grids first (ties by index): the cluster items, the CTA items, then the warp items,
    // each in decreasing size, so the longest solves start first
    std::vector<int> nrow(static_cast<size_t>(nblk_));
    for (int g = 0; g < nblk_; ++g)
        nrow[size_t(g)] = (rg[4 * size_t(g) + 1] - rg[4 * size_t(g)]) + (rg[4 * size_t(g) + 3] - rg[4 * size_t(g) + 2]);
    order_h_.resize(size_t(nblk_));
    std::iota(order_h_.begin(), order_h_.end(), 0);
    std::stable_sort(order_h_.begin(), order_h_.end(),
                     [&](int x, int y) { return nrow[size_t(x)] > nrow[size_t(y)]; });
    order_.upload(order_h_, s);
    status_.zero(s);
    sched_ = fixed.cta_threads ? fixed : tune(s, P, val, val32, rg, ranges_d, b3, x3);
    if (fixed.cta_threads) sched_.tuned = false;
    status_.zero(s);
    launch(s, P, val, val32, ranges_d, b3, x3, tol, delta, maxit, sched_, true);
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
        // start: diagonal and b twice, x, r, p; per iteration: stored entries (column 4 + FP32 value
        // 4), p gathered once, its own value read and q written (3 x 4 each), pass B (D^-1 4; x read
        // and written 16, p 4, r read and written 8, q 4 per direction) and pass C (D^-1 4; r 4, p
        // read and written 8 per direction); replacements are not counted
        const double n = nrow[size_t(g)];
        bytes_ += n * (12.0 + 48.0 + 3 * (8.0 + 4.0 + 4.0)) +
                  gi * n * (8.0 * avg_entries + 36.0 + 4.0 + 3 * 32.0 + 4.0 + 3 * 12.0);
    }
    return res;
}

}  // namespace porsol
