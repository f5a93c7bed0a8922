// k_amg.cu -- aggregation AMG: pairwise matching, Galerkin products, Chebyshev V-cycle,
// FP64 dense coarsest-level solve.  Every floating-point reduction has a fixed order (no
// floating-point atomics), so hierarchy and preconditioner are run-to-run reproducible.
#include <algorithm>
#include <cmath>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include <mutex>
#include <type_traits>
#include <unordered_map>

#include "amg.h"
#include "sell.cuh"

namespace porsol {

namespace {

constexpr int TB = 256;

__device__ __forceinline__ int slot_of(const int* sp, int r, int t) { return sp[r >> 5] + t * 32 + (r & 31); }

// Row r and lane q of the row for K lanes per row (K = 1: one thread per row; K = 0: one thread
// per row on the SELL-32x4 copy of the matrix).
// Batched solves skip the rows of converged blocks: act (one flag per 32-row slice of the level, null
// when every row works) is 0 where no block of the slice still iterates.  The slice is taken from
// the row clamped to the level, so all lanes of a warp (one slice, whatever its lanes per row) decide
// together.
__device__ __forceinline__ bool slice_idle(const unsigned char* act, int row, int n)
{
    return act != nullptr && n > 0 && act[min(row, n - 1) >> 5] == 0;
}

template <int K>
__device__ __forceinline__ void row_lane(int& r, int& q)
{
    constexpr int KK = K < 1 ? 1 : K;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    r = g / KK;
    q = g % KK;
}

// ---------------- exclusive scan ----------------
__global__ void k_scan_block(int n, const int* __restrict__ in, int* __restrict__ out, int* __restrict__ bsum)
{
    __shared__ int sh[1024];
    const int i = blockIdx.x * 1024 + threadIdx.x;
    const int v = i < n ? in[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) out[i] = sh[threadIdx.x] - v;
    if (threadIdx.x == 1023) bsum[blockIdx.x] = sh[1023];
}

__global__ void k_scan_sums(int nb, int* bsum, int* total)
{
    __shared__ int sh[1024];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += 1024) {
        const int i = base + threadIdx.x;
        const int v = i < nb ? bsum[i] : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            const int t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < nb) bsum[i] = carry + sh[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += sh[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

__global__ void k_scan_add(int n, int* __restrict__ out, const int* __restrict__ bsum)
{
    const int i = blockIdx.x * 1024 + threadIdx.x;
    if (i < n) out[i] += bsum[blockIdx.x];
}

// Short arrays (n <= SCAN_SINGLE): the whole exclusive scan in one block -- each thread loads its
// contiguous chunk (at most SCAN_PER values) into registers with all loads in flight at once, a
// two-level shuffle scan of the 1024 chunk sums, then each thread writes its chunk (one launch
// instead of three; a chunk walked load by load cost one memory latency per value, 57 us at 30 k).
constexpr int SCAN_PER = 32;
constexpr int SCAN_SINGLE = 1024 * SCAN_PER;
__global__ void __launch_bounds__(1024) k_scan_single(int n, const int* in, int* out, int* total)
{
    __shared__ int wsum[32];
    const int per = (n + 1023) / 1024;
    const int b = min(n, int(threadIdx.x) * per), e = min(n, b + per);
    int v[SCAN_PER];
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_PER; ++k) {
        v[k] = b + k < e ? in[b + k] : 0;
        s += v[k];
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int inc = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    if (w == 0) {
        const int v = wsum[lane];
        int vi = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, vi, o);
            if (lane >= o) vi += t;
        }
        wsum[lane] = vi - v;   // exclusive prefix of the warp sums
    }
    __syncthreads();
    int run = wsum[w] + inc - s;
#pragma unroll
    for (int k = 0; k < SCAN_PER; ++k) {
        if (b + k < e) out[b + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 1023 && total) *total = run;
}

// ---------------- aggregation ----------------
// rs_i = 1 / sqrt(|a_ii|): strengths |a_ij| rs_i rs_j are formed in FP32 (a coupling
// strength needs no more precision, and FP32 keeps the FP64 unit free).
template <class T>
__global__ void k_diag_rsqrt(int n, const int* __restrict__ diag, const T* __restrict__ A, float* __restrict__ rs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) rs[i] = rsqrtf(fabsf(float(A[diag[i]])));
}

// Symmetric 32-bit hash of an edge {i, j}: equal strengths (common on uniform grids) are
// ordered by this pseudo-random priority, the same from both endpoints, so locally
// dominant edges are unique and mutual-best matching pairs most rows in a few sweeps.
__device__ __forceinline__ unsigned edge_hash(int i, int j)
{
    const unsigned lo = unsigned(min(i, j)), hi = unsigned(max(i, j));
    unsigned x = lo * 0x9E3779B1u + hi * 0x85EBCA77u;
    x ^= x >> 15;
    x *= 0x2C1B3C6Du;
    x ^= x >> 12;
    x *= 0x297A2D39u;
    x ^= x >> 15;
    return x;
}

// (s, hash) lexicographic comparison with the column as the last key
__device__ __forceinline__ bool stronger(float s, unsigned h, int j, float bs, unsigned bh, int bj)
{
    return s > bs || (s == bs && (h > bh || (h == bh && j < bj)));
}

// Entry (j, a) of row i as a candidate: kept when its neighbour has the wanted state, its strength
// s = a' rs_i rs_j (a' = -a for negative couplings, |a| otherwise) passes the floor, and it beats the
// best so far.  stronger() is a total order, so the best is the same whatever the order of the entries.
__device__ __forceinline__ void consider(int i, int j, float a, int stj, float rsj, float ri, int want_state,
                                         bool neg, float floor_s, float& bs, unsigned& bh, int& bj)
{
    if (j == i || stj != want_state) return;
    const float s = (neg ? -a : fabsf(a)) * ri * rsj;
    if (!(s > 0.0f && s >= floor_s)) return;
    const unsigned h = edge_hash(i, j);
    if (bj < 0 || stronger(s, h, j, bs, bh, bj)) {
        bs = s;
        bh = h;
        bj = j;
    }
}

// The best candidate over this lane's entries q, q + K, ... of row i.  With one or two lanes per row
// (long walks per lane) the columns and values of four entries are loaded before their four state
// and scale gathers: one dependent load chain per four entries instead of one per entry.  More lanes
// walk a few entries each and keep the plain loop (and 32 registers).
template <int K, class T>
__device__ __forceinline__ void best_in_row(int i, int q, const int* __restrict__ sp, const int* __restrict__ col,
                                            const int* __restrict__ rowlen, const T* __restrict__ A,
                                            const float* __restrict__ rs, const int* __restrict__ state,
                                            int want_state, bool neg, float floor_s, float& bs, unsigned& bh,
                                            int& bj)
{
    const float ri = rs[i];
    const int len = rowlen[i];
    const int k0 = sp[i >> 5] + (i & 31);
    int t = q;
    if constexpr (K <= 2)
    for (; t + 3 * K < len; t += 4 * K) {
        const int ka = k0 + 32 * t;
        const int j0 = col[ka], j1 = col[ka + 32 * K], j2 = col[ka + 64 * K], j3 = col[ka + 96 * K];
        const float a0 = float(A[ka]), a1 = float(A[ka + 32 * K]), a2 = float(A[ka + 64 * K]),
                    a3 = float(A[ka + 96 * K]);
        const int s0 = state[j0], s1 = state[j1], s2 = state[j2], s3 = state[j3];
        const float r0 = rs[j0], r1 = rs[j1], r2 = rs[j2], r3 = rs[j3];
        consider(i, j0, a0, s0, r0, ri, want_state, neg, floor_s, bs, bh, bj);
        consider(i, j1, a1, s1, r1, ri, want_state, neg, floor_s, bs, bh, bj);
        consider(i, j2, a2, s2, r2, ri, want_state, neg, floor_s, bs, bh, bj);
        consider(i, j3, a3, s3, r3, ri, want_state, neg, floor_s, bs, bh, bj);
    }
    for (; t < len; t += K) {
        const int k = k0 + 32 * t;
        const int j = col[k];
        consider(i, j, float(A[k]), state[j], rs[j], ri, want_state, neg, floor_s, bs, bh, bj);
    }
}

// state: 0 free, 1 paired, 2 isolated (no off-diagonal coupling: never aggregated),
// 3 free without a free strong neighbour (strengths are symmetric and neighbours only ever
// become paired, so such a row cannot pair in a later sweep; it is skipped from then on and
// ends as a singleton or joins a pair)
template <class T>
__global__ void k_isolated(int n, const int* __restrict__ sp, const int* __restrict__ col,
                           const int* __restrict__ rowlen, const T* __restrict__ A, int* __restrict__ state,
                           int* __restrict__ partner, int* __restrict__ join)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    bool iso = true;
    const int len = rowlen[i];
    for (int t = 0; t < len && iso; ++t) {
        const int k = slot_of(sp, i, t);
        if (col[k] != i && A[k] != T(0)) iso = false;
    }
    state[i] = iso ? 2 : 0;
    partner[i] = -1;
    join[i] = -1;
}

// best candidate of K lanes: (strength, hash, column) is a strict total order over the distinct
// columns of a row, so the reduction gives the one-lane scan's answer in any lane order
template <int K>
__device__ __forceinline__ void best_of_lanes(float& bs, unsigned& bh, int& bj)
{
#pragma unroll
    for (int o = K >> 1; o > 0; o >>= 1) {
        const float s2 = __shfl_xor_sync(0xffffffffu, bs, o);
        const unsigned h2 = __shfl_xor_sync(0xffffffffu, bh, o);
        const int j2 = __shfl_xor_sync(0xffffffffu, bj, o);
        if (j2 >= 0 && (bj < 0 || stronger(s2, h2, j2, bs, bh, bj))) {
            bs = s2;
            bh = h2;
            bj = j2;
        }
    }
}

// Block-aggregated append of row i (when take) to a worklist: one atomic per block, the rows of
// a block in thread order.  Every thread of the block calls it (block-uniform loops only).
__device__ __forceinline__ void wl_append_block(bool take, int i, int* __restrict__ wl, int* __restrict__ cnt)
{
    __shared__ int wcnt[32];
    __shared__ int wofs[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const unsigned m = __ballot_sync(0xffffffffu, take);
    if (lane == 0) wcnt[w] = __popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
        int tot = 0;
        for (int k = 0; k < nw; ++k) {
            wofs[k] = tot;
            tot += wcnt[k];
        }
        const int base = tot ? atomicAdd(cnt, tot) : 0;
        for (int k = 0; k < nw; ++k) wofs[k] += base;
    }
    __syncthreads();
    if (take) wl[wofs[w] + __popc(m & ((1u << lane) - 1u))] = i;
    __syncthreads();   // wcnt/wofs are reused by the next call
}

// Strongest free neighbour of every free row of a worklist (-1 if none); wl == nullptr: every
// row, one thread (or K lanes) per row in row order.  K lanes per row (lane q scans the entries
// q, q + K, ...): coarse levels have few, long rows, and one thread per row leaves the SMs idle
// behind a chain of dependent gathers.  Grid-stride with K consecutive lanes per row, so every
// warp iteration is uniform and the lane reduction sees whole rows.
template <class T, int K>
__global__ void k_pick_wl(int n, const int* __restrict__ wl, const int* __restrict__ wlcnt, const int* __restrict__ sp,
                          const int* __restrict__ col, const int* __restrict__ rowlen, const T* __restrict__ A,
                          const float* __restrict__ rs, const int* __restrict__ state, int* __restrict__ best, int neg,
                          float theta)
{
    const long long total = (long long)(wl ? *wlcnt : n) * K;
    const int lane = threadIdx.x & 31;
    for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < total;
         base += (long long)gridDim.x * blockDim.x) {
        const long long g = base + lane;
        const bool valid = g < total;
        const int i = valid ? (wl ? wl[g / K] : int(g / K)) : 0;
        const int q = int(g % K);
        const bool active = valid && state[i] == 0;
        float bs = 0.0f;
        unsigned bh = 0u;
        int bj = -1;
        if (active) best_in_row<K>(i, q, sp, col, rowlen, A, rs, state, 0, neg != 0, theta, bs, bh, bj);
        if (K > 1) best_of_lanes<K>(bs, bh, bj);
        if (valid && q == 0) best[i] = active ? bj : -1;
    }
}

// Mutual best picks pair; rows without a candidate become state 3.  Over a worklist (wl ==
// nullptr: every row); the rows that stay free form the next sweep's worklist.  A sweep's
// decisions depend only on the picks and states of the sweep, not on the order of its rows.
__global__ void k_match_wl(int n, const int* __restrict__ wl, const int* __restrict__ wlcnt, int* __restrict__ state,
                           const int* __restrict__ best, int* __restrict__ partner, int* __restrict__ wl_next,
                           int* __restrict__ cnt_next)
{
    const int total = wl ? *wlcnt : n;
    for (int base = blockIdx.x * blockDim.x; base < total; base += gridDim.x * blockDim.x) {
        const int g = base + threadIdx.x;
        bool keep = false;
        int i = 0;
        if (g < total) {
            i = wl ? wl[g] : g;
            if (state[i] == 0) {
                const int j = best[i];
                if (j >= 0 && best[j] == i) {
                    state[i] = 1;
                    partner[i] = j;
                } else if (j < 0) {
                    state[i] = 3;
                } else {
                    keep = true;
                }
            }
        }
        wl_append_block(keep, i, wl_next, cnt_next);
    }
}

// unmatched rows pick their strongest paired neighbour (|a_ij| scaled); K lanes per row as k_pick_wl
template <class T, int K>
__global__ void k_join(int n, const int* __restrict__ sp, const int* __restrict__ col, const int* __restrict__ rowlen,
                       const T* __restrict__ A, const float* __restrict__ rs, const int* __restrict__ state,
                       int* __restrict__ join)
{
    int i, q;
    row_lane<K>(i, q);
    const bool valid = i < n;
    if (K <= 1 && !valid) return;
    const bool active = valid && (state[i] == 0 || state[i] == 3);
    float bs = 0.0f;
    unsigned bh = 0u;
    int bj = -1;
    if (active) best_in_row<K>(i, q, sp, col, rowlen, A, rs, state, 1, false, 0.0f, bs, bh, bj);
    if (K > 1) best_of_lanes<K>(bs, bh, bj);
    if (active && q == 0) join[i] = bj;
}

__global__ void k_rep_flag(int n, const int* __restrict__ state, const int* __restrict__ partner,
                           const int* __restrict__ join, int* __restrict__ flag)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int st = state[i];
    flag[i] = (((st == 0 || st == 3) && join[i] < 0) || (st == 1 && i < partner[i])) ? 1 : 0;
}

__global__ void k_assign(int n, const int* __restrict__ state, const int* __restrict__ partner,
                         const int* __restrict__ join, const int* __restrict__ flag, const int* __restrict__ cidx,
                         int* __restrict__ agg)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int st = state[i];
    int a;
    if (st == 2) a = -1;
    else if (flag[i]) a = cidx[i];
    else if (st == 1) a = cidx[partner[i]];
    else {
        const int t = join[i];
        a = cidx[min(t, partner[t])];
    }
    agg[i] = a;
}

__global__ void k_compose(int n, int* __restrict__ agg1, const int* __restrict__ agg2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const int a = agg1[i];
        agg1[i] = a < 0 ? -1 : agg2[a];
    }
}

__global__ void k_count_members(int n, const int* __restrict__ agg, int* __restrict__ cnt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && agg[i] >= 0) atomicAdd(&cnt[agg[i]], 1);
}

__global__ void k_fill_members(int n, const int* __restrict__ agg, int* __restrict__ pos, int* __restrict__ idx)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && agg[i] >= 0) idx[atomicAdd(&pos[agg[i]], 1)] = i;
}

__global__ void k_sort_members(int nc, const int* __restrict__ ptr, int* __restrict__ idx)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= nc) return;
    const int b = ptr[I], e = ptr[I + 1];
    for (int p = b + 1; p < e; ++p) {
        const int key = idx[p];
        int q = p - 1;
        while (q >= b && idx[q] > key) {
            idx[q + 1] = idx[q];
            --q;
        }
        idx[q + 1] = key;
    }
}

// ---------------- Galerkin products ----------------
// Merge the member rows of aggregate I, mapping columns through agg (isolated columns,
// agg < 0, carry no coupling and are skipped): sorted unique keys with summed values.
template <class T, int CAP>
__device__ int merge_rows(const int* __restrict__ sp, const int* __restrict__ col, const int* __restrict__ rowlen,
                          const T* __restrict__ A, const int* __restrict__ agg, const int* __restrict__ ptr,
                          const int* __restrict__ idx, int I, int* kc, double* kv)
{
    int m = 0;
    for (int q = ptr[I]; q < ptr[I + 1]; ++q) {
        const int r = idx[q];
        for (int t = 0; t < rowlen[r]; ++t) {
            const int k = slot_of(sp, r, t);
            const int c = agg[col[k]];
            if (c < 0) continue;
            const double v = double(A[k]);
            int pos = m;
            while (pos > 0 && kc[pos - 1] > c) --pos;
            if (pos > 0 && kc[pos - 1] == c) {
                kv[pos - 1] += v;
                continue;
            }
            for (int u = m; u > pos; --u) {
                kc[u] = kc[u - 1];
                kv[u] = kv[u - 1];
            }
            kc[pos] = c;
            kv[pos] = v;
            ++m;   // m <= CAP: the host picks CAP >= sum of member row lengths
        }
    }
    return m;
}

template <class T, int CAP>
__global__ void k_gal_count(int nc, const int* __restrict__ sp, const int* __restrict__ col,
                            const int* __restrict__ rowlen, const T* __restrict__ A, const int* __restrict__ agg,
                            const int* __restrict__ ptr, const int* __restrict__ idx, int* __restrict__ rowlen_c)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= nc) return;
    int kc[CAP];
    double kv[CAP];
    rowlen_c[I] = merge_rows<T, CAP>(sp, col, rowlen, A, agg, ptr, idx, I, kc, kv);
}

template <class T, int CAP>
__global__ void k_gal_fill(int nc, const int* __restrict__ sp, const int* __restrict__ col,
                           const int* __restrict__ rowlen, const T* __restrict__ A, const int* __restrict__ agg,
                           const int* __restrict__ ptr, const int* __restrict__ idx, const int* __restrict__ sp_c,
                           int* __restrict__ col_c, T* __restrict__ val_c, int* __restrict__ diag_c)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= nc) return;
    int kc[CAP];
    double kv[CAP];
    const int m = merge_rows<T, CAP>(sp, col, rowlen, A, agg, ptr, idx, I, kc, kv);
    const int s = I >> 5;
    const int w = (sp_c[s + 1] - sp_c[s]) >> 5;
    int dslot = -1;
    for (int t = 0; t < w; ++t) {
        const int k = sp_c[s] + t * 32 + (I & 31);
        if (t < m) {
            col_c[k] = kc[t];
            val_c[k] = T(kv[t]);
            if (kc[t] == I) dslot = k;
        } else {
            col_c[k] = I;
            val_c[k] = T(0);
        }
    }
    diag_c[I] = dslot;
}

// Per coarse row: upper bound of its merged length (sum of the member rows' lengths); the
// largest bound goes to *maxb.
__global__ void k_gal_rowbound(int nc, const int* __restrict__ ptr, const int* __restrict__ idx,
                               const int* __restrict__ rowlen, int* __restrict__ bnd, int* __restrict__ maxb)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    int b = 0;
    if (I < nc) {
        for (int q = ptr[I]; q < ptr[I + 1]; ++q) b += rowlen[idx[q]];
        bnd[I] = b;
    }
    for (int o = 16; o > 0; o >>= 1) b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxb, b);
}

// ---- Galerkin product in two passes: candidates, then a sort-free merge ----
// Pass 0: where each member row's candidates go: aggregate I's segment starts at goff[I]; its
// members (sorted) follow one another.
__global__ void k_gal_woff(int nc, const int* __restrict__ ptr, const int* __restrict__ idx,
                           const int* __restrict__ rowlen, const int* __restrict__ goff, int* __restrict__ woff)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= nc) return;
    int w = goff[I];
    for (int q = ptr[I]; q < ptr[I + 1]; ++q) {
        const int r = idx[q];
        woff[r] = w;
        w += rowlen[r];
    }
}

// Pass 1, K lanes per fine row (K = 1 on the finest levels: consecutive rows read consecutive SELL
// entries; up to 16 on coarse levels of long rows, as the matching sweeps): the row's entries with
// their columns mapped through agg (-1: an isolated column, no coupling) written to its aggregate's
// candidate segment.  Rows outside every aggregate (isolated) are skipped.
template <class T, int K>
__global__ void k_gal_cand(int n, const int* __restrict__ sp, const int* __restrict__ col,
                           const int* __restrict__ rowlen, const T* __restrict__ A, const int* __restrict__ agg,
                           const int* __restrict__ woff, int* __restrict__ ckey, T* __restrict__ cval)
{
    int i, q;
    row_lane<K>(i, q);
    if (i >= n || agg[i] < 0) return;
    const int w = woff[i], len = rowlen[i];
    const int b = sp[i >> 5] + (i & 31);
    int t = q;
    if constexpr (K <= 2)   // long walks per lane: four entries' loads and gathers in flight at once
        for (; t + 3 * K < len; t += 4 * K) {
            const int k = b + 32 * t;
            const int c0 = col[k], c1 = col[k + 32 * K], c2 = col[k + 64 * K], c3 = col[k + 96 * K];
            const T v0 = A[k], v1 = A[k + 32 * K], v2 = A[k + 64 * K], v3 = A[k + 96 * K];
            const int g0 = agg[c0], g1 = agg[c1], g2 = agg[c2], g3 = agg[c3];
            ckey[w + t] = g0;
            ckey[w + t + K] = g1;
            ckey[w + t + 2 * K] = g2;
            ckey[w + t + 3 * K] = g3;
            cval[w + t] = v0;
            cval[w + t + K] = v1;
            cval[w + t + 2 * K] = v2;
            cval[w + t + 3 * K] = v3;
        }
    for (; t < len; t += K) {
        const int k = b + 32 * t;
        ckey[w + t] = agg[col[k]];
        cval[w + t] = A[k];
    }
}

// Pass 2, L lanes per coarse row (L = 16: two rows per warp, or 32): the candidates
// [goff[I], goff[I+1]) in chunks of L (one per lane).  Equal columns of a chunk are found with
// __match_any_sync on (row in the warp, column); the lowest lane of each group sums the group's values
// in lane order (FP64) and adds the sum to the column's entry of the row's list (found by a scan of
// the list, or appended in lane order when new).  The list (first-occurrence order) is written over
// the row's own segment, with its length and the diagonal's position.  Every sum has a fixed order,
// so the product is run-to-run reproducible.  Shared memory per warp: 32 FP64 staging values and,
// per row, cap columns and cap FP64 entries of the list.
constexpr int GD_WARPS = 4;
template <class T, int L>
__global__ void __launch_bounds__(GD_WARPS * 32) k_gal_dedup(int nc, int cap, const int* __restrict__ goff,
                                                            int* __restrict__ tcol, T* __restrict__ tval,
                                                            int* __restrict__ rowlen_c, int* __restrict__ dpos,
                                                            int* __restrict__ status)
{
    constexpr int R = 32 / L;   // rows per warp
    extern __shared__ __align__(16) unsigned char gd_smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = lane / L, sl = lane % L;
    const int I0 = (blockIdx.x * GD_WARPS + w) * R;
    if (I0 >= nc) return;   // warp-uniform
    const int I = I0 + sub;
    const bool row = I < nc;
    double* stage = reinterpret_cast<double*>(gd_smem) + w * (32 + R * cap);
    double* lsum = stage + 32 + sub * cap;
    int* lkey = reinterpret_cast<int*>(reinterpret_cast<double*>(gd_smem) + GD_WARPS * (32 + R * cap)) +
                (w * R + sub) * cap;
    const int b = row ? goff[I] : 0, e = row ? goff[I + 1] : 0;
    // chunks of the warp: the most any of its rows needs
    int nch = (e - b + L - 1) / L;
#pragma unroll
    for (int o = 16; o >= L; o >>= 1) nch = max(nch, __shfl_xor_sync(0xffffffffu, nch, o));
    const unsigned rowmask = (L == 32 ? 0xffffffffu : ((1u << L) - 1u)) << (sub * L);
    int d = 0;
    for (int ch = 0; ch < nch; ++ch) {
        const int p = b + ch * L + sl;
        const bool valid = p < e;
        const int key = valid ? tcol[p] : -1;
        const bool active = key >= 0;
        stage[lane] = valid ? double(tval[p]) : 0.0;
        const unsigned long long tag =
            active ? ((unsigned long long)sub << 32) | unsigned(key) : (1ull << 63) | unsigned(lane);
        const unsigned peers = __match_any_sync(0xffffffffu, tag);
        const bool leader = active && (__ffs(peers) - 1) == lane;
        __syncwarp();
        double csum = 0.0;
        int at = -1;
        if (leader) {
            for (unsigned m = peers; m; m &= m - 1) csum += stage[__ffs(m) - 1];
            for (int q = 0; q < d; ++q)
                if (lkey[q] == key) {
                    at = q;
                    break;
                }
        }
        const unsigned fresh = __ballot_sync(0xffffffffu, leader && at < 0) & rowmask;
        if (leader) {
            if (at < 0) {
                at = d + __popc(fresh & ((1u << lane) - 1u));
                if (at < cap) {
                    lkey[at] = key;
                    lsum[at] = csum;
                } else {
                    atomicOr(status, ST_BAD_INDEX);
                }
            } else {
                lsum[at] += csum;
            }
        }
        d = min(d + __popc(fresh), cap);
        __syncwarp();
    }
    int dp = -1;
    if (row)
        for (int q = sl; q < d; q += L) {
            tcol[b + q] = lkey[q];
            tval[b + q] = T(lsum[q]);
            if (lkey[q] == I) dp = q;
        }
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) dp = max(dp, __shfl_xor_sync(0xffffffffu, dp, o));
    if (row && sl == 0) {
        rowlen_c[I] = d;
        dpos[I] = dp;
    }
}

// One warp per slice of the coarse matrix (lane = row): copy each row from the temporary
// buffer, pad past the row length (col = row, value 0; rows past nc get col = 0) and record
// the diagonal's slot (-1 if the row has none; k_check_diag reports it).
template <class T>
__global__ void k_gal_scatter(int nc, int nslices, const int* __restrict__ sp_c, const int* __restrict__ off,
                              const int* __restrict__ tcol, const T* __restrict__ tval,
                              const int* __restrict__ rowlen_c, const int* __restrict__ dpos, int* __restrict__ col_c,
                              T* __restrict__ val_c, int* __restrict__ diag_c)
{
    const int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (s >= nslices) return;
    const int lane = threadIdx.x & 31;
    const int I = s * 32 + lane;
    const int b = sp_c[s], w = (sp_c[s + 1] - b) >> 5;
    const bool row = I < nc;
    const int len = row ? rowlen_c[I] : 0;
    const int o = row ? off[I] : 0;
#pragma unroll 4   // independent entries: several loads in flight per lane
    for (int t = 0; t < w; ++t) {
        const int k = b + t * 32 + lane;
        if (t < len) {
            col_c[k] = tcol[o + t];
            val_c[k] = tval[o + t];
        } else {
            col_c[k] = row ? I : 0;
            val_c[k] = T(0);
        }
    }
    if (row) {
        const int d = dpos[I];
        diag_c[I] = d >= 0 ? b + d * 32 + lane : -1;
    }
}

__global__ void k_slice_width(int n, int nslices, const int* __restrict__ rowlen, int* __restrict__ width)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nslices) return;
    int w = 0;
    for (int r = s * 32; r < min(n, s * 32 + 32); ++r) w = max(w, rowlen[r]);
    width[s] = w * 32;
}

template <class T>
__global__ void k_pad_tail(int nc, int nslices, const int* __restrict__ sp_c, int* __restrict__ col_c,
                           T* __restrict__ val_c)
{
    const int lane = threadIdx.x;
    const int s = nslices - 1;
    const int r = s * 32 + lane;
    if (r < nc) return;
    const int w = (sp_c[s + 1] - sp_c[s]) >> 5;
    for (int t = 0; t < w; ++t) {
        const int k = sp_c[s] + t * 32 + lane;
        col_c[k] = 0;
        val_c[k] = T(0);
    }
}

__global__ void k_check_diag(int n, const int* __restrict__ diag, int* status)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && diag[i] < 0) atomicOr(status, ST_BAD_INDEX);
}

// ---------------- Chebyshev smoother ----------------
// dinv = 1/a_ii and the Gershgorin bound max_i sum_j |a_ij| / a_ii of D^-1 A.  The bound
// is an estimate for the Chebyshev interval, so it is summed in FP32 (GB300's FP64 rate is a
// small fraction of its FP32 rate) and reduced per block before one atomic per block.
template <class T>
__global__ void __launch_bounds__(256) k_cheb_setup(int n, const int* __restrict__ sp, const int* __restrict__ rowlen,
                                                    const int* __restrict__ diag, const T* __restrict__ A,
                                                    T* __restrict__ dinv, unsigned long long* gmax, int* status)
{
    __shared__ float sg[8];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float g = 0.0f;
    if (i < n) {
        const T a = A[diag[i]];
        float s = 0.0f;
        const int b = sp[i >> 5] + (i & 31);
        const int len = rowlen[i];
        for (int t = 0; t < len; ++t) s += fabsf(float(A[b + 32 * t]));
        if (!(a > T(0)) || !isfinite(s)) {
            atomicOr(status, ST_NONFINITE);
        } else {
            dinv[i] = T(1) / a;
            g = s / float(a);
        }
    }
    for (int o = 16; o > 0; o >>= 1) g = fmaxf(g, __shfl_xor_sync(0xffffffffu, g, o));
    if ((threadIdx.x & 31) == 0) sg[threadIdx.x >> 5] = g;
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = sg[0];
        for (int w = 1; w < int(blockDim.x >> 5); ++w) m = fmaxf(m, sg[w]);
        atomicMax(gmax, (unsigned long long)__double_as_longlong(double(m)));
    }
}

// start from x = 0: r = D^-1 b, d = r / theta
template <class T>
__global__ void k_cheb_start0(int n, const T* __restrict__ dinv, const T* __restrict__ b, T* __restrict__ r,
                              T* __restrict__ d, T inv_theta, const int* stop, const unsigned char* __restrict__ act)
{
    chain_wait();
    if (*stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || slice_idle(act, i, n)) return;
    const T ri = dinv[i] * b[i];
    r[i] = ri;
    d[i] = ri * inv_theta;
}


// sum_j a_rj x(j) for row r: the coalesced one-thread-per-row form for K = 1, the SELL-32x4 copy
// (sp, col, A its slice offsets, columns and FP16 values) for K = 0, the SELL-32x4 copy with 16-bit
// column offsets (col: CI = short) for K = -1, K lanes otherwise
template <int K, class T, class V, class XF, class CI>
__device__ __forceinline__ T row_dot(const int* __restrict__ sp, const CI* __restrict__ col, const V* __restrict__ A,
                                     const int* __restrict__ rowlen, int r, int q, bool valid, XF xf)
{
    if constexpr (K == -1) {
        return valid ? sell4_dot16<T>(sp, col, A, r, xf) : T(0);
    } else if constexpr (K == 0) {
        return valid ? sell4_dot<T>(sp, col, A, r, xf) : T(0);
    } else if constexpr (K == 1) {
        return valid ? sell_dot<T>(sp, col, A, r, xf) : T(0);
    } else {
        return sell_dot_lanes<K, T>(sp, col, A, rowlen, r, q, valid, xf);
    }
}

// Scaled form (SCALED, FP32 hierarchies): the matrix read is D^-1 A in FP16 (V = __half), so the
// row dot already carries the 1/a_ii factor; the unscaled residual multiplies it back by a_ii.

// start from y = t + w P xc (xc may be null: y = t): x = y, r = D^-1 (b - A y), d = r / theta
template <class T, int K, class V, bool SCALED, class CI = int>
__global__ void k_cheb_start(int n, const int* __restrict__ sp, const CI* __restrict__ col,
                             const int* __restrict__ rowlen, const V* __restrict__ A, const T* __restrict__ dinv,
                             const T* __restrict__ b, const T* __restrict__ t, const T* __restrict__ xc,
                             const int* __restrict__ agg, T wp, T* __restrict__ x, T* __restrict__ r,
                             T* __restrict__ d, T inv_theta, const int* stop, const unsigned char* __restrict__ act)
{
    chain_wait();
    if (*stop) return;
    int i, q;
    row_lane<K>(i, q);
    if (slice_idle(act, i, n)) return;
    const bool valid = i < n;
    if (K <= 1 && !valid) return;
    T acc;
    if (xc) {
        acc = row_dot<K, T>(sp, col, A, rowlen, i, q, valid, [t, xc, agg, wp](int j) {
            const int aj = agg[j];
            return t[j] + (aj >= 0 ? wp * xc[aj] : T(0));
        });
    } else {
        acc = row_dot<K, T>(sp, col, A, rowlen, i, q, valid, [t](int j) { return t[j]; });
    }
    if (!valid || q != 0) return;
    if (xc) {
        const int ai = agg[i];
        x[i] = t[i] + (ai >= 0 ? wp * xc[ai] : T(0));
    }
    const T ri = SCALED ? dinv[i] * b[i] - acc : dinv[i] * (b[i] - acc);
    r[i] = ri;
    d[i] = ri * inv_theta;
}

// y = t + w P xc (the coarse correction), for the levels whose smoother then gathers one vector
template <class T>
__global__ void k_prolong_add(int n, const T* __restrict__ t, const T* __restrict__ xc, const int* __restrict__ agg,
                              T wp, T* __restrict__ y, const int* stop, const unsigned char* __restrict__ act)
{
    chain_wait();
    if (*stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || slice_idle(act, i, n)) return;
    const int ai = agg[i];
    y[i] = t[i] + (ai >= 0 ? wp * xc[ai] : T(0));
}

// x_out = x_in + d_in; r -= D^-1 A d_in; d_out = c1 d_in + c2 r; final: x_out += d_out
template <class T, int K, class V, bool SCALED, class CI = int>
__global__ void k_cheb_step(int n, const int* __restrict__ sp, const CI* __restrict__ col,
                            const int* __restrict__ rowlen, const V* __restrict__ A, const T* __restrict__ dinv,
                            const T* x_in, const T* __restrict__ d_in, T* __restrict__ r, T* __restrict__ d_out,
                            T* x_out, T c1, T c2, int final_step, const int* stop,
                            const unsigned char* __restrict__ act)
{
    chain_wait();
    if (*stop) return;
    int i, q;
    row_lane<K>(i, q);
    if (slice_idle(act, i, n)) return;
    const bool valid = i < n;
    if (K <= 1 && !valid) return;
    // FP32: the row's own values are loaded before the row dot, so their loads overlap its gathers
    // (in FP64 the early values would take the kernel past 32 registers)
    constexpr bool early = sizeof(T) == 4;
    const bool own = valid && q == 0;
    T di = T(0), xo = T(0), r0 = T(0), dv = T(0);
    if (early && own) {
        di = d_in[i];
        xo = x_in ? x_in[i] : T(0);
        r0 = r[i];
        if (!SCALED) dv = dinv[i];
    }
    const T acc = row_dot<K, T>(sp, col, A, rowlen, i, q, valid, [d_in](int j) { return d_in[j]; });
    if (!own) return;
    if (!early) {
        di = d_in[i];
        xo = x_in ? x_in[i] : T(0);
        r0 = r[i];
        if (!SCALED) dv = dinv[i];
    }
    T xi = xo + di;
    const T ri = SCALED ? r0 - acc : r0 - dv * acc;
    const T dn = c1 * di + c2 * ri;
    if (final_step) xi += dn;
    r[i] = ri;
    d_out[i] = dn;
    x_out[i] = xi;
}

// ---- finest-level smoother step with bulk-copied matrix slices ----
// The finest level's SELL-32x4 copy streams 6 bytes per entry.  Here lane 0 of each warp (one
// slice) has the TMA engine copy the slice's columns and FP16 values into the warp's part of
// shared memory with two cp.async.bulk transfers completing on the warp's own mbarrier, so the
// warp waits for one transfer instead of a column load per group before its gathers.  The sums are
// those of k_cheb_step<T, 0, __half, true> in the same order.  Every wait is bounded: on a timeout
// the warp sets ST_TIMEOUT, waits once more (bounded) for its copies and returns without writing.
constexpr int BULK_SLICES = 8;
constexpr unsigned long long BULK_WAIT_NS = 20000000ull;  // 20 ms: a copy of a few KB takes microseconds
constexpr long long BULK_WAIT_TRIES = 1LL << 26;          // backstop should the timer not advance

__device__ __forceinline__ unsigned smem_u32(const void* p) { return unsigned(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// wait for phase 0 of the barrier; false when it has not completed within limit_ns
__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned long long limit_ns)
{
    const unsigned long long t0 = global_ns();
    for (long long it = 0; it < BULK_WAIT_TRIES; ++it) {
        unsigned ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(ok)
            : "r"(bar)
            : "memory");
        if (ok) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
    return false;
}

// Dynamic shared memory: 128 bytes for the warps' barriers (per warp one the copies complete on,
// and one gate used only by the self-test), then BULK_SLICES column areas of cap entries
// (sizeof(CI) B each: 4 for columns, 2 for 16-bit column offsets), then BULK_SLICES value areas
// (2 B each).  cap and the slice offsets are multiples of 128 entries, so every copy starts and
// ends on a 16-byte boundary.  extra_tx (0 in solves) makes the gate barrier wait for bytes that
// no copy delivers: the self-test of the timeout path, whose copies still complete on their own
// barrier, so the warp sees them land before it leaves.
template <class CI>
__device__ __forceinline__ int4 x4_columns(const CI* p, int row);
template <>
__device__ __forceinline__ int4 x4_columns<int>(const int* p, int)
{
    return *reinterpret_cast<const int4*>(p);
}
template <>
__device__ __forceinline__ int4 x4_columns<short>(const short* p, int row)
{
    const short4 c = *reinterpret_cast<const short4*>(p);
    return make_int4(row + c.x, row + c.y, row + c.z, row + c.w);
}

template <class T, class CI>
__global__ void __launch_bounds__(BULK_SLICES * 32)
    k_cheb_step_bulk(int n, int nslices, const int* __restrict__ sp4, const CI* __restrict__ col4,
                     const __half* __restrict__ a4, const T* x_in, const T* __restrict__ d_in, T* __restrict__ r,
                     T* __restrict__ d_out, T* x_out, T c1, T c2, int final_step, const int* stop, int cap,
                     int* status, unsigned extra_tx)
{
    constexpr unsigned CB = sizeof(CI);
    extern __shared__ __align__(128) unsigned char smem[];
    chain_wait();
    if (*stop) return;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int s = blockIdx.x * BULK_SLICES + w;
    if (s >= nslices) return;  // whole warps
    const int e0 = sp4[s], ne = sp4[s + 1] - e0;
    if (ne <= 0 || ne > cap || (e0 & 127)) {  // a slice wider than its staging area: no copy
        if (lane == 0) atomicOr(status, ST_BAD_INDEX);
        return;
    }
    const unsigned bar = smem_u32(smem + 8 * w);
    const unsigned gate = smem_u32(smem + 64 + 8 * w);
    CI* scol = reinterpret_cast<CI*>(smem + 128) + size_t(w) * cap;
    __half* sval = reinterpret_cast<__half*>(smem + 128 + size_t(BULK_SLICES) * cap * CB) + size_t(w) * cap;
    if (lane == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        if (extra_tx) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(gate) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(unsigned(ne) * (CB + 2u))
                     : "memory");
        if (extra_tx)
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(gate), "r"(extra_tx)
                         : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(scol)),
                     "l"(col4 + e0), "r"(unsigned(ne) * CB), "r"(bar)
                     : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(sval)),
                     "l"(a4 + e0), "r"(unsigned(ne) * 2u), "r"(bar)
                     : "memory");
    }
    __syncwarp();
    if (!((extra_tx == 0 || mbar_wait_bounded(gate, BULK_WAIT_NS)) && mbar_wait_bounded(bar, BULK_WAIT_NS))) {
        if (lane == 0) atomicOr(status, ST_TIMEOUT);
        mbar_wait_bounded(bar, BULK_WAIT_NS);  // the copies themselves may still be in flight
        return;
    }
    const int i = s * 32 + lane;
    if (i >= n) return;  // padding rows of the last slice
    const int G = ne >> 7;   // at most 4 (the staging area's cap)
    const CI* cp = scol + 4 * lane;
    const uint2* vp = reinterpret_cast<const uint2*>(sval) + lane;
    // the row's own values first, then every group unrolled: the columns come from shared memory, so
    // the gathers of all groups can be in flight together; the products are added in entry order
    const T di = d_in[i];
    const T xo = x_in ? x_in[i] : T(0);
    const T r0 = r[i];
    T acc = T(0);
#pragma unroll
    for (int g = 0; g < 4; ++g) {
        if (g < G) {
            const int4 c = x4_columns<CI>(cp + 128 * g, i);
            const uint2 h = vp[32 * g];
            const T x0 = d_in[c.x], x1 = d_in[c.y], x2 = d_in[c.z], x3 = d_in[c.w];
            const float2 v01 = __half22float2(*reinterpret_cast<const __half2*>(&h.x));
            const float2 v23 = __half22float2(*reinterpret_cast<const __half2*>(&h.y));
            acc += T(v01.x) * x0;
            acc += T(v01.y) * x1;
            acc += T(v23.x) * x2;
            acc += T(v23.y) * x3;
        }
    }
    T xi = xo + di;
    const T ri = r0 - acc;
    const T dn = c1 * di + c2 * ri;
    if (final_step) xi += dn;
    r[i] = ri;
    d_out[i] = dn;
    x_out[i] = xi;
}

template <class T, int K, class V, bool SCALED, class CI = int>
__global__ void k_resid(int n, const int* __restrict__ sp, const CI* __restrict__ col, const int* __restrict__ rowlen,
                        const V* __restrict__ A, const T* __restrict__ diagv, const T* __restrict__ b,
                        const T* __restrict__ x, T* __restrict__ r, const int* stop,
                        const unsigned char* __restrict__ act)
{
    chain_wait();
    if (*stop) return;
    int i, q;
    row_lane<K>(i, q);
    if (slice_idle(act, i, n)) return;
    const bool valid = i < n;
    if (K <= 1 && !valid) return;
    const T acc = row_dot<K, T>(sp, col, A, rowlen, i, q, valid, [x](int j) { return x[j]; });
    if (!valid || q != 0) return;
    r[i] = SCALED ? b[i] - diagv[i] * acc : b[i] - acc;
}

// D^-1 A in FP16 (padding slots stay 0) and the diagonal, for the scaled smoother
template <class T>
__global__ void k_scale_half(int n, const int* __restrict__ sp, const int* __restrict__ rowlen,
                             const int* __restrict__ diag, const T* __restrict__ A, const T* __restrict__ dinv,
                             __half* __restrict__ ah, T* __restrict__ diagv)
{
    const int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int nslices = (n + 31) >> 5;
    if (s >= nslices) return;
    const int lane = threadIdx.x & 31, r = s * 32 + lane;
    const int b = sp[s], w = (sp[s + 1] - b) >> 5;
    const bool row = r < n;
    const T di = row ? dinv[r] : T(0);
    for (int t = 0; t < w; ++t) {
        const int k = b + 32 * t + lane;
        ah[k] = __float2half_rn(row ? float(A[k] * di) : 0.0f);
    }
    if (row) diagv[r] = A[diag[r]];
}

// SELL-32x4 copy of a level for the one-thread-per-row smoother: per slice, groups of four
// consecutive entries of each row, lane-interleaved (entry t of row r at
// sp4[r/32] + 128 (t/4) + 4 (r%32) + t%4), so a row's four columns come in one 16-byte load and its
// four FP16 values in one 8-byte load.  Rows are padded to a multiple of four entries (col = row,
// value 0).  groups[s] = 128 * ceil(width / 4).
// 16-bit column offsets of a coarse level's SELL pattern (col - row; 0 on the padding rows of the last
// slice), one warp per slice, and the level's largest |col - row| into *maxoff: above 32767 the
// truncated copy is not used
__global__ void k_col_offsets(int n, int nslices, const int* __restrict__ sp, const int* __restrict__ col,
                              short* __restrict__ off, int* __restrict__ maxoff)
{
    const int sl = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (sl >= nslices) return;   // whole warps
    const int lane = threadIdx.x & 31, r = sl * 32 + lane;
    const int b = sp[sl], w = (sp[sl + 1] - b) >> 5;
    int mo = 0;
    for (int t = 0; t < w; ++t) {
        const int k = b + 32 * t + lane;
        const int o = r < n ? col[k] - r : 0;
        mo = max(mo, abs(o));
        off[k] = short(o);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mo = max(mo, __shfl_xor_sync(0xffffffffu, mo, o));
    if (lane == 0 && mo > 0) atomicMax(maxoff, mo);
}

__global__ void k_slice_groups(int nslices, const int* __restrict__ sp, int* __restrict__ groups)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nslices) groups[s] = ((((sp[s + 1] - sp[s]) >> 5) + 3) >> 2) * 128;
}

// the SELL-32x4 copy written straight from A (FP16 D^-1 A as k_scale_half), and the diagonal.
// CI = int stores the columns; CI = short stores col - row (padding 0), and the largest |col - row|
// of the level goes to *maxoff: above 32767 the offsets do not fit and the int copy is written
// instead (the padding rows of the last slice point at row 0 in the int copy, at themselves here).
template <class T, class CI>
__global__ void k_scale_half4(int n, int nslices, const int* __restrict__ sp, const int* __restrict__ col,
                              const int* __restrict__ diag, const T* __restrict__ A, const T* __restrict__ dinv,
                              const int* __restrict__ sp4, CI* __restrict__ col4, __half* __restrict__ ah4,
                              T* __restrict__ diagv, int* __restrict__ maxoff)
{
    const int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (s >= nslices) return;
    const int lane = threadIdx.x & 31, r = s * 32 + lane;
    const bool row = r < n;
    const T di = row ? dinv[r] : T(0);
    const int b = sp[s], w = (sp[s + 1] - b) >> 5;
    const int b4 = sp4[s], g4 = (sp4[s + 1] - b4) >> 7;
    int mo = 0;
    for (int t = 0; t < 4 * g4; ++t) {
        const int dst = b4 + 128 * (t >> 2) + 4 * lane + (t & 3);
        if (t < w) {
            const int k = b + 32 * t + lane;
            const int c = col[k];
            if constexpr (std::is_same<CI, short>::value) {
                const int o = row ? c - r : 0;
                mo = max(mo, abs(o));
                col4[dst] = short(max(-32768, min(32767, o)));
            } else {
                col4[dst] = c;
            }
            ah4[dst] = __float2half_rn(row ? float(A[k] * di) : 0.0f);
        } else {
            if constexpr (std::is_same<CI, short>::value) col4[dst] = 0;
            else col4[dst] = row ? r : 0;
            ah4[dst] = __float2half_rn(0.0f);
        }
    }
    if (row) diagv[r] = A[diag[r]];
    if (maxoff) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mo = max(mo, __shfl_xor_sync(0xffffffffu, mo, o));
        if (lane == 0 && mo > 0) atomicMax(maxoff, mo);
    }
}

template <class T>
__global__ void k_restrict(int nc, const int* __restrict__ ptr, const int* __restrict__ idx, const T* __restrict__ r,
                           T* __restrict__ bc, const int* stop, const unsigned char* __restrict__ act)
{
    chain_wait();
    if (*stop) return;
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= nc || slice_idle(act, I, nc)) return;
    T s = 0;
    for (int q = ptr[I]; q < ptr[I + 1]; ++q) s += r[idx[q]];
    bc[I] = s;
}

// k_restrict fused with the coarse level's first Chebyshev start from zero (k_cheb_start0 on bc):
// the same sums, the same rc and dc
template <class T>
__global__ void k_restrict_start0(int nc, const int* __restrict__ ptr, const int* __restrict__ idx,
                                  const T* __restrict__ r, T* __restrict__ bc, const T* __restrict__ dinv_c,
                                  T* __restrict__ rc, T* __restrict__ dc, T inv_theta, const int* stop,
                                  const unsigned char* __restrict__ act)
{
    chain_wait();
    if (*stop) return;
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= nc || slice_idle(act, I, nc)) return;
    T s = 0;
    for (int q = ptr[I]; q < ptr[I + 1]; ++q) s += r[idx[q]];
    bc[I] = s;
    const T ri = dinv_c[I] * s;
    rc[I] = ri;
    dc[I] = ri * inv_theta;
}

// ---- block skipping (batched solves) ----
// block of each coarse row: that of its first member (aggregates never cross blocks)
__global__ void k_level_blocks(int nc, const int* __restrict__ ptr, const int* __restrict__ idx,
                               const int* __restrict__ blk_f, int* __restrict__ blk_c)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I < nc) blk_c[I] = blk_f[idx[ptr[I]]];
}

// act[s] = 1 when a row of slice s belongs to a block still iterating (conv == 0); one warp per slice
__global__ void k_slice_active(int n, int nslices, const int* __restrict__ blk, const int* __restrict__ conv,
                               unsigned char* __restrict__ act, const int* stop)
{
    chain_wait();
    if (*stop) return;
    const int sl = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (sl >= nslices) return;   // whole warps
    const int r = sl * 32 + (threadIdx.x & 31);
    const bool live = r < n && conv[blk[r]] == 0;
    const unsigned any = __ballot_sync(0xffffffffu, live);
    if ((threadIdx.x & 31) == 0) act[sl] = any ? 1 : 0;
}

// ---------------- K-cycle (Krylov-accelerated coarse correction) ----------------
// y = A x on a level (plain SELL, one thread per row)
template <class T>
__global__ void k_lv_spmv(int n, const int* __restrict__ sp, const int* __restrict__ col, const T* __restrict__ A,
                          const T* __restrict__ x, T* __restrict__ y, const int* stop)
{
    chain_wait();
    if (*stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    y[i] = sell_dot<T>(sp, col, A, i, [x](int j) { return x[j]; });
}

// Up to three dot products a_d . b_d at once (null pairs skipped): per block partial sums
// (FP64 per warp, fixed order) into part[3 * block + d]; a one-block kernel finishes them.
template <class T>
__global__ void __launch_bounds__(256) k_kdots(int n, const T* __restrict__ a0, const T* __restrict__ b0,
                                               const T* __restrict__ a1, const T* __restrict__ b1,
                                               const T* __restrict__ a2, const T* __restrict__ b2,
                                               double* __restrict__ part, const int* stop)
{
    chain_wait();
    if (*stop) return;
    __shared__ double sh[3][8];
    double v[3] = {0.0, 0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        v[0] += double(a0[i]) * double(b0[i]);
        if (a1) v[1] += double(a1[i]) * double(b1[i]);
        if (a2) v[2] += double(a2[i]) * double(b2[i]);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[d] += __shfl_xor_sync(0xffffffffu, v[d], o);
        if (lane == 0) sh[d][w] = v[d];
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int k = 0; k < int(blockDim.x >> 5); ++k) t += sh[threadIdx.x][k];
        part[3 * blockIdx.x + threadIdx.x] = t;
    }
}

// Finish the dots (block partials summed in block order) and form the coefficients, in c[0..7]
// of the level: step 1 (c1 = B b, v1 = A c1): rho1 = c1.v1, alpha1 = c1.b, a = alpha1 / rho1;
// step 2 (c2 = B r2, v2 = A c2, r2 = b - a v1): gamma = c2.v1, beta = c2.v2, alpha2 = c2.r2,
// rho2 = beta - gamma^2 / rho1, x = k1 c1 + k2 c2 with k2 = alpha2 / rho2,
// k1 = a - gamma k2 / rho1 (the flexible-CG iterate after two steps).  A non-positive curvature
// falls back to one step (k2 = 0) or to the plain cycle (k1 = 1).
__global__ void k_kfinish(int nblocks, const double* __restrict__ part, double* __restrict__ c, int step,
                          const int* stop)
{
    chain_wait();
    if (*stop) return;
    __shared__ double sh[3][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double v[3] = {0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
#pragma unroll
        for (int d = 0; d < 3; ++d) v[d] += part[3 * b + d];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[d] += __shfl_xor_sync(0xffffffffu, v[d], o);
        if (lane == 0) sh[d][w] = v[d];
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    double t[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < int(blockDim.x >> 5); ++k)
        for (int d = 0; d < 3; ++d) t[d] += sh[d][k];
    if (step == 1) {
        const double rho1 = t[0], alpha1 = t[1];
        const bool ok = rho1 > 0.0 && isfinite(rho1) && isfinite(alpha1);
        c[0] = rho1;
        c[1] = alpha1;
        c[2] = ok ? alpha1 / rho1 : 0.0;
        c[3] = ok ? 1.0 : 0.0;
    } else {
        const double rho1 = c[0], a = c[2];
        const double gamma = t[0], beta = t[1], alpha2 = t[2];
        double k1 = 1.0, k2 = 0.0;
        if (c[3] != 0.0) {
            const double rho2 = beta - gamma * gamma / rho1;
            if (rho2 > 1e-12 * beta && isfinite(rho2) && isfinite(alpha2)) {
                k2 = alpha2 / rho2;
                k1 = a - gamma * k2 / rho1;
            } else {
                k1 = a;
            }
        }
        c[4] = k1;
        c[5] = k2;
    }
}

// r2 = b - a v1
template <class T>
__global__ void k_kresid(int n, const T* __restrict__ b, const T* __restrict__ v1, const double* __restrict__ c,
                         T* __restrict__ r2, const int* stop)
{
    chain_wait();
    if (*stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) r2[i] = T(double(b[i]) - c[2] * double(v1[i]));
}

// x = k1 c1 + k2 c2
template <class T>
__global__ void k_kcombine(int n, const T* __restrict__ c1, const T* __restrict__ c2, const double* __restrict__ c,
                           T* __restrict__ x, const int* stop)
{
    chain_wait();
    if (*stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = T(c[4] * double(c1[i]) + c[5] * double(c2[i]));
}

// ---------------- coarsest level ----------------
template <class T>
__global__ void k_dense_from_sell(int n, const int* __restrict__ sp, const int* __restrict__ col,
                                  const int* __restrict__ rowlen, const T* __restrict__ A, double* __restrict__ D)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int j = 0; j < n; ++j) D[(size_t)i * n + j] = 0.0;
    for (int t = 0; t < rowlen[i]; ++t) {
        const int k = slot_of(sp, i, t);
        D[(size_t)i * n + col[k]] += double(A[k]);
    }
}

// In-place Cholesky (lower) of the dense SPD matrix D, then Dinv = L^-T L^-1.  One block.
__global__ void k_dense_cholesky_inverse(int n, double* __restrict__ D, double* __restrict__ Linv,
                                         double* __restrict__ Dinv, int* status)
{
    for (int k = 0; k < n; ++k) {
        if (threadIdx.x == 0) {
            const double a = D[(size_t)k * n + k];
            if (!(a > 0.0) || !isfinite(a)) atomicOr(status, ST_NONFINITE);
            D[(size_t)k * n + k] = sqrt(a > 0.0 ? a : 1.0);
        }
        __syncthreads();
        const double lkk = D[(size_t)k * n + k];
        for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) D[(size_t)i * n + k] /= lkk;
        __syncthreads();
        const int m = n - k - 1;
        for (long long q = threadIdx.x; q < (long long)m * m; q += blockDim.x) {
            const int i = k + 1 + int(q / m), j = k + 1 + int(q % m);
            if (j <= i) D[(size_t)i * n + j] -= D[(size_t)i * n + k] * D[(size_t)j * n + k];
        }
        __syncthreads();
    }
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        for (int i = 0; i < n; ++i) Linv[(size_t)i * n + j] = 0.0;
        for (int i = j; i < n; ++i) {
            double s = (i == j) ? 1.0 : 0.0;
            for (int k = j; k < i; ++k) s -= D[(size_t)i * n + k] * Linv[(size_t)k * n + j];
            Linv[(size_t)i * n + j] = s / D[(size_t)i * n + i];
        }
    }
    __syncthreads();
    for (long long q = threadIdx.x; q < (long long)n * n; q += blockDim.x) {
        const int i = int(q / n), j = int(q % n);
        double s = 0.0;
        for (int k = max(i, j); k < n; ++k) s += Linv[(size_t)k * n + i] * Linv[(size_t)k * n + j];
        Dinv[q] = s;
    }
}

// Inverse of the dense SPD matrix D (n <= DENSE_SMEM_N) by Gauss-Jordan elimination in shared
// memory, one block of 32 x 32 threads (thread (tx, ty) owns the entries (ty + 32 a, tx + 32 b)):
// for SPD matrices the pivots are the diagonal (no pivoting, as LDL^T).  Per pivot k, first every
// entry outside row and column k is updated from the old row and column, then row and column k are
// scaled: two barriers per pivot.  Non-positive or non-finite pivots set ST_NONFINITE.
constexpr int DENSE_SMEM_N = 160;   // 200 KB of doubles
__global__ void __launch_bounds__(1024) k_dense_gauss_jordan(int n, const double* __restrict__ D,
                                                             double* __restrict__ Dinv, int* status)
{
    extern __shared__ double A[];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int q = threadIdx.x; q < n * n; q += blockDim.x) A[q] = D[q];
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        const double akk = A[k * n + k];
        if (!(akk > 0.0) || !isfinite(akk)) {
            if (threadIdx.x == 0) atomicOr(status, ST_NONFINITE);
            return;   // uniform: every thread read the same pivot
        }
        const double piv = 1.0 / akk;
        for (int i = ty; i < n; i += 32) {
            if (i == k) continue;
            const double aik = A[i * n + k] * piv;
            for (int j = tx; j < n; j += 32)
                if (j != k) A[i * n + j] -= aik * A[k * n + j];
        }
        __syncthreads();
        if (ty == 0)
            for (int j = tx; j < n; j += 32)
                if (j != k) A[k * n + j] *= piv;
        if (ty == 1)
            for (int i = tx; i < n; i += 32) A[i * n + k] = (i == k) ? piv : -A[i * n + k] * piv;
        __syncthreads();
    }
    for (int q = threadIdx.x; q < n * n; q += blockDim.x) Dinv[q] = A[q];
}

template <class T>
__global__ void k_dense_apply(int n, const double* __restrict__ Dinv, const T* __restrict__ b, T* __restrict__ x,
                              const int* stop, const unsigned char* __restrict__ act, const int* __restrict__ blk,
                              const int* __restrict__ conv)
{
    chain_wait();
    if (*stop) return;
    extern __shared__ double sb[];
    // batched solves (blk, conv not null): the block-diagonal inverse couples nothing across blocks,
    // but its zeros would still carry a converged block's values (0 * Inf is NaN), so those enter as
    // 0: a converged block's rows are only partly recomputed, from partly stale inputs, and in FP32
    // that mix can overflow
    for (int j = threadIdx.x; j < n; j += blockDim.x) sb[j] = (conv && conv[blk[j]] != 0) ? 0.0 : double(b[j]);
    __syncthreads();
    // one warp per row, blockDim/32 rows per block: a large coarsest level (up to 2048 rows
    // when coarsening stalls) spreads over many SMs instead of one
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int i = blockIdx.x * nw + warp;
    if (i >= n || slice_idle(act, i, n)) return;   // one row per warp
    double s = 0.0;
    for (int j = lane; j < n; j += 32) s += Dinv[(size_t)i * n + j] * sb[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) x[i] = T(s);
}

int read_int(cudaStream_t s, const int* d)
{
    int v = 0;
    PORSOL_CUDA(cudaMemcpyAsync(&v, d, sizeof(int), cudaMemcpyDeviceToHost, s));
    PORSOL_CUDA(cudaStreamSynchronize(s));
    return v;
}

// Lanes per row of a level.  Levels with many rows are bandwidth-bound and keep one thread per
// row (consecutive threads on consecutive rows give fully coalesced SELL loads; more lanes only
// add instructions).  Small levels (under 20k rows, 30-60 entries per row) are latency-bound:
// one thread would walk its long row serially, so 3-6 entries per lane are used there.  Between
// the two, levels of long rows under 64k rows, whose one-thread-per-row launch fills about one
// 256-thread block per SM (on the 1M-cell system: 44k rows of 52 entries, 14.5 us per smoothing
// step against 12.5 us with 8 lanes), double the lanes until the launch has about 2^18 threads,
// keeping at least five entries per lane.  At 121k rows of 42 entries the one-thread-per-row
// SELL-32x4 step was faster than 4 lanes (13.8 against 15.0 us).
constexpr long long LANES_FILL_THREADS = 1LL << 18;
int lanes_for(int n, long long nent)
{
    const double avg = n > 0 ? double(nent) / n : 0.0;
    if (avg <= 8.0) return 1;
    if (n >= 65536) return 1;
    if (n >= 20000) {
        int k = 1;
        while (k < 8 && (long long)n * k < LANES_FILL_THREADS && avg / (2 * k) >= 5.0) k *= 2;
        return k;
    }
    int k = 2;
    while (k < 16 && k * 6 < avg) k *= 2;
    return k;
}

// Lanes per row of the matching sweeps: rows longer than about 12 entries (the coarse
// levels) are scanned by up to 16 lanes, at least 4 entries per lane.
int pick_lanes(int n, long long nent)
{
    const double avg = n > 0 ? double(nent) / n : 0.0;
    if (avg <= 12.0) return 1;
    int k = 1;
    while (k < 16 && 8 * k <= avg) k *= 2;
    return k;
}

#define PORSOL_LANES(K, LAUNCH)                                                                                    \
    switch (K) {                                                                                                   \
    case 1: { constexpr int KL = 1; LAUNCH; } break;                                                              \
    case 2: { constexpr int KL = 2; LAUNCH; } break;                                                              \
    case 4: { constexpr int KL = 4; LAUNCH; } break;                                                              \
    case 8: { constexpr int KL = 8; LAUNCH; } break;                                                              \
    default: { constexpr int KL = 16; LAUNCH; } break;                                                            \
    }

// Blocks of the grid-stride matching launches: at most 8 per SM (the device's SM count).
int stride_blocks(long long threads)
{
    static int cap = 0;
    if (cap == 0) {
        int dev = 0, sms = 0;
        PORSOL_CUDA(cudaGetDevice(&dev));
        PORSOL_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        cap = std::max(1, 8 * sms);
    }
    return std::max(1, std::min(div_up(std::max(threads, 1LL), TB), cap));
}

// Process-wide cache of autotuned lanes per row, keyed by level shape.
std::mutex& tune_mutex()
{
    static std::mutex m;
    return m;
}
std::unordered_map<long long, int>& tune_cache()
{
    static std::unordered_map<long long, int> c;
    return c;
}

}  // namespace

void exclusive_scan(cudaStream_t s, int n, const int* in, int* out, int* total_dev, DBuf<int>& scratch)
{
    if (n <= SCAN_SINGLE) {
        PORSOL_LAUNCH(k_scan_single<<<1, 1024, 0, s>>>(n, in, out, total_dev));
        PORSOL_CUDA(cudaGetLastError());
        return;
    }
    const int nb = std::max(1, div_up(n, 1024));
    if ((int)scratch.n < nb) scratch.alloc(nb);
    if (n > 0) PORSOL_LAUNCH(k_scan_block<<<nb, 1024, 0, s>>>(n, in, out, scratch.p));
    else PORSOL_CUDA(cudaMemsetAsync(scratch.p, 0, sizeof(int), s));
    PORSOL_LAUNCH(k_scan_sums<<<1, 1024, 0, s>>>(n > 0 ? nb : 1, scratch.p, total_dev));
    if (n > 0) PORSOL_LAUNCH(k_scan_add<<<nb, 1024, 0, s>>>(n, out, scratch.p));
    PORSOL_CUDA(cudaGetLastError());
}

template <class T>
void Amg<T>::pairwise(cudaStream_t s, const SellPattern& P, const T* A, int n, bool neg, double theta, bool join,
                      Aggregates& out)
{
    DBuf<float>& d = s_rs_;
    DBuf<int>&state = s_state_, &partner = s_partner_, &jn = s_join_, &best = s_best_, &flag = s_flag_,
    &cidx = s_cidx_;
    d.alloc(n);
    state.alloc(n);
    partner.alloc(n);
    jn.alloc(n);
    best.alloc(n);
    flag.alloc(n);
    cidx.alloc(n + 1);
    const int nb = div_up(n, TB);
    PORSOL_LAUNCH(k_diag_rsqrt<T><<<nb, TB, 0, s>>>(n, P.diag.p, A, d.p));
    PORSOL_LAUNCH(k_isolated<T><<<nb, TB, 0, s>>>(n, P.slice_ptr.p, P.col.p, P.rowlen.p, A, state.p, partner.p, jn.p));
    // Mutual-best matching: each sweep pairs at least the strongest remaining edge; the
    // stall fallback (join) runs more sweeps so chains and stars also pair up.
    const int sweeps = join ? 8 : 4;
    const int lanes = pick_lanes(n, P.nent);
    // The first sweep visits every row (one thread or K lanes per row); each later sweep only the
    // rows still free after the previous one (a worklist the match kernel builds), in grid-stride
    // launches of at most 8 blocks per SM: the decisions are those of full sweeps, the later
    // sweeps cost a fraction of the first.
    s_wl_[0].alloc(n);
    s_wl_[1].alloc(n);
    s_wlcnt_.alloc(2);
    const int nbk = div_up((long long)n * lanes, TB);
    const int nbp = stride_blocks((long long)n * lanes);
    const int nbm = stride_blocks(n);
    for (int sweep = 0; sweep < sweeps; ++sweep) {
        const int cur = sweep & 1, nxt = cur ^ 1;
        const int* wl = sweep == 0 ? nullptr : s_wl_[cur].p;
        PORSOL_LANES(lanes, PORSOL_LAUNCH((k_pick_wl<T, KL><<<sweep == 0 ? nbk : nbp, TB, 0, s>>>(
                                n, wl, s_wlcnt_.p + cur, P.slice_ptr.p, P.col.p, P.rowlen.p, A, d.p, state.p, best.p,
                                neg ? 1 : 0, float(theta)))));
        PORSOL_CUDA(cudaMemsetAsync(s_wlcnt_.p + nxt, 0, sizeof(int), s));
        PORSOL_LAUNCH(k_match_wl<<<sweep == 0 ? nb : nbm, TB, 0, s>>>(n, wl, s_wlcnt_.p + cur, state.p, best.p,
                                                                      partner.p, s_wl_[nxt].p, s_wlcnt_.p + nxt));
    }
    if (join)
        PORSOL_LANES(lanes, PORSOL_LAUNCH((k_join<T, KL><<<nbk, TB, 0, s>>>(n, P.slice_ptr.p, P.col.p, P.rowlen.p, A, d.p,
                                                                           state.p, jn.p))));
    PORSOL_LAUNCH(k_rep_flag<<<nb, TB, 0, s>>>(n, state.p, partner.p, jn.p, flag.p));
    exclusive_scan(s, n, flag.p, cidx.p, cidx.p + n, scan_blocks_);
    out.n = n;
    out.nc = read_int(s, cidx.p + n);
    out.agg.alloc(n);
    PORSOL_LAUNCH(k_assign<<<nb, TB, 0, s>>>(n, state.p, partner.p, jn.p, flag.p, cidx.p, out.agg.p));
    PORSOL_CUDA(cudaGetLastError());
}

template <class T>
void Amg<T>::members(cudaStream_t s, Aggregates& a)
{
    const int n = a.n, nc = a.nc;
    DBuf<int>&cnt = s_cnt_, &pos = s_pos_;
    cnt.alloc(std::max(nc, 1));
    pos.alloc(std::max(nc, 1));
    PORSOL_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int) * std::max(nc, 1), s));
    a.ptr.alloc(nc + 1);
    PORSOL_LAUNCH(k_count_members<<<div_up(n, TB), TB, 0, s>>>(n, a.agg.p, cnt.p));
    exclusive_scan(s, nc, cnt.p, a.ptr.p, a.ptr.p + nc, scan_blocks_);
    a.idx.alloc(std::max(n, 1));   // members <= rows; no host read of the exact count
    PORSOL_CUDA(cudaMemcpyAsync(pos.p, a.ptr.p, sizeof(int) * nc, cudaMemcpyDeviceToDevice, s));
    PORSOL_LAUNCH(k_fill_members<<<div_up(n, TB), TB, 0, s>>>(n, a.agg.p, pos.p, a.idx.p));
    PORSOL_LAUNCH(k_sort_members<<<div_up(nc, TB), TB, 0, s>>>(nc, a.ptr.p, a.idx.p));
    PORSOL_CUDA(cudaGetLastError());
}

template <class T>
void Amg<T>::aggregate_round(cudaStream_t s, const SellPattern& P, const T* A, int n, bool neg_first,
                             Aggregates& out)
{
    int first = -1;
    if (neg_first) {
        pairwise(s, P, A, n, true, o_.strength, false, out);
        first = out.nc;
    }
    if (!neg_first || out.nc > 0.8 * n) pairwise(s, P, A, n, false, 0.0, true, out);
    static const bool debug = std::getenv("PORSOL_DEBUG_AMG") != nullptr;
    if (debug) std::fprintf(stderr, "[amg] round n=%d strong-negative pairs -> %d, final -> %d\n", n, first, out.nc);
}

template <class T>
void Amg<T>::galerkin(cudaStream_t s, const SellPattern& P, const T* A, const Aggregates& a, SellPattern& Pc,
                      DBuf<T>& Ac)
{
    const int nc = a.nc;
    Pc.n = nc;
    Pc.nslices = div_up(nc, 32);
    Pc.rowlen.alloc(std::max(nc, 1));
    Pc.diag.alloc(std::max(nc, 1));
    Pc.slice_ptr.alloc(Pc.nslices + 1);
    iscratch_.alloc(4);
    PORSOL_CUDA(cudaMemsetAsync(iscratch_.p, 0, sizeof(int), s));
    s_bnd_.alloc(std::max(nc, 1));
    s_goff_.alloc(nc + 1);
    PORSOL_LAUNCH(k_gal_rowbound<<<div_up(nc, TB), TB, 0, s>>>(nc, a.ptr.p, a.idx.p, P.rowlen.p, s_bnd_.p,
                                                                iscratch_.p));
    exclusive_scan(s, nc, s_bnd_.p, s_goff_.p, s_goff_.p + nc, scan_blocks_);
    int hb[2] = {0, 0};
    PORSOL_CUDA(cudaMemcpyAsync(&hb[0], iscratch_.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    PORSOL_CUDA(cudaMemcpyAsync(&hb[1], s_goff_.p + nc, sizeof(int), cudaMemcpyDeviceToHost, s));
    PORSOL_CUDA(cudaStreamSynchronize(s));
    const int bound = hb[0], total = hb[1];
    PORSOL_REQUIRE(bound <= 2048, PORSOL_ERR_BAD_ARG, "AMG: aggregate rows too long for the Galerkin merge");
    const bool warp = bound <= 1024;
    if (warp) {
        // candidates of every aggregate row into a compact temporary, merged there, then the SELL layout
        s_tcol_.alloc(std::max(total, 1));
        s_tval_.alloc(std::max(total, 1));
        s_dpos_.alloc(std::max(nc, 1));
        s_woff_.alloc(std::max(P.n, 1));
        PORSOL_LAUNCH(k_gal_woff<<<div_up(nc, TB), TB, 0, s>>>(nc, a.ptr.p, a.idx.p, P.rowlen.p, s_goff_.p,
                                                               s_woff_.p));
        const int cl = pick_lanes(P.n, P.nent);
        PORSOL_LANES(cl, PORSOL_LAUNCH((k_gal_cand<T, KL><<<div_up((long long)P.n * cl, TB), TB, 0, s>>>(
                             P.n, P.slice_ptr.p, P.col.p, P.rowlen.p, A, a.agg.p, s_woff_.p, s_tcol_.p, s_tval_.p))));
        // rows of up to 64 candidates (the finest levels' pairs and quadruples) take half a warp each
        const int cap = std::max(32, (bound + 31) / 32 * 32);
        if (bound <= 64) {
            const size_t shm = size_t(GD_WARPS) * ((32 + 2 * cap) * sizeof(double) + 2 * cap * sizeof(int));
            PORSOL_LAUNCH((k_gal_dedup<T, 16><<<div_up(nc, 2 * GD_WARPS), GD_WARPS * 32, shm, s>>>(
                nc, cap, s_goff_.p, s_tcol_.p, s_tval_.p, Pc.rowlen.p, s_dpos_.p, status_.p)));
        } else {
            const size_t shm = size_t(GD_WARPS) * ((32 + cap) * sizeof(double) + cap * sizeof(int));
            if (shm > 48 * 1024)
                PORSOL_CUDA(cudaFuncSetAttribute(k_gal_dedup<T, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 int(shm)));
            PORSOL_LAUNCH((k_gal_dedup<T, 32><<<div_up(nc, GD_WARPS), GD_WARPS * 32, shm, s>>>(
                nc, cap, s_goff_.p, s_tcol_.p, s_tval_.p, Pc.rowlen.p, s_dpos_.p, status_.p)));
        }
    } else {
        const int nb = div_up(nc, 64);
        PORSOL_COUNT_LAUNCH();
        k_gal_count<T, 2048><<<nb, 64, 0, s>>>(nc, P.slice_ptr.p, P.col.p, P.rowlen.p, A, a.agg.p, a.ptr.p, a.idx.p,
                                               Pc.rowlen.p);
    }
    DBuf<int>& width = s_width_;
    width.alloc(Pc.nslices);
    PORSOL_LAUNCH(k_slice_width<<<div_up(Pc.nslices, TB), TB, 0, s>>>(nc, Pc.nslices, Pc.rowlen.p, width.p));
    exclusive_scan(s, Pc.nslices, width.p, Pc.slice_ptr.p, Pc.slice_ptr.p + Pc.nslices, scan_blocks_);
    Pc.nent = read_int(s, Pc.slice_ptr.p + Pc.nslices);
    Pc.col.alloc(std::max<long long>(Pc.nent, 1));
    Ac.alloc(std::max<long long>(Pc.nent, 1));
    if (warp) {
        PORSOL_LAUNCH(k_gal_scatter<T><<<div_up(Pc.nslices, TB / 32), TB, 0, s>>>(
            nc, Pc.nslices, Pc.slice_ptr.p, s_goff_.p, s_tcol_.p, s_tval_.p, Pc.rowlen.p, s_dpos_.p, Pc.col.p, Ac.p,
            Pc.diag.p));
    } else {
        const int nb = div_up(nc, 64);
        PORSOL_COUNT_LAUNCH();
        k_gal_fill<T, 2048><<<nb, 64, 0, s>>>(nc, P.slice_ptr.p, P.col.p, P.rowlen.p, A, a.agg.p, a.ptr.p, a.idx.p,
                                              Pc.slice_ptr.p, Pc.col.p, Ac.p, Pc.diag.p);
        if (nc > 0) PORSOL_LAUNCH(k_pad_tail<T><<<1, 32, 0, s>>>(nc, Pc.nslices, Pc.slice_ptr.p, Pc.col.p, Ac.p));
    }
    PORSOL_LAUNCH(k_check_diag<<<div_up(nc, TB), TB, 0, s>>>(nc, Pc.diag.p, status_.p));
    PORSOL_CUDA(cudaGetLastError());
}

template <class T>
void Amg<T>::smoother_setup(cudaStream_t s, Level& L, int level)
{
    const int n = L.n;
    L.dinv.alloc(n);
    // the Gershgorin bound stays on the device; setup() reads all levels' bounds in one copy
    PORSOL_LAUNCH(k_cheb_setup<T><<<div_up(n, TB), TB, 0, s>>>(n, L.P->slice_ptr.p, L.P->rowlen.p, L.P->diag.p, L.A, L.dinv.p,
                                                 s_gmax_.p + level, status_.p));
    PORSOL_CUDA(cudaGetLastError());
    L.half = o_.half_smoother && std::is_same<T, float>::value;
    // one thread per row without timing (the rule's choice): the smoother reads the SELL-32x4
    // copy only, written in place of the plain FP16 copy
    // (the x4 copy pads each row to a multiple of four entries; its offsets are 32-bit too)
    L.v4 = L.half && o_.layout4 && !o_.autotune && lanes_for(n, L.P->nent) == 1 &&
           (long long)L.P->nent + 96LL * L.P->nslices < (1LL << 31) - 1;
    const SellPattern& P = *L.P;
    L.c16 = false;
    if (L.v4) {
        L.sp4.alloc(size_t(P.nslices) + 1);
        s_width_.alloc(std::max(P.nslices, 1));
        PORSOL_LAUNCH(k_slice_groups<<<div_up(P.nslices, TB), TB, 0, s>>>(P.nslices, P.slice_ptr.p, s_width_.p));
        exclusive_scan(s, P.nslices, s_width_.p, L.sp4.p, L.sp4.p + P.nslices, scan_blocks_);
        // at most 3 padding entries per row: no host read of the exact size
        const size_t cap = size_t(P.nent) + 96 * size_t(P.nslices);
        L.ah4.alloc(cap);
        L.diagv.alloc(n);
        // 16-bit column offsets first; setup() checks the level's largest offset with the other
        // levels' bounds in one copy and rewrites the copy with 32-bit columns where it does not fit
        L.off4.alloc(cap);
        L.c16 = true;
        PORSOL_LAUNCH(k_scale_half4<T, short><<<div_up(P.nslices, TB / 32), TB, 0, s>>>(
            n, P.nslices, P.slice_ptr.p, P.col.p, P.diag.p, L.A, L.dinv.p, L.sp4.p, L.off4.p, L.ah4.p, L.diagv.p,
            s_maxoff_.p + level));
        PORSOL_CUDA(cudaGetLastError());
    } else if (L.half) {
        L.ah.alloc(size_t(L.P->nent));
        L.diagv.alloc(n);
        PORSOL_LAUNCH(k_scale_half<T><<<div_up(L.P->nslices, TB / 32), TB, 0, s>>>(
            n, L.P->slice_ptr.p, L.P->rowlen.p, L.P->diag.p, L.A, L.dinv.p, L.ah.p, L.diagv.p));
        PORSOL_CUDA(cudaGetLastError());
    }
    L.t.alloc(n);
    L.r.alloc(n);
    L.d0.alloc(n);
    L.d1.alloc(n);
    L.lanes = L.v4 ? 1 : tune_lanes(s, L);
    // coarse levels smoothed one thread per row on the plain layout (FP64 hierarchies): 16-bit column
    // offsets as the system matrix has them, when the level's couplings allow (checked in setup())
    if (level > 0) {
        SellPattern& O = L.own;
        O.off16.n = 0;   // a copy from an earlier setup is never used
        if (!L.half && !L.v4 && L.lanes == 1 && O.nent > 0) {
            O.off16.alloc(size_t(O.nent));
            PORSOL_LAUNCH(k_col_offsets<<<div_up(O.nslices, TB / 32), TB, 0, s>>>(n, O.nslices, O.slice_ptr.p,
                                                                                  O.col.p, O.off16.p,
                                                                                  s_maxoff_.p + level));
            PORSOL_CUDA(cudaGetLastError());
        }
    }
    // bulk-staged step: FP32 hierarchies on the level whose slice widths the host knows (the system
    // matrix), when every slice has at most four groups (18 KB of shared memory per 8 slices at 3)
    L.bulk_groups = 0;
    if (L.v4 && o_.bulk_stage && std::is_same<T, float>::value && P.h_slice_ptr.size() == size_t(P.nslices) + 1) {
        int gmax = 0;
        for (int sl = 0; sl < P.nslices; ++sl)
            gmax = std::max(gmax, (((P.h_slice_ptr[sl + 1] - P.h_slice_ptr[sl]) / 32) + 3) / 4);
        if (gmax >= 1 && gmax <= 4) L.bulk_groups = gmax;
    }
}

// Lane schedule autotuner: for a level shape not seen before, time one smoother step with 1, 2,
// 4, 8 and 16 lanes per row and keep the fastest.  Shapes are bucketed by value width, log2 of
// the row count and the mean padded row length, so nearby hierarchies (the next solve of an
// IMPES run, the next batch of sub-grids) reuse the choice without timing again.
template <class T>
int Amg<T>::tune_lanes(cudaStream_t s, Level& L)
{
    const int n = L.n;
    const int rule = lanes_for(n, L.P->nent);
    if (!o_.autotune || n < 1024) return rule;
    const int avg = int(std::lround(double(L.P->nent) / n));
    int lg = 0;
    while ((2LL << lg) <= n) ++lg;
    const long long key = ((long long)(L.half ? 2 : sizeof(T)) << 40) | ((long long)lg << 20) | (long long)avg;
    {
        std::lock_guard<std::mutex> lk(tune_mutex());
        auto it = tune_cache().find(key);
        if (it != tune_cache().end()) return it->second;
    }
    tune_stop_.alloc(1);
    tune_stop_.zero(s);
    L.d0.zero(s);
    L.r.zero(s);
    cudaEvent_t a, b;
    PORSOL_CUDA(cudaEventCreate(&a));
    PORSOL_CUDA(cudaEventCreate(&b));
    const SellPattern& P = *L.P;
    auto step = [&](int lanes) {
        const int nbk = div_up(n * lanes, TB);
        if (L.half) {
            PORSOL_LANES(lanes, PORSOL_LAUNCH((k_cheb_step<T, KL, __half, true><<<nbk, TB, 0, s>>>(
                                    n, P.slice_ptr.p, P.col.p, P.rowlen.p, L.ah.p, L.dinv.p, nullptr, L.d0.p, L.r.p,
                                    L.d1.p, L.t.p, T(0.5), T(0.5), 0, tune_stop_.p, nullptr))));
        } else {
            PORSOL_LANES(lanes, PORSOL_LAUNCH((k_cheb_step<T, KL, T, false><<<nbk, TB, 0, s>>>(
                                    n, P.slice_ptr.p, P.col.p, P.rowlen.p, L.A, L.dinv.p, nullptr, L.d0.p, L.r.p,
                                    L.d1.p, L.t.p, T(0.5), T(0.5), 0, tune_stop_.p, nullptr))));
        }
    };
    int best = rule;
    float best_ms = 1e30f;
    float rule_ms = 1e30f;
    for (int lanes : {1, 2, 4, 8, 16}) {
        step(lanes);   // warm-up
        PORSOL_CUDA(cudaEventRecord(a, s));
        for (int r = 0; r < 3; ++r) step(lanes);
        PORSOL_CUDA(cudaEventRecord(b, s));
        PORSOL_CUDA(cudaEventSynchronize(b));
        float ms = 0.f;
        PORSOL_CUDA(cudaEventElapsedTime(&ms, a, b));
        if (lanes == rule) rule_ms = ms;
        if (ms < best_ms) {
            best_ms = ms;
            best = lanes;
        }
    }
    if (best_ms > 0.9f * rule_ms) best = rule;   // keep the rule unless another schedule is clearly faster
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    PORSOL_CUDA(cudaGetLastError());
    std::lock_guard<std::mutex> lk(tune_mutex());
    tune_cache()[key] = best;
    return best;
}

template <class T>
void Amg<T>::build_coarse_solver(cudaStream_t s, const SellPattern& P, const T* A, int n)
{
    nc_ = n;
    DBuf<double>&D = s_D_, &Linv = s_Linv_;
    D.alloc(std::max<size_t>((size_t)n * n, 1));
    Linv.alloc(std::max<size_t>((size_t)n * n, 1));
    cinv_.alloc(std::max<size_t>((size_t)n * n, 1));
    if (n > 0) {
        PORSOL_LAUNCH(k_dense_from_sell<T><<<div_up(n, 128), 128, 0, s>>>(n, P.slice_ptr.p, P.col.p, P.rowlen.p, A, D.p));
        if (n <= DENSE_SMEM_N) {
            const int shm = n * n * int(sizeof(double));
            PORSOL_CUDA(cudaFuncSetAttribute(k_dense_gauss_jordan, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             DENSE_SMEM_N * DENSE_SMEM_N * int(sizeof(double))));
            PORSOL_LAUNCH(k_dense_gauss_jordan<<<1, 1024, shm, s>>>(n, D.p, cinv_.p, status_.p));
        } else {
            PORSOL_LAUNCH(k_dense_cholesky_inverse<<<1, 1024, 0, s>>>(n, D.p, Linv.p, cinv_.p, status_.p));
        }
    }
    PORSOL_CUDA(cudaGetLastError());
    const int st = read_int(s, status_.p);
    PORSOL_REQUIRE(st == 0, PORSOL_ERR_NONFINITE, "AMG: coarsest matrix is not positive definite");
}

// the next level takes the Galerkin product held in tmp_pat_ / tmp_val_
template <class T>
void Amg<T>::adopt_tmp(Level& next)
{
    std::swap(next.own.slice_ptr, tmp_pat_.slice_ptr);
    std::swap(next.own.col, tmp_pat_.col);
    std::swap(next.own.rowlen, tmp_pat_.rowlen);
    std::swap(next.own.diag, tmp_pat_.diag);
    next.own.n = tmp_pat_.n;
    next.own.nslices = tmp_pat_.nslices;
    next.own.nent = tmp_pat_.nent;
    std::swap(next.own_val, tmp_val_);
}

template <class T>
void Amg<T>::setup(cudaStream_t s, const SellPattern& P0, const T* A0, const AmgOpts& o)
{
    this->bump_generation();
    o_ = o;
    sizes_.clear();
    nnzs_.clear();
    status_.alloc(1);
    status_.zero(s);
    s_gmax_.alloc(size_t(std::max(o.max_levels, 1)));
    s_gmax_.zero(s);
    s_maxoff_.alloc(size_t(std::max(o.max_levels, 1)));
    s_maxoff_.zero(s);
    if (lv_.empty()) lv_.push_back(std::make_unique<Level>());
    nlev_ = 1;
    {
        Level& L0 = *lv_[0];
        L0.n = P0.n;
        L0.P = &P0;
        L0.A = A0;
    }
    sizes_.push_back(P0.n);
    nnzs_.push_back(P0.nent);
    while (lv_[nlev_ - 1]->n > o.coarse_target && nlev_ < o.max_levels) {
        Level& L = *lv_[nlev_ - 1];
        const int n = L.n;
        const SellPattern& P = *L.P;
        smoother_setup(s, L, nlev_ - 1);
        if (int(lv_.size()) <= nlev_) lv_.push_back(std::make_unique<Level>());
        Level& next = *lv_[nlev_];
        // first pairing round on this level's matrix; L.agg maps rows to the intermediate level
        aggregate_round(s, P, L.A, n, o_.round1_negative, L.agg);
        members(s, L.agg);
        galerkin(s, P, L.A, L.agg, tmp_pat_, tmp_val_);
        const int nc1 = L.agg.nc;
        if (nc1 > o.coarse_target) {
            // round 2 on the intermediate matrix: aggregates of about four rows
            aggregate_round(s, tmp_pat_, tmp_val_.p, nc1, o_.round2_negative, agg2_);
            members(s, agg2_);
            galerkin(s, tmp_pat_, tmp_val_.p, agg2_, next.own, next.own_val);
            PORSOL_LAUNCH(k_compose<<<div_up(n, TB), TB, 0, s>>>(n, L.agg.agg.p, agg2_.agg.p));
            L.agg.nc = agg2_.nc;
            if (nlev_ > 1 && n < o.round3_below && agg2_.nc > o.coarse_target) {
                // round 3 on the level just formed (coarse levels only)
                aggregate_round(s, next.own, next.own_val.p, agg2_.nc, o_.round2_negative, agg2_);
                members(s, agg2_);
                galerkin(s, next.own, next.own_val.p, agg2_, tmp_pat_, tmp_val_);
                adopt_tmp(next);
                PORSOL_LAUNCH(k_compose<<<div_up(n, TB), TB, 0, s>>>(n, L.agg.agg.p, agg2_.agg.p));
                L.agg.nc = agg2_.nc;
            }
            members(s, L.agg);
        } else {
            adopt_tmp(next);
        }
        PORSOL_CUDA(cudaGetLastError());
        next.n = L.agg.nc;
        next.P = &next.own;
        next.A = next.own_val.p;
        next.b.alloc(std::max(next.n, 1));
        next.x.alloc(std::max(next.n, 1));
        sizes_.push_back(next.n);
        nnzs_.push_back(next.own.nent);
        ++nlev_;
        if (next.n > 0.9 * n) break;   // coarsening stalled
    }
    // block-diagonal systems: each level's row -> block map and its slice flags (all iterating)
    for (int l = 0; l < nlev_; ++l) {
        Level& L = *lv_[size_t(l)];
        if (!blk0_) {
            L.blkp = nullptr;
            continue;
        }
        if (l == 0) {
            L.blkp = blk0_;
        } else {
            Level& F = *lv_[size_t(l - 1)];
            L.blk.alloc(std::max(L.n, 1));
            PORSOL_LAUNCH(k_level_blocks<<<div_up(L.n, TB), TB, 0, s>>>(L.n, F.agg.ptr.p, F.agg.idx.p, F.blkp, L.blk.p));
            L.blkp = L.blk.p;
        }
        L.act.alloc(size_t(std::max(L.P->nslices, 1)));
        PORSOL_CUDA(cudaMemsetAsync(L.act.p, 1, L.act.n, s));
    }
    PORSOL_CUDA(cudaGetLastError());
    // Chebyshev intervals of the smoothed levels and the x4 copies' largest column offsets (one
    // copy each for all levels)
    {
        std::vector<unsigned long long> gb(size_t(nlev_), 0ULL);
        std::vector<int> mo(size_t(nlev_), 0);
        PORSOL_CUDA(cudaMemcpyAsync(gb.data(), s_gmax_.p, sizeof(unsigned long long) * gb.size(),
                                    cudaMemcpyDeviceToHost, s));
        PORSOL_CUDA(cudaMemcpyAsync(mo.data(), s_maxoff_.p, sizeof(int) * mo.size(), cudaMemcpyDeviceToHost, s));
        PORSOL_CUDA(cudaStreamSynchronize(s));
        for (int l = 0; l + 1 < nlev_; ++l) {
            double gm;
            std::memcpy(&gm, &gb[size_t(l)], sizeof(gm));
            lv_[l]->lmax = gm > 0 ? gm : 1.0;
            Level& L = *lv_[l];
            if (l > 0 && L.own.off16.n != 0 && mo[size_t(l)] > 32767) L.own.off16.n = 0;   // offsets do not fit
            if (L.v4 && L.c16 && mo[size_t(l)] > 32767) {
                // couplings too far from the diagonal for 16-bit offsets: 32-bit columns
                const SellPattern& P = *L.P;
                L.col4.alloc(size_t(P.nent) + 96 * size_t(P.nslices));
                PORSOL_LAUNCH(k_scale_half4<T, int><<<div_up(P.nslices, TB / 32), TB, 0, s>>>(
                    L.n, P.nslices, P.slice_ptr.p, P.col.p, P.diag.p, L.A, L.dinv.p, L.sp4.p, L.col4.p, L.ah4.p,
                    L.diagv.p, nullptr));
                PORSOL_CUDA(cudaGetLastError());
                L.c16 = false;
            }
        }
    }
    // K-cycle vectors and scalars
    kcoef_.alloc(8 * size_t(std::max(nlev_, 1)));
    kcoef_.zero(s);
    kpart_.alloc(3 * size_t(stride_blocks(lv_[0]->n)));
    for (int l = 1; l < nlev_; ++l)
        if (k_level(l)) {
            Level& K = *lv_[l];
            for (DBuf<T>* v : {&K.kc1, &K.kc2, &K.kv1, &K.kv2, &K.kr2}) v->alloc(std::max(K.n, 1));
        }
    Level& C = *lv_[nlev_ - 1];
    PORSOL_REQUIRE(C.n <= 2048, PORSOL_ERR_BAD_ARG, "AMG: coarsening stalled above the dense-solve limit");
    build_coarse_solver(s, *C.P, C.A, C.n);
    const int st = read_int(s, status_.p);
    PORSOL_REQUIRE(st == 0, PORSOL_ERR_NONFINITE, "AMG setup: non-positive diagonal or missing diagonal entry");
}

template <class T>
int Amg<T>::solve_status(cudaStream_t s) const
{
    return status_.p ? read_int(s, status_.p) : 0;
}

// One Chebyshev application (degree o_.cheb_degree) on [lmax/30, lmax]:
//   from_zero: x = p(D^-1 A) D^-1 b;  otherwise from y = x0 (+ w P xc when xc is given).
template <class T>
void Amg<T>::chebyshev(cudaStream_t s, Level& L, const T* b, T* x, bool from_zero, const T* xc, const int* agg,
                       const int* stop, bool started)
{
    const int n = L.n;
    const int nb = div_up(n, TB);
    const SellPattern& P = *L.P;
    const double bmax = L.lmax, amin = L.lmax / 30.0;
    const double theta = 0.5 * (bmax + amin), delta = 0.5 * (bmax - amin);
    const double sigma = theta / delta;
    double rho = 1.0 / sigma;
    T* d = L.d0.p;
    T* dn = L.d1.p;
    const unsigned char* act = level_act(L);
    if (from_zero) {
        if (!started) chain(k_cheb_start0<T>, nb, TB, 0, s, n, L.dinv.p, b, L.r.p, d, T(1.0 / theta), stop, act);
    } else {
        // x holds the start vector (or the pre-smoothed t when xc is given; then x gets y)
        const T* t = xc ? L.t.p : x;
        const int nbk = div_up(n * L.lanes, TB);
        // levels smoothed one thread per row (the large ones): form y = t + w P xc first, so the
        // start's row dot gathers one vector instead of t, agg and xc (the same y, the same sums)
        if (xc && L.lanes == 1) {
            chain(k_prolong_add<T>, nb, TB, 0, s, n, t, xc, agg, T(o_.prolong), x, stop, act);
            t = x;
            xc = nullptr;
        }
        if (L.v4 && L.c16) {
            chain(k_cheb_start<T, -1, __half, true, short>, nb, TB, 0, s, n, L.sp4.p, L.off4.p, nullptr, L.ah4.p,
                L.dinv.p, b, x, nullptr, nullptr, T(o_.prolong), x, L.r.p, d, T(1.0 / theta), stop, act);
        } else if (L.v4) {
            chain(k_cheb_start<T, 0, __half, true>, nb, TB, 0, s, n, L.sp4.p, L.col4.p, nullptr, L.ah4.p, L.dinv.p, b,
                x, nullptr, nullptr, T(o_.prolong), x, L.r.p, d, T(1.0 / theta), stop, act);
        } else if (L.half) {
            PORSOL_LANES(L.lanes, chain(k_cheb_start<T, KL, __half, true>, nbk, TB, 0, s, n, P.slice_ptr.p, P.col.p,
                P.rowlen.p, L.ah.p, L.dinv.p, b, t, xc, agg, T(o_.prolong), x, L.r.p, d, T(1.0 / theta), stop, act));
        } else if (plain16(L)) {
            chain(k_cheb_start<T, 1, T, false, short>, nb, TB, 0, s, n, P.slice_ptr.p, P.off16.p, P.rowlen.p, L.A,
                L.dinv.p, b, t, xc, agg, T(o_.prolong), x, L.r.p, d, T(1.0 / theta), stop, act);
        } else {
            PORSOL_LANES(L.lanes, chain(k_cheb_start<T, KL, T, false>, nbk, TB, 0, s, n, P.slice_ptr.p, P.col.p,
                P.rowlen.p, L.A, L.dinv.p, b, t, xc, agg, T(o_.prolong), x, L.r.p, d, T(1.0 / theta), stop, act));
        }
    }
    const int deg = std::max(1, o_.cheb_degree);
    for (int k = 1; k <= deg; ++k) {
        const double rho1 = 1.0 / (2.0 * sigma - rho);
        const double c1 = rho1 * rho, c2 = 2.0 * rho1 / delta;
        const T* xin = (from_zero && k == 1) ? nullptr : x;
        // algorithmic bytes: matrix values + columns (16-bit offsets on c16 levels), d gathered
        // once, dinv (unscaled form only), r and x in, r/d/x out
        const double bytes = double(P.nent) * ((L.half ? 2 : sizeof(T)) +
                                               ((L.v4 && L.c16) || plain16(L) ? 2 : 4)) +
                             double(n) * sizeof(T) * ((xin ? 7 : 6) - (L.half ? 1 : 0));
        const bool prof_here = prof_ && prof_->on && &L == lv_[0].get();  // finest level only
        cudaEvent_t ev = nullptr;
        if (prof_here) prof_->begin(s, PK_CHEB, bytes, &ev);
        const int nbk = div_up(n * L.lanes, TB);
        if (L.bulk_groups > 0 && L.c16) {
            const int cap = 128 * L.bulk_groups;   // entries per slice
            const size_t shm = 128 + size_t(BULK_SLICES) * cap * 4;
            chain(k_cheb_step_bulk<T, short>, div_up(P.nslices, BULK_SLICES), BULK_SLICES * 32, shm, s, n, P.nslices,
                L.sp4.p, L.off4.p, L.ah4.p, xin, d, L.r.p, dn, x, T(c1), T(c2), k == deg ? 1 : 0, stop, cap,
                status_.p, 0u);
        } else if (L.bulk_groups > 0) {
            const int cap = 128 * L.bulk_groups;   // entries per slice
            const size_t shm = 128 + size_t(BULK_SLICES) * cap * 6;
            chain(k_cheb_step_bulk<T, int>, div_up(P.nslices, BULK_SLICES), BULK_SLICES * 32, shm, s, n, P.nslices,
                L.sp4.p, L.col4.p, L.ah4.p, xin, d, L.r.p, dn, x, T(c1), T(c2), k == deg ? 1 : 0, stop, cap,
                status_.p, 0u);
        } else if (L.v4 && L.c16) {
            chain(k_cheb_step<T, -1, __half, true, short>, nb, TB, 0, s, n, L.sp4.p, L.off4.p, nullptr, L.ah4.p,
                L.dinv.p, xin, d, L.r.p, dn, x, T(c1), T(c2), k == deg ? 1 : 0, stop, act);
        } else if (L.v4) {
            chain(k_cheb_step<T, 0, __half, true>, nb, TB, 0, s, n, L.sp4.p, L.col4.p, nullptr, L.ah4.p, L.dinv.p,
                xin, d, L.r.p, dn, x, T(c1), T(c2), k == deg ? 1 : 0, stop, act);
        } else if (L.half) {
            PORSOL_LANES(L.lanes, chain(k_cheb_step<T, KL, __half, true>, nbk, TB, 0, s, n, P.slice_ptr.p, P.col.p,
                P.rowlen.p, L.ah.p, L.dinv.p, xin, d, L.r.p, dn, x, T(c1), T(c2), k == deg ? 1 : 0, stop, act));
        } else if (plain16(L)) {
            chain(k_cheb_step<T, 1, T, false, short>, nb, TB, 0, s, n, P.slice_ptr.p, P.off16.p, P.rowlen.p, L.A,
                L.dinv.p, xin, d, L.r.p, dn, x, T(c1), T(c2), k == deg ? 1 : 0, stop, act);
        } else {
            PORSOL_LANES(L.lanes, chain(k_cheb_step<T, KL, T, false>, nbk, TB, 0, s, n, P.slice_ptr.p, P.col.p,
                P.rowlen.p, L.A, L.dinv.p, xin, d, L.r.p, dn, x, T(c1), T(c2), k == deg ? 1 : 0, stop, act));
        }
        if (prof_here) prof_->end(s, PK_CHEB, bytes, ev);
        rho = rho1;
        std::swap(d, dn);
    }
    PORSOL_CUDA(cudaGetLastError());
}

template <class T>
void Amg<T>::vcycle(cudaStream_t s, int l, const T* b, T* x, const int* stop, bool started)
{
    if (l == nlev_ - 1) {
        if (nc_ > 0)
            chain(k_dense_apply<T>, div_up(nc_, 8), 256, nc_ * sizeof(double), s, nc_, cinv_.p, b, x, stop,
                level_act(*lv_[size_t(l)]), lv_[size_t(l)]->blkp, level_act(*lv_[size_t(l)]) ? conv_ : nullptr);
        return;
    }
    Level& L = *lv_[l];
    Level& Nx = *lv_[l + 1];
    const int n = L.n;
    const int nb = div_up(n, TB);
    const SellPattern& P = *L.P;
    // pre-smoothing into t
    chebyshev(s, L, b, L.t.p, true, nullptr, nullptr, stop, started);
    for (int k = 1; k < o_.smooth_steps; ++k) chebyshev(s, L, b, L.t.p, false, nullptr, nullptr, stop);
    // restrict the residual
    if (L.v4 && L.c16) {
        chain(k_resid<T, -1, __half, true, short>, nb, TB, 0, s, n, L.sp4.p, L.off4.p, nullptr, L.ah4.p, L.diagv.p, b,
            L.t.p, L.r.p, stop, level_act(L));
    } else if (L.v4) {
        chain(k_resid<T, 0, __half, true>, nb, TB, 0, s, n, L.sp4.p, L.col4.p, nullptr, L.ah4.p, L.diagv.p, b, L.t.p,
            L.r.p, stop, level_act(L));
    } else if (L.half) {
        PORSOL_LANES(L.lanes, chain(k_resid<T, KL, __half, true>, div_up(n * L.lanes, TB), TB, 0, s, n, P.slice_ptr.p,
            P.col.p, P.rowlen.p, L.ah.p, L.diagv.p, b, L.t.p, L.r.p, stop, level_act(L)));
    } else if (plain16(L)) {
        chain(k_resid<T, 1, T, false, short>, nb, TB, 0, s, n, P.slice_ptr.p, P.off16.p, P.rowlen.p, L.A, L.diagv.p,
            b, L.t.p, L.r.p, stop, level_act(L));
    } else {
        PORSOL_LANES(L.lanes, chain(k_resid<T, KL, T, false>, div_up(n * L.lanes, TB), TB, 0, s, n, P.slice_ptr.p,
            P.col.p, P.rowlen.p, L.A, L.diagv.p, b, L.t.p, L.r.p, stop, level_act(L)));
    }
    // the coarse level's cycle starts with a Chebyshev start from zero on Nx.b (its first cycle
    // under a K-cycle): done here, in the restriction; the coarsest level solves directly
    const bool fuse = l + 1 < nlev_ - 1;
    if (fuse)
        chain(k_restrict_start0<T>, div_up(Nx.n, TB), TB, 0, s, Nx.n, L.agg.ptr.p, L.agg.idx.p, L.r.p, Nx.b.p,
            Nx.dinv.p, Nx.r.p, Nx.d0.p, T(cheb_inv_theta(Nx)), stop, level_act(Nx));
    else
        chain(k_restrict<T>, div_up(Nx.n, TB), TB, 0, s, Nx.n, L.agg.ptr.p, L.agg.idx.p, L.r.p, Nx.b.p, stop,
            level_act(Nx));
    if (k_level(l + 1)) kcycle(s, l + 1, Nx.b.p, Nx.x.p, stop, fuse);
    else vcycle(s, l + 1, Nx.b.p, Nx.x.p, stop, fuse);
    // post-smoothing from t + w P xc
    chebyshev(s, L, b, x, false, Nx.x.p, L.agg.agg.p, stop);
    for (int k = 1; k < o_.smooth_steps; ++k) chebyshev(s, L, b, x, false, nullptr, nullptr, stop);
    PORSOL_CUDA(cudaGetLastError());
}

// K-cycle on level l (Notay and Vassilevski's Krylov-accelerated multigrid cycle): the level's
// system A_l x = b is solved by two flexible-CG steps whose preconditioner B is the cycle of
// level l (itself recursive), instead of one application of B.  Every scalar stays on the device,
// so the cycle is captured into the CG iteration's graph with the rest.
template <class T>
void Amg<T>::kcycle(cudaStream_t s, int l, const T* b, T* x, const int* stop, bool started)
{
    Level& L = *lv_[l];
    const int n = L.n, nb = div_up(n, TB);
    const SellPattern& P = *L.P;
    const int nd = stride_blocks(n);
    double* c = kcoef_.p + 8 * l;
    vcycle(s, l, b, L.kc1.p, stop, started);
    chain(k_lv_spmv<T>, nb, TB, 0, s, n, P.slice_ptr.p, P.col.p, L.A, L.kc1.p, L.kv1.p, stop);
    chain(k_kdots<T>, nd, 256, 0, s, n, L.kc1.p, L.kv1.p, L.kc1.p, b, nullptr, nullptr, kpart_.p, stop);
    chain(k_kfinish, 1, 1024, 0, s, nd, kpart_.p, c, 1, stop);
    chain(k_kresid<T>, nb, TB, 0, s, n, b, L.kv1.p, c, L.kr2.p, stop);
    vcycle(s, l, L.kr2.p, L.kc2.p, stop);
    chain(k_lv_spmv<T>, nb, TB, 0, s, n, P.slice_ptr.p, P.col.p, L.A, L.kc2.p, L.kv2.p, stop);
    chain(k_kdots<T>, nd, 256, 0, s, n, L.kc2.p, L.kv1.p, L.kc2.p, L.kv2.p, L.kc2.p, L.kr2.p, kpart_.p, stop);
    chain(k_kfinish, 1, 1024, 0, s, nd, kpart_.p, c, 2, stop);
    chain(k_kcombine<T>, nb, TB, 0, s, n, L.kc1.p, L.kc2.p, c, x, stop);
    PORSOL_CUDA(cudaGetLastError());
}

// Mirrors the launches of vcycle() and chebyshev(): the algorithmic bytes of each kernel (see the
// declaration).
template <class T>
double Amg<T>::apply_bytes(std::vector<double>* per_level) const
{
    if (per_level) per_level->assign(size_t(nlev_), 0.0);
    return nlev_ > 0 ? cycle_bytes(0, per_level) : 0.0;
}

// bytes of one cycle started on level l (its own kernels, the coarse correction below it)
template <class T>
double Amg<T>::cycle_bytes(int l, std::vector<double>* per_level, bool started) const
{
    const double sx = sizeof(T);
    double b = 0.0;
    if (l == nlev_ - 1) {
        b = double(nc_) * nc_ * 8.0 + 2.0 * nc_ * sx;   // dense inverse, b in, x out
        if (per_level) (*per_level)[size_t(l)] += b;
        return b;
    }
    const Level& L = *lv_[l];
    const double n = L.n, nc = lv_[l + 1]->n;
    const double vb = L.half ? 2.0 : sx, cb = ((L.v4 && L.c16) || plain16(L)) ? 2.0 : 4.0;
    const double mat = double(L.P->nent) * (vb + cb);
    const int deg = std::max(1, o_.cheb_degree);
    // Chebyshev steps of one application: the first from x = 0 after start0 has no x_in
    auto steps = [&](bool from_zero) {
        double t = 0.0;
        for (int k = 1; k <= deg; ++k) {
            const bool xin = !(from_zero && k == 1);
            t += mat + n * sx * (5.0 + (xin ? 1.0 : 0.0) + (L.half ? 0.0 : 1.0));
        }
        return t;
    };
    const double start = mat + 5.0 * n * sx;           // t gathered, dinv, b in; r, d out
    // pre-smoothing from zero: dinv (and b unless the restriction fused the start) in; r, d out
    b += (started ? 3.0 : 4.0) * n * sx + steps(true);
    b += (o_.smooth_steps - 1) * (start + steps(false));
    b += mat + n * sx * (L.half ? 4.0 : 3.0);            // residual
    b += n * (sx + 4.0) + nc * (4.0 + sx);               // restriction
    const bool fuse = l + 1 < nlev_ - 1;                 // the coarse start is done by the restriction
    if (L.lanes == 1)                                    // post-smoothing from t + w P xc
        b += n * (2.0 * sx + 4.0) + nc * sx + start;
    else
        b += start + n * (sx + 4.0) + nc * sx;
    b += steps(false);
    b += (o_.smooth_steps - 1) * (start + steps(false));
    if (per_level) (*per_level)[size_t(l)] += b;
    double below;
    if (k_level(l + 1)) {
        // two cycles of level l + 1, two products with its FP32/FP64 matrix, the dots, r2 and x
        const Level& C = *lv_[l + 1];
        const double kb = 2.0 * (double(C.P->nent) * (sx + 4.0) + 2.0 * nc * sx) + 4.0 * nc * sx +
                          6.0 * nc * sx + 3.0 * nc * sx + 3.0 * nc * sx;
        if (per_level) (*per_level)[size_t(l + 1)] += kb;
        below = kb + cycle_bytes(l + 1, per_level, fuse) + cycle_bytes(l + 1, per_level);
    } else {
        below = cycle_bytes(l + 1, per_level, fuse);
    }
    return b + below;
}

template <class T>
void Amg<T>::set_block_state(const int* conv)
{
    if (conv != conv_) {
        conv_ = conv;
        this->bump_generation();   // the captured cycle's kernels take other arguments
    }
}

template <class T>
void Amg<T>::apply(cudaStream_t s, const T* r, T* z, const int* stop)
{
    const bool prof_here = prof_ && prof_->on;
    ChainPause plain(prof_here);   // events between the kernels time each one
    cudaEvent_t ev = nullptr;
    if (prof_here) prof_->begin(s, PK_VCYCLE, 0.0, &ev);
    if (conv_ && nlev_ > 0 && lv_[0]->blkp)
        for (int l = 0; l < nlev_; ++l) {
            const Level& L = *lv_[size_t(l)];
            const int ns = L.P->nslices;
            chain(k_slice_active, div_up(ns, TB / 32), TB, 0, s, L.n, ns, L.blkp, conv_, L.act.p, stop);
        }
    vcycle(s, 0, r, z, stop);
    if (prof_here) prof_->end(s, PK_VCYCLE, 0.0, ev);
}

template class Amg<double>;
template class Amg<float>;

// Self-test of k_cheb_step_bulk and of its bounded wait: one step (c1 = 1/2, c2 = 1/4, from x = 0,
// final) on a 64-row system of two slices with one group each; row i holds the FP16 values
// 1/4, 1/2, 3/4, 1 at columns i, (i+1)%64, (i+5)%64, (i+17)%64 and d_j = 1 + j/64, r = 2 (every
// product and sum exact in FP32).  expire adds 16 bytes to what each warp's barrier waits for, so
// every wait runs out.  Returns the kernel's status bits; r, d, x receive the 64 outputs.
int bulk_step_selftest(bool expire, float* r_host, float* d_host, float* x_host)
{
    const int n = 64, ns = 2, cap = 128;
    std::vector<int> sp4 = {0, 128, 256}, col4(256);
    std::vector<__half> a4(256);
    std::vector<float> din(n), r0(n, 2.0f);
    const int off[4] = {0, 1, 5, 17};
    for (int i = 0; i < n; ++i) {
        din[i] = 1.0f + float(i) / 64.0f;
        for (int t = 0; t < 4; ++t) {
            const int dst = sp4[i / 32] + 4 * (i % 32) + t;
            col4[dst] = (i + off[t]) % n;
            a4[dst] = __float2half_rn(0.25f * float(t + 1));
        }
    }
    cudaStream_t s = nullptr;
    DBuf<int> dsp, dcol, dstop, dstat;
    DBuf<__half> da;
    DBuf<float> dd, dr, ddn, dx;
    dsp.upload(sp4, s);
    dcol.upload(col4, s);
    da.upload(a4, s);
    dd.upload(din, s);
    dr.upload(r0, s);
    ddn.alloc(n);
    dx.alloc(n);
    dstop.alloc(1);
    dstop.zero(s);
    dstat.alloc(1);
    dstat.zero(s);
    const size_t shm = 128 + size_t(BULK_SLICES) * cap * 6;
    PORSOL_LAUNCH((k_cheb_step_bulk<float, int><<<1, BULK_SLICES * 32, shm, s>>>(
        n, ns, dsp.p, dcol.p, da.p, nullptr, dd.p, dr.p, ddn.p, dx.p, 0.5f, 0.25f, 1, dstop.p, cap, dstat.p,
        expire ? 16u : 0u)));
    PORSOL_CUDA(cudaGetLastError());
    const int st = read_int(s, dstat.p);
    dr.download(r_host, n, s);
    ddn.download(d_host, n, s);
    dx.download(x_host, n, s);
    PORSOL_CUDA(cudaStreamSynchronize(s));
    return st;
}

}  // namespace porsol
