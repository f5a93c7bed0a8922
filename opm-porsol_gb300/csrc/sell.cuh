// sell.cuh -- row dot products of SELL-32 matrices with memory-level parallelism.
//
// Row r of a SELL-32 matrix: entries t = 0..w-1 at slice_ptr[r/32] + 32 t + r%32 (w = slice
// width; padding entries carry col = r, val = 0).  Each gather x[col[k]] depends on the load
// of col[k]; issuing the column and value loads of four entries before their four gathers
// keeps four independent memory chains in flight per thread.
#pragma once

#include <cuda_fp16.h>

namespace porsol {

// Column of stored entry k of row r: the column itself (int), or its 16-bit offset from the row
// (short; systems whose couplings all lie within 32767 rows of the diagonal).
__device__ __forceinline__ int sell_col(const int* __restrict__ col, int k, int) { return col[k]; }
__device__ __forceinline__ int sell_col(const short* __restrict__ off, int k, int r) { return r + off[k]; }

// sum_t val[k_t] * xf(col[k_t]) accumulated in Acc; xf maps a column index to the vector value.
template <class Acc, class TV, class XF, class CI = int>
__device__ __forceinline__ Acc sell_dot(const int* __restrict__ sp, const CI* __restrict__ col,
                                        const TV* __restrict__ val, int r, XF xf)
{
    const int s = r >> 5, lane = r & 31;
    const int b = sp[s], w = (sp[s + 1] - b) >> 5;
    Acc acc = Acc(0);
    int k = b + lane;
    int t = 0;
    for (; t + 4 <= w; t += 4, k += 128) {
        const int c0 = sell_col(col, k, r), c1 = sell_col(col, k + 32, r), c2 = sell_col(col, k + 64, r),
                  c3 = sell_col(col, k + 96, r);
        const Acc v0 = Acc(val[k]), v1 = Acc(val[k + 32]), v2 = Acc(val[k + 64]), v3 = Acc(val[k + 96]);
        const Acc x0 = Acc(xf(c0)), x1 = Acc(xf(c1)), x2 = Acc(xf(c2)), x3 = Acc(xf(c3));
        acc += v0 * x0;
        acc += v1 * x1;
        acc += v2 * x2;
        acc += v3 * x3;
    }
    for (; t < w; ++t, k += 32) acc += Acc(val[k]) * Acc(xf(sell_col(col, k, r)));
    return acc;
}

// The same dot product with K lanes per row (K = 2..32, a power of two; the K lanes of a row are
// consecutive in the warp).  Lane q sums entries t = q, q + K, ... below rowlen[r] (padding is
// skipped); the partial sums are combined with a fixed butterfly, so every lane of the group
// gets the same, deterministic total.  All 32 lanes of the warp must call it (valid = false for
// lanes past the last row).  Coarse AMG levels use it: their rows are long (30-60 entries) and
// few, and one thread per row would walk them serially.
template <int K, class Acc, class TV, class XF>
__device__ __forceinline__ Acc sell_dot_lanes(const int* __restrict__ sp, const int* __restrict__ col,
                                              const TV* __restrict__ val, const int* __restrict__ rowlen, int r,
                                              int q, bool valid, XF xf)
{
    Acc acc = Acc(0);
    if (valid) {
        const int b = sp[r >> 5] + (r & 31);
        const int len = rowlen[r];
        int t = q;
        for (; t + K < len; t += 2 * K) {
            const int k0 = b + 32 * t, k1 = b + 32 * (t + K);
            const int c0 = col[k0], c1 = col[k1];
            const Acc v0 = Acc(val[k0]), v1 = Acc(val[k1]);
            const Acc x0 = Acc(xf(c0)), x1 = Acc(xf(c1));
            acc += v0 * x0;
            acc += v1 * x1;
        }
        if (t < len) {
            const int k0 = b + 32 * t;
            acc += Acc(val[k0]) * Acc(xf(col[k0]));
        }
    }
#pragma unroll
    for (int o = K / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    return acc;
}

// Row dot product on the SELL-32x4 layout with FP16 values (entry t of row r at
// sp4[r/32] + 128 (t/4) + 4 (r%32) + t%4; the slice's group count is uniform in the warp): the
// columns and values of GB groups (4 GB entries) are loaded as 16- and 8-byte vectors before their
// gathers, then the products are added in entry order -- the same sequential sum as sell_dot on the
// plain layout (the extra padding adds exact zeros).  GB = 1 keeps the smoother kernels at 32
// registers (full occupancy); on the finest level of the 1M-cell system that beat 2-4 groups per
// round (40-64 registers) by 7 % of the whole solve.
template <class Acc, class XF, int GB = 1>
__device__ __forceinline__ Acc sell4_dot(const int* __restrict__ sp4, const int* __restrict__ col4,
                                         const __half* __restrict__ a4, int r, XF xf)
{
    const int s = r >> 5, lane = r & 31;
    const int b = sp4[s], G = (sp4[s + 1] - b) >> 7;
    const int4* cp = reinterpret_cast<const int4*>(col4 + b) + lane;
    const uint2* vp = reinterpret_cast<const uint2*>(a4 + b) + lane;
    Acc acc = Acc(0);
    for (int g0 = 0; g0 < G; g0 += GB) {
        int4 c[GB];
        uint2 h[GB];
#pragma unroll
        for (int u = 0; u < GB; ++u)
            if (g0 + u < G) {
                c[u] = __ldg(cp + 32 * (g0 + u));
                h[u] = __ldg(vp + 32 * (g0 + u));
            }
        Acc x[4 * GB];
#pragma unroll
        for (int u = 0; u < GB; ++u)
            if (g0 + u < G) {
                x[4 * u + 0] = Acc(xf(c[u].x));
                x[4 * u + 1] = Acc(xf(c[u].y));
                x[4 * u + 2] = Acc(xf(c[u].z));
                x[4 * u + 3] = Acc(xf(c[u].w));
            }
#pragma unroll
        for (int u = 0; u < GB; ++u)
            if (g0 + u < G) {
                const float2 v01 = __half22float2(*reinterpret_cast<const __half2*>(&h[u].x));
                const float2 v23 = __half22float2(*reinterpret_cast<const __half2*>(&h[u].y));
                acc += Acc(v01.x) * x[4 * u + 0];
                acc += Acc(v01.y) * x[4 * u + 1];
                acc += Acc(v23.x) * x[4 * u + 2];
                acc += Acc(v23.y) * x[4 * u + 3];
            }
    }
    return acc;
}

// The same row dot product on the SELL-32x4 layout with 16-bit column offsets: entry t of row r
// stores col - r as a signed 16-bit value (levels whose couplings all lie within 32767 rows of the
// diagonal, which the internal face numbering gives the finest levels), so a group's four columns
// come in one 8-byte load.  Same sum, in the same order, as sell4_dot.
template <class Acc, class XF>
__device__ __forceinline__ Acc sell4_dot16(const int* __restrict__ sp4, const short* __restrict__ off4,
                                           const __half* __restrict__ a4, int r, XF xf)
{
    const int s = r >> 5, lane = r & 31;
    const int b = sp4[s], G = (sp4[s + 1] - b) >> 7;
    const short4* cp = reinterpret_cast<const short4*>(off4 + b) + lane;
    const uint2* vp = reinterpret_cast<const uint2*>(a4 + b) + lane;
    Acc acc = Acc(0);
    for (int g = 0; g < G; ++g) {
        const short4 c = __ldg(cp + 32 * g);
        const uint2 h = __ldg(vp + 32 * g);
        const Acc x0 = Acc(xf(r + c.x)), x1 = Acc(xf(r + c.y)), x2 = Acc(xf(r + c.z)), x3 = Acc(xf(r + c.w));
        const float2 v01 = __half22float2(*reinterpret_cast<const __half2*>(&h.x));
        const float2 v23 = __half22float2(*reinterpret_cast<const __half2*>(&h.y));
        acc += Acc(v01.x) * x0;
        acc += Acc(v01.y) * x1;
        acc += Acc(v23.x) * x2;
        acc += Acc(v23.y) * x3;
    }
    return acc;
}

}  // namespace porsol
