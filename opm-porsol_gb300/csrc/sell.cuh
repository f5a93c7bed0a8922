// sell.cuh -- row dot products of SELL-32 matrices with memory-level parallelism.
//
// Row r of a SELL-32 matrix: entries t = 0..w-1 at slice_ptr[r/32] + 32 t + r%32 (w = slice
// width; padding entries carry col = r, val = 0).  Each gather x[col[k]] depends on the load
// of col[k]; issuing the column and value loads of four entries before their four gathers
// keeps four independent memory chains in flight per thread.
#pragma once

namespace porsol {

// sum_t val[k_t] * xf(col[k_t]) accumulated in Acc; xf maps a column index to the vector value.
template <class Acc, class TV, class XF>
__device__ __forceinline__ Acc sell_dot(const int* __restrict__ sp, const int* __restrict__ col,
                                        const TV* __restrict__ val, int r, XF xf)
{
    const int s = r >> 5, lane = r & 31;
    const int b = sp[s], w = (sp[s + 1] - b) >> 5;
    Acc acc = Acc(0);
    int k = b + lane;
    int t = 0;
    for (; t + 4 <= w; t += 4, k += 128) {
        const int c0 = col[k], c1 = col[k + 32], c2 = col[k + 64], c3 = col[k + 96];
        const Acc v0 = Acc(val[k]), v1 = Acc(val[k + 32]), v2 = Acc(val[k + 64]), v3 = Acc(val[k + 96]);
        const Acc x0 = Acc(xf(c0)), x1 = Acc(xf(c1)), x2 = Acc(xf(c2)), x3 = Acc(xf(c3));
        acc += v0 * x0;
        acc += v1 * x1;
        acc += v2 * x2;
        acc += v3 * x3;
    }
    for (; t < w; ++t, k += 32) acc += Acc(val[k]) * Acc(xf(col[k]));
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

}  // namespace porsol
