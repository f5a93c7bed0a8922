// k_amg.cu -- aggregation AMG: pairwise matching, Galerkin products, V-cycle kernels,
// FP64 dense coarsest-level solve.  Every reduction is ordered (no floating-point
// atomics), so the hierarchy and the preconditioner are run-to-run reproducible.
#include <algorithm>
#include <cmath>

#include "amg.h"

namespace porsol {

namespace {

constexpr int TB = 256;
constexpr int GAL_CAP = 160;   // max entries of a merged coarse row

__device__ __forceinline__ int slot_of(const int* sp, int r, int t) { return sp[r >> 5] + t * 32 + (r & 31); }

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
    // single block: sequential chunks, exclusive in place
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

// ---------------- matching ----------------
template <class T>
__global__ void k_diag_vals(int n, const int* __restrict__ diag, const T* __restrict__ A, double* __restrict__ d)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = fabs(double(A[diag[i]]));
}

template <class T>
__global__ void k_pick(int n, const int* __restrict__ sp, const int* __restrict__ col, const int* __restrict__ rowlen,
                       const T* __restrict__ A, const double* __restrict__ d, const int* __restrict__ state,
                       int* __restrict__ best, double theta)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (state[i] != 0) {
        best[i] = -1;
        return;
    }
    const double di = d[i];
    double bs = -1.0;
    int bj = -1;
    for (int t = 0; t < rowlen[i]; ++t) {
        const int k = slot_of(sp, i, t);
        const int j = col[k];
        if (j == i || state[j] != 0) continue;
        const double s = fabs(double(A[k])) / sqrt(di * d[j]);
        if (s >= theta && (s > bs || (s == bs && j < bj))) {
            bs = s;
            bj = j;
        }
    }
    best[i] = bj;
}

__global__ void k_match(int n, int* __restrict__ state, const int* __restrict__ best, int* __restrict__ partner)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || state[i] != 0) return;
    const int j = best[i];
    if (j >= 0 && best[j] == i) {
        state[i] = 1;
        partner[i] = j;
    }
}

__global__ void k_rep_flag(int n, const int* __restrict__ state, const int* __restrict__ partner, int* __restrict__ flag)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    flag[i] = (state[i] == 0 || i < partner[i]) ? 1 : 0;
}

__global__ void k_assign(int n, const int* __restrict__ state, const int* __restrict__ partner,
                         const int* __restrict__ flag, const int* __restrict__ cidx, int* __restrict__ agg,
                         int2* __restrict__ kids)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (flag[i]) {
        const int I = cidx[i];
        agg[i] = I;
        kids[I] = make_int2(i, state[i] ? partner[i] : -1);
    } else {
        agg[i] = cidx[partner[i]];
    }
}

// ---------------- Galerkin products over pairs ----------------
// Merge the rows of the (<=2) children, mapping columns through agg; sorted unique keys.
template <class T>
__device__ int merge_rows(const int* __restrict__ sp, const int* __restrict__ col, const int* __restrict__ rowlen,
                          const T* __restrict__ A, const int* __restrict__ agg, int2 kid, int* kc, double* kv,
                          bool* overflow)
{
    int m = 0;
    const int ch[2] = {kid.x, kid.y};
    for (int q = 0; q < 2; ++q) {
        const int r = ch[q];
        if (r < 0) continue;
        for (int t = 0; t < rowlen[r]; ++t) {
            const int k = slot_of(sp, r, t);
            const int c = agg[col[k]];
            const double v = double(A[k]);
            // insertion into sorted kc[0..m)
            int pos = m;
            while (pos > 0 && kc[pos - 1] > c) --pos;
            if (pos > 0 && kc[pos - 1] == c) {
                kv[pos - 1] += v;
                continue;
            }
            if (m >= GAL_CAP) {
                *overflow = true;
                continue;
            }
            for (int u = m; u > pos; --u) {
                kc[u] = kc[u - 1];
                kv[u] = kv[u - 1];
            }
            kc[pos] = c;
            kv[pos] = v;
            ++m;
        }
    }
    return m;
}

template <class T>
__global__ void k_gal_count(int nc, const int* __restrict__ sp, const int* __restrict__ col,
                            const int* __restrict__ rowlen, const T* __restrict__ A, const int* __restrict__ agg,
                            const int2* __restrict__ kids, int* __restrict__ rowlen_c, int* status)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= nc) return;
    int kc[GAL_CAP];
    double kv[GAL_CAP];
    bool of = false;
    const int m = merge_rows(sp, col, rowlen, A, agg, kids[I], kc, kv, &of);
    if (of) atomicOr(status, ST_BAD_INDEX);
    rowlen_c[I] = m;
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
__global__ void k_gal_fill(int nc, const int* __restrict__ sp, const int* __restrict__ col,
                           const int* __restrict__ rowlen, const T* __restrict__ A, const int* __restrict__ agg,
                           const int2* __restrict__ kids, const int* __restrict__ sp_c, int* __restrict__ col_c,
                           T* __restrict__ val_c, int* __restrict__ diag_c)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= nc) return;
    int kc[GAL_CAP];
    double kv[GAL_CAP];
    bool of = false;
    const int m = merge_rows(sp, col, rowlen, A, agg, kids[I], kc, kv, &of);
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

// padding rows of the last slice beyond nc
__global__ void k_pad_tail(int nc, int nslices, const int* __restrict__ sp_c, int* __restrict__ col_c,
                           void* val_c_raw, int elem)
{
    const int lane = threadIdx.x;
    const int s = nslices - 1;
    const int r = s * 32 + lane;
    if (r < nc) return;
    const int w = (sp_c[s + 1] - sp_c[s]) >> 5;
    for (int t = 0; t < w; ++t) {
        const int k = sp_c[s] + t * 32 + lane;
        col_c[k] = 0;
        if (elem == 8) ((double*)val_c_raw)[k] = 0.0;
        else ((float*)val_c_raw)[k] = 0.0f;
    }
}

template <class T>
__global__ void k_l1_dinv(int n, const int* __restrict__ sp, const int* __restrict__ rowlen, const T* __restrict__ A,
                          T* __restrict__ dinv, int* status)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int t = 0; t < rowlen[i]; ++t) s += fabs(double(A[slot_of(sp, i, t)]));
    if (!(s > 0.0) || !isfinite(s)) {
        atomicOr(status, ST_NONFINITE);
        s = 1.0;
    }
    dinv[i] = T(1.0 / s);
}

__global__ void k_compose(int n, int* __restrict__ agg1, const int* __restrict__ agg2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) agg1[i] = agg2[agg1[i]];
}

__global__ void k_kids4(int nc2, const int2* __restrict__ kids2, const int2* __restrict__ kids1, int4* __restrict__ out)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= nc2) return;
    int v[4] = {-1, -1, -1, -1};
    int m = 0;
    const int2 a = kids2[I];
    const int mids[2] = {a.x, a.y};
    for (int q = 0; q < 2; ++q) {
        if (mids[q] < 0) continue;
        const int2 b = kids1[mids[q]];
        if (b.x >= 0) v[m++] = b.x;
        if (b.y >= 0) v[m++] = b.y;
    }
    // sort ascending (m <= 4), -1 last
    for (int p = 1; p < m; ++p) {
        const int key = v[p];
        int q = p - 1;
        while (q >= 0 && v[q] > key) {
            v[q + 1] = v[q];
            --q;
        }
        v[q + 1] = key;
    }
    out[I] = make_int4(v[0], v[1], v[2], v[3]);
}

__global__ void k_kids2to4(int nc, const int2* __restrict__ k2, int4* __restrict__ out)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I < nc) out[I] = make_int4(k2[I].x, k2[I].y, -1, -1);
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
    // Linv: column j by thread j
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

template <class T>
__global__ void k_dense_apply(int n, const double* __restrict__ Dinv, const T* __restrict__ b, T* __restrict__ x,
                              const int* stop)
{
    if (*stop) return;
    extern __shared__ double sb[];
    for (int j = threadIdx.x; j < n; j += blockDim.x) sb[j] = double(b[j]);
    __syncthreads();
    // one warp per row
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int i = warp; i < n; i += nw) {
        double s = 0.0;
        for (int j = lane; j < n; j += 32) s += Dinv[(size_t)i * n + j] * sb[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) x[i] = T(s);
    }
}

// ---------------- V-cycle kernels ----------------
template <class T>
__global__ void k_jacobi0(int n, const T* __restrict__ dinv, const T* __restrict__ b, T* __restrict__ x,
                          const int* stop)
{
    if (*stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = dinv[i] * b[i];
}

// xo = x + dinv (b - A x)
template <class T>
__global__ void k_jacobi(int n, const int* __restrict__ sp, const int* __restrict__ col, const T* __restrict__ A,
                         const T* __restrict__ dinv, const T* __restrict__ b, const T* __restrict__ x,
                         T* __restrict__ xo, const int* stop)
{
    if (*stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = i >> 5, lane = i & 31;
    const int base = sp[s], w = (sp[s + 1] - base) >> 5;
    T acc = 0;
    int k = base + lane;
    for (int t = 0; t < w; ++t, k += 32) acc += A[k] * x[col[k]];
    xo[i] = x[i] + dinv[i] * (b[i] - acc);
}

// r = b - A x
template <class T>
__global__ void k_resid(int n, const int* __restrict__ sp, const int* __restrict__ col, const T* __restrict__ A,
                        const T* __restrict__ b, const T* __restrict__ x, T* __restrict__ r, const int* stop)
{
    if (*stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = i >> 5, lane = i & 31;
    const int base = sp[s], w = (sp[s + 1] - base) >> 5;
    T acc = 0;
    int k = base + lane;
    for (int t = 0; t < w; ++t, k += 32) acc += A[k] * x[col[k]];
    r[i] = b[i] - acc;
}

template <class T>
__global__ void k_restrict(int nc, const int4* __restrict__ kids, const T* __restrict__ r, T* __restrict__ bc,
                           const int* stop)
{
    if (*stop) return;
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= nc) return;
    const int4 k = kids[I];
    T s = r[k.x];
    if (k.y >= 0) s += r[k.y];
    if (k.z >= 0) s += r[k.z];
    if (k.w >= 0) s += r[k.w];
    bc[I] = s;
}

// Post-smoothing fused with the prolongation: with y = t + w P xc,
//   x = y + dinv (b - A y)
template <class T>
__global__ void k_prolong_smooth(int n, const int* __restrict__ sp, const int* __restrict__ col,
                                 const T* __restrict__ A, const T* __restrict__ dinv, const T* __restrict__ b,
                                 const T* __restrict__ t, const T* __restrict__ xc, const int* __restrict__ agg,
                                 T wp, T* __restrict__ x, const int* stop)
{
    if (*stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = i >> 5, lane = i & 31;
    const int base = sp[s], w = (sp[s + 1] - base) >> 5;
    T acc = 0;
    int k = base + lane;
    for (int q = 0; q < w; ++q, k += 32) {
        const int j = col[k];
        acc += A[k] * (t[j] + wp * xc[agg[j]]);
    }
    const T yi = t[i] + wp * xc[agg[i]];
    x[i] = yi + dinv[i] * (b[i] - acc);
}

template <class T>
__global__ void k_prolong(int n, const int* __restrict__ agg, const T* __restrict__ xc, T wp, T* __restrict__ x,
                          const int* stop)
{
    if (*stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] += wp * xc[agg[i]];
}

template <class T>
__global__ void k_copy(int n, const T* __restrict__ a, T* __restrict__ b, const int* stop)
{
    if (*stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[i];
}

int read_int(cudaStream_t s, const int* d)
{
    int v = 0;
    PORSOL_CUDA(cudaMemcpyAsync(&v, d, sizeof(int), cudaMemcpyDeviceToHost, s));
    PORSOL_CUDA(cudaStreamSynchronize(s));
    return v;
}

}  // namespace

void exclusive_scan(cudaStream_t s, int n, const int* in, int* out, int* total_dev, DBuf<int>& scratch)
{
    const int nb = std::max(1, div_up(n, 1024));
    if ((int)scratch.n < nb) scratch.alloc(nb);
    if (n > 0) k_scan_block<<<nb, 1024, 0, s>>>(n, in, out, scratch.p);
    else PORSOL_CUDA(cudaMemsetAsync(scratch.p, 0, sizeof(int), s));
    k_scan_sums<<<1, 1024, 0, s>>>(n > 0 ? nb : 1, scratch.p, total_dev);
    if (n > 0) k_scan_add<<<nb, 1024, 0, s>>>(n, out, scratch.p);
    PORSOL_CUDA(cudaGetLastError());
}

template <class T>
Amg<T>::~Amg() = default;

template <class T>
void Amg<T>::pairwise(cudaStream_t s, const SellPattern& P, const T* A, int n, double theta, DBuf<int>& agg,
                      DBuf<int2>& kids, int& ncoarse)
{
    best_.alloc(std::max<size_t>(best_.n, n));
    state_.alloc(std::max<size_t>(state_.n, n));
    flag_.alloc(std::max<size_t>(flag_.n, n + 1));
    scan_.alloc(std::max<size_t>(scan_.n, n + 1));
    DBuf<double> dval;
    dval.alloc(n);
    DBuf<int> partner;
    partner.alloc(n);
    const int nb = div_up(n, TB);
    k_diag_vals<T><<<nb, TB, 0, s>>>(n, P.diag.p, A, dval.p);
    PORSOL_CUDA(cudaMemsetAsync(state_.p, 0, n * sizeof(int), s));
    for (int sweep = 0; sweep < 4; ++sweep) {
        k_pick<T><<<nb, TB, 0, s>>>(n, P.slice_ptr.p, P.col.p, P.rowlen.p, A, dval.p, state_.p, best_.p, theta);
        k_match<<<nb, TB, 0, s>>>(n, state_.p, best_.p, partner.p);
    }
    k_rep_flag<<<nb, TB, 0, s>>>(n, state_.p, partner.p, flag_.p);
    exclusive_scan(s, n, flag_.p, scan_.p, scan_.p + n, scan_blocks_);
    ncoarse = read_int(s, scan_.p + n);
    agg.alloc(n);
    kids.alloc(std::max(ncoarse, 1));
    k_assign<<<nb, TB, 0, s>>>(n, state_.p, partner.p, flag_.p, scan_.p, agg.p, kids.p);
    PORSOL_CUDA(cudaGetLastError());
    PORSOL_CUDA(cudaStreamSynchronize(s));   // temporaries are freed on return
}

template <class T>
void Amg<T>::galerkin_pairs(cudaStream_t s, const SellPattern& P, const T* A, int n, const int* agg,
                            const int2* kids, int nc, SellPattern& Pc, DBuf<T>& Ac)
{
    (void)n;
    Pc.n = nc;
    Pc.nslices = div_up(nc, 32);
    Pc.rowlen.alloc(nc);
    Pc.diag.alloc(nc);
    Pc.slice_ptr.alloc(Pc.nslices + 1);
    const int nb = div_up(nc, 128);
    k_gal_count<T><<<nb, 128, 0, s>>>(nc, P.slice_ptr.p, P.col.p, P.rowlen.p, A, agg, kids, Pc.rowlen.p,
                                      status_.p);
    DBuf<int> width;
    width.alloc(Pc.nslices);
    k_slice_width<<<div_up(Pc.nslices, TB), TB, 0, s>>>(nc, Pc.nslices, Pc.rowlen.p, width.p);
    exclusive_scan(s, Pc.nslices, width.p, Pc.slice_ptr.p, Pc.slice_ptr.p + Pc.nslices, scan_blocks_);
    Pc.nent = read_int(s, Pc.slice_ptr.p + Pc.nslices);
    const int st = read_int(s, status_.p);
    PORSOL_REQUIRE(st == 0, PORSOL_ERR_BAD_ARG, "AMG: coarse row exceeds the Galerkin merge capacity");
    Pc.col.alloc(Pc.nent);
    Ac.alloc(Pc.nent);
    k_gal_fill<T><<<nb, 128, 0, s>>>(nc, P.slice_ptr.p, P.col.p, P.rowlen.p, A, agg, kids, Pc.slice_ptr.p,
                                     Pc.col.p, Ac.p, Pc.diag.p);
    k_pad_tail<<<1, 32, 0, s>>>(nc, Pc.nslices, Pc.slice_ptr.p, Pc.col.p, Ac.p, int(sizeof(T)));
    PORSOL_CUDA(cudaGetLastError());
    PORSOL_CUDA(cudaStreamSynchronize(s));
}

template <class T>
void Amg<T>::build_coarse_solver(cudaStream_t s, const SellPattern& P, const T* A, int n)
{
    nc_ = n;
    Pc_ = &P;
    Ac_ = A;
    DBuf<double> D, Linv;
    D.alloc((size_t)n * n);
    Linv.alloc((size_t)n * n);
    cinv_.alloc((size_t)n * n);
    k_dense_from_sell<T><<<div_up(n, 128), 128, 0, s>>>(n, P.slice_ptr.p, P.col.p, P.rowlen.p, A, D.p);
    k_dense_cholesky_inverse<<<1, 1024, 0, s>>>(n, D.p, Linv.p, cinv_.p, status_.p);
    PORSOL_CUDA(cudaGetLastError());
    const int st = read_int(s, status_.p);
    PORSOL_REQUIRE(st == 0, PORSOL_ERR_NONFINITE, "AMG: coarsest matrix is not positive definite");
}

template <class T>
void Amg<T>::setup(cudaStream_t s, const SellPattern& P0, const T* A0, const AmgOpts& o)
{
    o_ = o;
    lv_.clear();
    sizes_.clear();
    nnzs_.clear();
    status_.alloc(1);
    status_.zero(s);
    {
        auto L0 = std::make_unique<Level>();
        L0->n = P0.n;
        L0->P = &P0;
        L0->A = A0;
        lv_.push_back(std::move(L0));
    }
    sizes_.push_back(P0.n);
    nnzs_.push_back(P0.nent);
    const double theta = o.strength;
    while (lv_.back()->n > o.coarse_target && int(lv_.size()) < o.max_levels) {
        Level& L = *lv_.back();
        const int n = L.n;
        const SellPattern& P = *L.P;
        L.dinv.alloc(n);
        k_l1_dinv<T><<<div_up(n, TB), TB, 0, s>>>(n, P.slice_ptr.p, P.rowlen.p, L.A, L.dinv.p, status_.p);
        // round 1 on this level's matrix
        int nc1 = 0;
        DBuf<int2> kids1;
        pairwise(s, P, L.A, n, theta, L.agg, kids1, nc1);
        if (nc1 > 0.8 * n) pairwise(s, P, L.A, n, 0.0, L.agg, kids1, nc1);
        galerkin_pairs(s, P, L.A, n, L.agg.p, kids1.p, nc1, tmp_pat_, tmp_val_);
        auto next = std::make_unique<Level>();
        if (nc1 > o.coarse_target) {
            // round 2 on the intermediate matrix: aggregates of up to four rows
            int nc2 = 0;
            DBuf<int2> kids2;
            pairwise(s, tmp_pat_, tmp_val_.p, nc1, theta, tmp_agg_, kids2, nc2);
            if (nc2 > 0.8 * nc1) pairwise(s, tmp_pat_, tmp_val_.p, nc1, 0.0, tmp_agg_, kids2, nc2);
            galerkin_pairs(s, tmp_pat_, tmp_val_.p, nc1, tmp_agg_.p, kids2.p, nc2, next->own, next->own_val);
            k_compose<<<div_up(n, TB), TB, 0, s>>>(n, L.agg.p, tmp_agg_.p);
            L.children.alloc(nc2);
            k_kids4<<<div_up(nc2, TB), TB, 0, s>>>(nc2, kids2.p, kids1.p, L.children.p);
            next->n = nc2;
        } else {
            std::swap(next->own.slice_ptr, tmp_pat_.slice_ptr);
            std::swap(next->own.col, tmp_pat_.col);
            std::swap(next->own.rowlen, tmp_pat_.rowlen);
            std::swap(next->own.diag, tmp_pat_.diag);
            next->own.n = tmp_pat_.n;
            next->own.nslices = tmp_pat_.nslices;
            next->own.nent = tmp_pat_.nent;
            std::swap(next->own_val, tmp_val_);
            L.children.alloc(nc1);
            k_kids2to4<<<div_up(nc1, TB), TB, 0, s>>>(nc1, kids1.p, L.children.p);
            next->n = nc1;
        }
        PORSOL_CUDA(cudaGetLastError());
        L.x.alloc(n);
        L.r.alloc(n);
        next->P = &next->own;
        next->A = next->own_val.p;
        next->b.alloc(std::max(next->n, 1));
        next->x.alloc(std::max(next->n, 1));
        sizes_.push_back(next->n);
        nnzs_.push_back(next->own.nent);
        PORSOL_CUDA(cudaStreamSynchronize(s));
        const bool stalled = next->n > 0.9 * n;
        lv_.push_back(std::move(next));
        if (stalled) break;
    }
    Level& C = *lv_.back();
    PORSOL_REQUIRE(C.n <= 2048, PORSOL_ERR_BAD_ARG, "AMG: coarsening stalled above the dense-solve limit");
    build_coarse_solver(s, *C.P, C.A, C.n);
    const int st = read_int(s, status_.p);
    PORSOL_REQUIRE(st == 0, PORSOL_ERR_NONFINITE, "AMG setup: non-finite or non-positive smoother diagonal");
}

template <class T>
void Amg<T>::vcycle(cudaStream_t s, int l, const T* b, T* x, const int* stop)
{
    if (l == int(lv_.size()) - 1) {
        const int threads = 512;
        k_dense_apply<T><<<1, threads, nc_ * sizeof(double), s>>>(nc_, cinv_.p, b, x, stop);
        return;
    }
    Level& L = *lv_[l];
    Level& Nx = *lv_[l + 1];
    const int n = L.n;
    const int nb = div_up(n, TB);
    const SellPattern& P = *L.P;
    const int ncn = Nx.n;
    T* bc = Nx.b.p;
    T* xc = Nx.x.p;
    T* t = L.x.p;   // pre-smoothed iterate
    T* r = L.r.p;
    k_jacobi0<T><<<nb, TB, 0, s>>>(n, L.dinv.p, b, t, stop);
    for (int sw = 1; sw < o_.smooth_steps; ++sw) {
        k_jacobi<T><<<nb, TB, 0, s>>>(n, P.slice_ptr.p, P.col.p, L.A, L.dinv.p, b, t, r, stop);
        std::swap(t, r);
    }
    k_resid<T><<<nb, TB, 0, s>>>(n, P.slice_ptr.p, P.col.p, L.A, b, t, r, stop);
    k_restrict<T><<<div_up(ncn, TB), TB, 0, s>>>(ncn, L.children.p, r, bc, stop);
    vcycle(s, l + 1, bc, xc, stop);
    const T wp = T(o_.prolong);
    if (o_.smooth_steps == 1) {
        k_prolong_smooth<T><<<nb, TB, 0, s>>>(n, P.slice_ptr.p, P.col.p, L.A, L.dinv.p, b, t, xc, L.agg.p, wp, x,
                                              stop);
    } else {
        k_prolong<T><<<nb, TB, 0, s>>>(n, L.agg.p, xc, wp, t, stop);
        T* cur = t;
        T* nxt = r;
        for (int sw = 0; sw < o_.smooth_steps; ++sw) {
            T* dst = (sw == o_.smooth_steps - 1) ? x : nxt;
            k_jacobi<T><<<nb, TB, 0, s>>>(n, P.slice_ptr.p, P.col.p, L.A, L.dinv.p, b, cur, dst, stop);
            nxt = cur;
            cur = dst;
        }
    }
    PORSOL_CUDA(cudaGetLastError());
}

template <class T>
void Amg<T>::apply(cudaStream_t s, const T* r, T* z, const int* stop)
{
    vcycle(s, 0, r, z, stop);
}

template class Amg<double>;
template class Amg<float>;

}  // namespace porsol
