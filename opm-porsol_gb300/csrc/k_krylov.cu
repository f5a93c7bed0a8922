// k_krylov.cu -- SELL-32 SpMV, fused CG updates with deterministic last-block
// reductions, and level-scheduled ILU(0).
//
// Reductions: every block writes one FP64 partial sum; the last block to arrive (arrival
// counter + threadfence) adds the partials in block order and updates the CG scalars in
// device memory.  The summation order is fixed, so results are run-to-run reproducible.
#include <algorithm>
#include <cmath>

#include "krylov.h"
#include "sell.cuh"

namespace porsol {

namespace {

constexpr int RB = 256;  // threads per block of the vector kernels

// Blocks of the reduction kernels: at most 8 per SM, grid-stride beyond.  The last-block
// reduction costs one fence + atomic per block, so a grid of one thread per row (12k blocks at
// 3 M rows) spends more time arriving than summing.  The cap depends only on the device, so
// the summation order stays fixed.
int red_blocks(int n)
{
    static int cap = 0;
    if (cap == 0) {
        int dev = 0, sms = 0;
        PORSOL_CUDA(cudaGetDevice(&dev));
        PORSOL_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        cap = std::max(1, 8 * sms);
    }
    return std::max(1, std::min(div_up(std::max(n, 1), RB), cap));
}

template <class V>
__device__ __forceinline__ V warp_sum(V v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block reduce + last-block finalisation.  Returns true in thread 0 of the last block,
// with *total holding the full sum.  The per-thread value type V is the vector type: FP32
// vectors are summed in FP32 within a warp (32 terms) and in FP64 from there on, so the
// FP64 unit (a small fraction of GB300's FP32 rate) only sees one value per warp.
template <class V>
__device__ bool block_reduce_last(V v0, double* partial, unsigned int* counter, double* total)
{
    __shared__ double ws[RB / 32];
    __shared__ bool amlast;
    const double v = double(warp_sum<V>(v0));
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
        t = warp_sum<double>(t);
        if (threadIdx.x == 0) {
            partial[blockIdx.x] = t;
            __threadfence();
            const unsigned int prev = atomicAdd(counter, 1u);
            amlast = (prev == gridDim.x - 1);
        }
    }
    __syncthreads();
    if (!amlast) return false;
    // last block: sum partials in block order
    __threadfence();
    double s = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) s += ((volatile double*)partial)[b];
    // fixed-order tree over threads
    s = warp_sum<double>(s);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[w];
        *total = t;
        *counter = 0u;
    }
    return threadIdx.x == 0;
}

// Row r of a SELL matrix times x, accumulated in the vector type TX (FP32 rows stay on the
// FP32 pipe).
template <class TV, class TX, class CI>
__device__ __forceinline__ TX sell_row(const int* __restrict__ sp, const CI* __restrict__ col,
                                       const TV* __restrict__ val, const TX* __restrict__ x, int r)
{
    return sell_dot<TX>(sp, col, val, r, [x](int j) { return x[j]; });
}

template <class TV, class TX>
__global__ void k_spmv(int n, const int* __restrict__ sp, const int* __restrict__ col, const TV* __restrict__ val,
                       const TX* __restrict__ x, TX* __restrict__ y)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    y[r] = TX(sell_row(sp, col, val, x, r));
}

template <class TV, class TX>
__global__ void k_residual(int n, const int* __restrict__ sp, const int* __restrict__ col,
                           const TV* __restrict__ val, const TX* __restrict__ x, const TX* __restrict__ b,
                           TX* __restrict__ y)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    y[r] = b[r] - sell_row(sp, col, val, x, r);
}

// r = b - A x; def0 = ||r||
template <class TV, class T, class CI>
__global__ void __launch_bounds__(RB) k_cg_init(int n, const int* __restrict__ sp, const CI* __restrict__ col,
                                                const TV* __restrict__ val, const T* __restrict__ x,
                                                const T* __restrict__ b, T* __restrict__ r, CgDev* st,
                                                double* partial, unsigned int* counter, CgHostView* hv)
{
    chain_wait();
    T v = 0;
    for (int i = blockIdx.x * RB + threadIdx.x; i < n; i += gridDim.x * RB) {
        const T ri = b[i] - sell_row(sp, col, val, x, i);
        r[i] = ri;
        v += ri * ri;
    }
    double tot;
    if (block_reduce_last<T>(v, partial, counter, &tot)) {
        const double d0 = sqrt(tot);
        st->def0 = d0;
        st->def = d0;
        st->iter = 0;
        st->breakdown = 0;
        st->converged = (d0 < 1e-30) ? 1 : 0;
        st->stop = st->converged;
        hv->def0 = d0;
        hv->def = d0;
        hv->iter = 0;
        hv->converged = st->converged;
        hv->stop = st->stop;
        hv->breakdown = 0;
        __threadfence_system();
    }
}

// rho = z . r ; which = 0: first direction p = z, rholast = rho; which = 1: rho for beta
template <class T>
__global__ void __launch_bounds__(RB) k_dot_zr(int n, const T* __restrict__ z, const T* __restrict__ r, CgDev* st,
                                               double* partial, unsigned int* counter)
{
    chain_wait();
    if (st->stop) return;
    T v = 0;
    for (int i = blockIdx.x * RB + threadIdx.x; i < n; i += gridDim.x * RB) v += z[i] * r[i];
    double tot;
    if (block_reduce_last<T>(v, partial, counter, &tot)) {
        st->rho = tot;
        st->beta = tot / st->rholast;
    }
}

template <class T>
__global__ void k_first_direction(int n, const T* __restrict__ z, T* __restrict__ p, CgDev* st)
{
    chain_wait();
    if (st->stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = z[i];
    if (i == 0) st->rholast = st->rho;   // other threads do not read rholast here
}

// q = A p ; alpha = p . q
template <class TV, class T, class CI>
__global__ void __launch_bounds__(RB) k_spmv_pq(int n, const int* __restrict__ sp, const CI* __restrict__ col,
                                                const TV* __restrict__ val, const T* __restrict__ p,
                                                T* __restrict__ q, CgDev* st, double* partial,
                                                unsigned int* counter)
{
    chain_wait();
    if (st->stop) return;
    T v = 0;
    for (int i = blockIdx.x * RB + threadIdx.x; i < n; i += gridDim.x * RB) {
        const T qi = sell_row(sp, col, val, p, i);
        q[i] = qi;
        v += p[i] * qi;
    }
    double tot;
    if (block_reduce_last<T>(v, partial, counter, &tot)) {
        st->alpha = tot;
        st->lambda = st->rholast / tot;
    }
}

// lambda = rholast/alpha; x += lambda p; r -= lambda q; def = ||r||; convergence test
template <class T>
__global__ void __launch_bounds__(RB) k_cg_update(int n, T* __restrict__ x, T* __restrict__ r,
                                                  const T* __restrict__ p, const T* __restrict__ q, CgDev* st,
                                                  double* partial, unsigned int* counter, CgHostView* hv)
{
    chain_wait();
    if (st->stop) return;
    const double alpha = st->alpha;
    const T lambda = T(st->lambda);
    T v = 0;
    for (int i = blockIdx.x * RB + threadIdx.x; i < n; i += gridDim.x * RB) {
        x[i] = x[i] + lambda * p[i];
        const T ri = r[i] - lambda * q[i];
        r[i] = ri;
        v += ri * ri;
    }
    double tot;
    if (block_reduce_last<T>(v, partial, counter, &tot)) {
        const double def = sqrt(tot);
        st->def = def;
        st->iter += 1;
        if (!(alpha > 0.0) || !isfinite(def)) st->breakdown = 1;
        if (def < st->def0 * st->tol || def < 1e-30) st->converged = 1;
        st->stop = st->converged || st->breakdown || st->iter >= st->maxit;
        hv->def = def;
        hv->iter = st->iter;
        hv->converged = st->converged;
        hv->breakdown = st->breakdown;
        hv->stop = st->stop;
        __threadfence_system();
    }
}

// beta = rho/rholast; p = z + beta p; rholast = rho for the next iteration (no thread of
// this kernel reads rholast)
template <class T>
__global__ void k_cg_direction(int n, const T* __restrict__ z, T* __restrict__ p, CgDev* st)
{
    chain_wait();
    if (st->stop) return;
    const T beta = T(st->beta);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = z[i] + beta * p[i];
    if (i == 0) st->rholast = st->rho;
}

template <class TA, class TB>
__global__ void k_convert(long long n, const TA* __restrict__ a, TB* __restrict__ b)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) b[i] = TB(a[i]);
}

__global__ void k_axpy_add(int n, const double* __restrict__ y, double* __restrict__ x)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] += y[i];
}

__global__ void k_dirichlet_guess(int n, const int* __restrict__ sp, const int* __restrict__ col,
                                  const int* __restrict__ rowlen, const double* __restrict__ val,
                                  const double* __restrict__ b, double* __restrict__ x)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int s = r >> 5, lane = r & 31;
    const int base = sp[s];
    bool isD = true;
    double d = 0.0;
    for (int t = 0; t < rowlen[r]; ++t) {
        const int k = base + t * 32 + lane;
        if (col[k] == r) d = val[k];
        else if (val[k] != 0.0) isD = false;
    }
    x[r] = isD ? b[r] / d : 0.0;
}

template <class T>
__global__ void __launch_bounds__(RB) k_norm2(int n, const T* __restrict__ x, double* partial, unsigned int* counter,
                                              double* out)
{
    T v = 0;
    for (int i = blockIdx.x * RB + threadIdx.x; i < n; i += gridDim.x * RB) v += x[i] * x[i];
    double tot;
    if (block_reduce_last<T>(v, partial, counter, &tot)) *out = tot;
}

// ---------------- mixed-precision CG with reliable updates ----------------
__device__ __forceinline__ void rc_publish(const RcDev* st, CgHostView* hv)
{
    hv->def0 = st->def0;
    hv->def = st->true_def;
    hv->iter = st->iter;
    hv->converged = st->converged;
    hv->breakdown = st->breakdown;
    hv->stop = st->stop;
    __threadfence_system();
}

// r64 = b - A x (FP64); def0 = sigma = ||r64||
template <class CI>
__global__ void __launch_bounds__(RB) k_rc_init(int n, const int* __restrict__ sp, const CI* __restrict__ col,
                                                const double* __restrict__ val, const double* __restrict__ x,
                                                const double* __restrict__ b, double* __restrict__ r64, RcDev* st,
                                                double* partial, unsigned int* counter, CgHostView* hv)
{
    chain_wait();
    double v = 0.0;
    for (int i = blockIdx.x * RB + threadIdx.x; i < n; i += gridDim.x * RB) {
        const double ri = b[i] - sell_row(sp, col, val, x, i);
        r64[i] = ri;
        v += ri * ri;
    }
    double tot;
    if (block_reduce_last<double>(v, partial, counter, &tot)) {
        const double d = sqrt(tot);
        st->def0 = st->true_def = st->sigma = d;
        st->isig = d > 0.0 ? 1.0 / d : 0.0;
        st->factor = 1.0;
        st->iter = st->nrep = st->replace = st->breakdown = 0;
        st->converged = (d < 1e-30) ? 1 : 0;
        st->stop = st->converged || !isfinite(d);
        st->breakdown = !isfinite(d);
        rc_publish(st, hv);
    }
}

// r32 = r64 / sigma; p *= factor (after a replacement, or at the start when p is unused)
__global__ void k_rc_rescale(int n, const double* __restrict__ r64, float* __restrict__ r, float* __restrict__ p,
                             const RcDev* st, int init)
{
    chain_wait();
    if (st->stop || !(init || st->replace)) return;
    const double is = st->isig;
    const float f = float(st->factor);
    for (int i = blockIdx.x * RB + threadIdx.x; i < n; i += gridDim.x * RB) {
        r[i] = float(r64[i] * is);
        if (!init) p[i] *= f;
    }
}

// q = A32 p; alpha = rho / (p . q)
template <class CI>
__global__ void __launch_bounds__(RB) k_rc_pq(int n, const int* __restrict__ sp, const CI* __restrict__ col,
                                              const float* __restrict__ val, const float* __restrict__ p,
                                              float* __restrict__ q, RcDev* st, double* partial,
                                              unsigned int* counter, CgHostView* hv)
{
    chain_wait();
    if (st->stop) return;
    float v = 0.0f;
    for (int i = blockIdx.x * RB + threadIdx.x; i < n; i += gridDim.x * RB) {
        const float qi = sell_row(sp, col, val, p, i);
        q[i] = qi;
        v += p[i] * qi;
    }
    double tot;
    if (block_reduce_last<float>(v, partial, counter, &tot)) {
        if (!(tot > 0.0) || !isfinite(tot)) {
            st->alpha = 0.0;
            st->breakdown = 1;
            st->stop = 1;
            rc_publish(st, hv);
        } else {
            st->alpha = st->rho / tot;
        }
    }
}

// x += sigma alpha p (FP64); r -= alpha q; decide on a replacement
__global__ void __launch_bounds__(RB) k_rc_update(int n, double* __restrict__ x, float* __restrict__ r,
                                                  const float* __restrict__ p, const float* __restrict__ q,
                                                  RcDev* st, double* partial, unsigned int* counter,
                                                  CgHostView* hv)
{
    chain_wait();
    if (st->stop) return;
    const double sa = st->sigma * st->alpha;
    const float a = float(st->alpha);
    float v = 0.0f;
    for (int i = blockIdx.x * RB + threadIdx.x; i < n; i += gridDim.x * RB) {
        x[i] += sa * double(p[i]);
        const float ri = r[i] - a * q[i];
        r[i] = ri;
        v += ri * ri;
    }
    double tot;
    if (block_reduce_last<float>(v, partial, counter, &tot)) {
        const double defs = sqrt(tot);
        st->defs = defs;
        st->iter += 1;
        const double est = defs * st->sigma;
        st->replace = (defs < st->delta || est < st->tol * st->def0 || est < 1e-30 || !isfinite(defs) ||
                       st->iter >= st->maxit)
                          ? 1
                          : 0;
        hv->iter = st->iter;
        __threadfence_system();
    }
}

// Replacement: r64 = b - A x in FP64; convergence is decided on this true residual only
template <class CI>
__global__ void __launch_bounds__(RB) k_rc_true(int n, const int* __restrict__ sp, const CI* __restrict__ col,
                                                const double* __restrict__ val, const double* __restrict__ x,
                                                const double* __restrict__ b, double* __restrict__ r64, RcDev* st,
                                                double* partial, unsigned int* counter, CgHostView* hv)
{
    chain_wait();
    if (st->stop || !st->replace) return;
    double v = 0.0;
    for (int i = blockIdx.x * RB + threadIdx.x; i < n; i += gridDim.x * RB) {
        const double ri = b[i] - sell_row(sp, col, val, x, i);
        r64[i] = ri;
        v += ri * ri;
    }
    double tot;
    if (block_reduce_last<double>(v, partial, counter, &tot)) {
        const double d = sqrt(tot);
        st->true_def = d;
        st->nrep += 1;
        if (!isfinite(d)) {
            st->breakdown = 1;
            st->stop = 1;
        } else if (d < st->tol * st->def0 || d < 1e-30) {
            st->converged = 1;
            st->stop = 1;
        } else if (st->iter >= st->maxit) {
            st->stop = 1;
        } else {
            // continue on the rescaled system: r and p in units of the new sigma
            st->factor = st->sigma / d;
            st->rho *= st->factor * st->factor;
            st->sigma = d;
            st->isig = 1.0 / d;
        }
        rc_publish(st, hv);
    }
}

// rho_new = z . r; beta = rho_new / rho
__global__ void __launch_bounds__(RB) k_rc_zr(int n, const float* __restrict__ z, const float* __restrict__ r,
                                              RcDev* st, double* partial, unsigned int* counter, int init)
{
    chain_wait();
    if (st->stop) return;
    float v = 0.0f;
    for (int i = blockIdx.x * RB + threadIdx.x; i < n; i += gridDim.x * RB) v += z[i] * r[i];
    double tot;
    if (block_reduce_last<float>(v, partial, counter, &tot)) {
        st->beta = init ? 0.0 : tot / st->rho;
        st->rho = tot;
        st->replace = 0;
    }
}

// p = z + beta p (beta = 0 at the start)
__global__ void k_rc_direction(int n, const float* __restrict__ z, float* __restrict__ p, const RcDev* st, int init)
{
    chain_wait();
    if (st->stop) return;
    const float beta = float(st->beta);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = init ? z[i] : z[i] + beta * p[i];
}

// ---------------- ILU(0) ----------------
__device__ __forceinline__ int sell_slot(const int* sp, int r, int t) { return sp[r >> 5] + t * 32 + (r & 31); }

__global__ void k_ilu_factor_level(int nrows, const int* __restrict__ rows, const int* __restrict__ sp,
                                   const int* __restrict__ col, const int* __restrict__ rowlen,
                                   const int* __restrict__ diag, double* __restrict__ lu, int* status)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nrows) return;
    const int i = rows[q];
    const int li = rowlen[i];
    for (int t = 0; t < li; ++t) {
        const int ij = sell_slot(sp, i, t);
        const int j = col[ij];
        if (j >= i) break;
        const int jj = diag[j];
        lu[ij] *= lu[jj];                     // L_ij = a_ij * inv(a_jj)
        const double lij = lu[ij];
        // a_ik -= L_ij a_jk for k > j present in both rows
        const int lj = rowlen[j];
        int tj = 0;
        while (tj < lj && col[sell_slot(sp, j, tj)] <= j) ++tj;
        int ti = t + 1;
        while (ti < li && tj < lj) {
            const int ik = sell_slot(sp, i, ti), jk = sell_slot(sp, j, tj);
            const int ci = col[ik], cj = col[jk];
            if (ci == cj) {
                lu[ik] -= lij * lu[jk];
                ++ti;
                ++tj;
            } else if (ci < cj) {
                ++ti;
            } else {
                ++tj;
            }
        }
    }
    const int d = diag[i];
    const double piv = lu[d];
    if (!(fabs(piv) > 0.0) || !isfinite(piv)) atomicOr(status, ST_NONFINITE);
    lu[d] = 1.0 / piv;
}

__global__ void k_ilu_lower_level(int nrows, const int* __restrict__ rows, const int* __restrict__ sp,
                                  const int* __restrict__ col, const int* __restrict__ diag,
                                  const double* __restrict__ lu, const double* __restrict__ r, double* __restrict__ z,
                                  const int* stop)
{
    chain_wait();
    if (*stop) return;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nrows) return;
    const int i = rows[q];
    double v = r[i];
    const int d = diag[i];
    for (int k = sp[i >> 5] + (i & 31); k < d; k += 32) v -= lu[k] * z[col[k]];
    z[i] = v;
}

__global__ void k_ilu_upper_level(int nrows, const int* __restrict__ rows, const int* __restrict__ sp,
                                  const int* __restrict__ col, const int* __restrict__ rowlen,
                                  const int* __restrict__ diag, const double* __restrict__ lu, double* __restrict__ z,
                                  const int* stop)
{
    chain_wait();
    if (*stop) return;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nrows) return;
    const int i = rows[q];
    const int d = diag[i];
    const int end = sp[i >> 5] + rowlen[i] * 32 + (i & 31);
    double v = z[i];
    for (int k = d + 32; k < end; k += 32) v -= lu[k] * z[col[k]];
    z[i] = lu[d] * v;
}

}  // namespace

// ----------------------------------------------------------------------------
void RedScratch::ensure(int blocks, cudaStream_t s)
{
    if (blocks <= max_blocks) return;
    partial.alloc(blocks);
    counter.alloc(1);
    counter.zero(s);
    max_blocks = blocks;
}

template <class TV, class TX>
void spmv(cudaStream_t s, const SellPattern& P, const TV* val, const TX* x, TX* y)
{
    if (P.n == 0) return;
    PORSOL_LAUNCH(k_spmv<TV, TX><<<div_up(P.n, RB), RB, 0, s>>>(P.n, P.slice_ptr.p, P.col.p, val, x, y));
    PORSOL_CUDA(cudaGetLastError());
}

template <class TV, class TX>
void residual(cudaStream_t s, const SellPattern& P, const TV* val, const TX* x, const TX* b, TX* y)
{
    if (P.n == 0) return;
    PORSOL_LAUNCH(k_residual<TV, TX><<<div_up(P.n, RB), RB, 0, s>>>(P.n, P.slice_ptr.p, P.col.p, val, x, b, y));
    PORSOL_CUDA(cudaGetLastError());
}

template void spmv<double, double>(cudaStream_t, const SellPattern&, const double*, const double*, double*);
template void spmv<float, float>(cudaStream_t, const SellPattern&, const float*, const float*, float*);
template void residual<double, double>(cudaStream_t, const SellPattern&, const double*, const double*,
                                       const double*, double*);
template void residual<float, float>(cudaStream_t, const SellPattern&, const float*, const float*, const float*,
                                     float*);

template <class TV, class T>
void PcgSolver<TV, T>::setup(int n, cudaStream_t s)
{
    if (n == n_ && hview_) return;
    n_ = n;
    r_.alloc(n);
    z_.alloc(n);
    p_.alloc(n);
    q_.alloc(n);
    st_.alloc(1);
    red_.ensure(div_up(std::max(n, 1), RB), s);
    if (!hview_) {
        PORSOL_CUDA(cudaHostAlloc((void**)&hview_, sizeof(CgHostView), cudaHostAllocMapped));
        PORSOL_CUDA(cudaHostGetDevicePointer((void**)&dview_, hview_, 0));
    }
    if (ev_.empty()) {
        ev_.resize(4);
        for (auto& e : ev_) PORSOL_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
}

template <class TV, class T>
PcgSolver<TV, T>::~PcgSolver()
{
    if (exec_) cudaGraphExecDestroy(exec_);
    if (hview_) cudaFreeHost(hview_);
    for (auto& e : ev_) cudaEventDestroy(e);
}

template <class TV, class T>
void PcgSolver<TV, T>::iteration(cudaStream_t s, const SellPattern& P, const TV* val, Precond<T>& M, T* x,
                                 Profiler* prof, int prof_kernel)
{
    const int n = P.n;
    const int nb = div_up(n, RB), nr = red_blocks(n);
    const int* stop = &st_.p->stop;
    const double spmv_bytes = double(P.nent) * (sizeof(TV) + (P.has_off16() ? 2 : 4)) + 2.0 * n * sizeof(T);
    {
        const bool pf = prof && prof->on && prof_kernel >= 0;
        cudaEvent_t ev = nullptr;
        if (pf) prof->begin(s, prof_kernel, spmv_bytes, &ev);
        if (P.has_off16())
            chain(k_spmv_pq<TV, T, short>, nr, RB, 0, s, n, P.slice_ptr.p, P.off16.p, val, p_.p, q_.p, st_.p,
                red_.partial.p, red_.counter.p);
        else
            chain(k_spmv_pq<TV, T, int>, nr, RB, 0, s, n, P.slice_ptr.p, P.col.p, val, p_.p, q_.p, st_.p,
                red_.partial.p, red_.counter.p);
        if (pf) prof->end(s, prof_kernel, spmv_bytes, ev);
    }
    chain(k_cg_update<T>, nr, RB, 0, s, n, x, r_.p, p_.p, q_.p, st_.p, red_.partial.p, red_.counter.p, dview_);
    M.apply(s, r_.p, z_.p, stop);
    chain(k_dot_zr<T>, nr, RB, 0, s, n, z_.p, r_.p, st_.p, red_.partial.p, red_.counter.p);
    chain(k_cg_direction<T>, nb, RB, 0, s, n, z_.p, p_.p, st_.p);
}

template <class TV, class T>
CgResult PcgSolver<TV, T>::solve(cudaStream_t s, const SellPattern& P, const TV* val, Precond<T>& M, const T* b,
                                 T* x, double tol, int maxit, Profiler* prof, int prof_kernel)
{
    const int n = P.n;
    ChainPause plain(prof && prof->on);   // events between the kernels time each one
    CgResult res;
    if (n == 0) {
        res.converged = true;
        return res;
    }
    setup(n, s);
    M.set_block_state(nullptr);   // one system: every row works
    const int nb = div_up(n, RB), nr = red_blocks(n);
    CgDev init{};
    init.tol = tol;
    init.maxit = maxit;
    PORSOL_CUDA(cudaMemcpyAsync(st_.p, &init, sizeof(CgDev), cudaMemcpyHostToDevice, s));
    if (P.has_off16())
        chain(k_cg_init<TV, T, short>, nr, RB, 0, s, n, P.slice_ptr.p, P.off16.p, val, x, b, r_.p, st_.p,
            red_.partial.p, red_.counter.p, dview_);
    else
        chain(k_cg_init<TV, T, int>, nr, RB, 0, s, n, P.slice_ptr.p, P.col.p, val, x, b, r_.p, st_.p, red_.partial.p,
            red_.counter.p, dview_);
    PORSOL_CUDA(cudaGetLastError());
    const int* stop = &st_.p->stop;
    M.apply(s, r_.p, z_.p, stop);
    chain(k_dot_zr<T>, nr, RB, 0, s, n, z_.p, r_.p, st_.p, red_.partial.p, red_.counter.p);
    chain(k_first_direction<T>, nb, RB, 0, s, n, z_.p, p_.p, st_.p);
    PORSOL_CUDA(cudaGetLastError());
    // One iteration is captured into a CUDA graph (re-captured when the matrix, vectors or
    // preconditioner change) unless per-kernel profiling is on.
    const bool graphs = use_graphs_ && !(prof && prof->on);
    if (graphs) {
        const void* key[5] = {&P, val, x, (const void*)&M, nullptr};
        bool same = exec_ && key_gen_ == M.generation();
        for (int k = 0; k < 4 && same; ++k) same = key_[k] == key[k];
        if (!same) {
            if (exec_) {
                cudaGraphExecDestroy(exec_);
                exec_ = nullptr;
            }
            cudaGraph_t g;
            const long long l0 = g_launches.load();
            PORSOL_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            iteration(s, P, val, M, x, nullptr, -1);
            PORSOL_CUDA(cudaStreamEndCapture(s, &g));
            nodes_ = g_launches.load() - l0;   // captured, not run: counted at each replay
            g_launches.fetch_sub(nodes_);
            PORSOL_CUDA(cudaGraphInstantiate(&exec_, g, 0));
            PORSOL_CUDA(cudaGraphDestroy(g));
            for (int k = 0; k < 4; ++k) key_[k] = key[k];
            key_gen_ = M.generation();
        }
    }
    // Iterations are queued ahead; the host waits on the event of iteration i - LOOKAHEAD
    // and reads the mapped stop flag.  Iterations queued after convergence are no-ops.
    const int LOOKAHEAD = 2;
    int it = 0;
    bool done = false;
    while (!done) {
        if (it < maxit) {
            if (graphs) {
                PORSOL_CUDA(cudaGraphLaunch(exec_, s));
                g_launches.fetch_add(nodes_);
            } else {
                iteration(s, P, val, M, x, prof, prof_kernel);
            }
            PORSOL_CUDA(cudaGetLastError());
            PORSOL_CUDA(cudaEventRecord(ev_[it % ev_.size()], s));
            ++it;
        }
        if (it >= LOOKAHEAD || it >= maxit) {
            const int wait_it = (it >= maxit) ? it - 1 : it - LOOKAHEAD;
            PORSOL_CUDA(cudaEventSynchronize(ev_[wait_it % ev_.size()]));
            if (hview_->stop || it >= maxit) {
                if (it >= maxit) PORSOL_CUDA(cudaStreamSynchronize(s));
                done = hview_->stop || it >= maxit;
            }
        }
    }
    PORSOL_CUDA(cudaStreamSynchronize(s));
    res.iterations = hview_->iter;
    res.def0 = hview_->def0;
    res.def = hview_->def;
    res.converged = hview_->converged != 0;
    res.breakdown = hview_->breakdown != 0;
    res.reduction = res.def0 > 0 ? res.def / res.def0 : 0.0;
    return res;
}

template class PcgSolver<double, double>;

// ---------------- ReliableCg host side ----------------
void ReliableCg::setup(int n, cudaStream_t s)
{
    if (n != n_) {
        r_.alloc(n);
        z_.alloc(n);
        p_.alloc(n);
        q_.alloc(n);
        r64_.alloc(n);
        n_ = n;
    }
    st_.alloc(1);
    red_.ensure(div_up(std::max(n, 1), RB), s);
    if (!hview_) {
        PORSOL_CUDA(cudaHostAlloc((void**)&hview_, sizeof(CgHostView), cudaHostAllocMapped));
        PORSOL_CUDA(cudaHostGetDevicePointer((void**)&dview_, hview_, 0));
    }
    if (ev_.empty()) {
        ev_.resize(4);
        for (auto& e : ev_) PORSOL_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
}

ReliableCg::~ReliableCg()
{
    if (exec_) cudaGraphExecDestroy(exec_);
    if (hview_) cudaFreeHost(hview_);
    for (auto& e : ev_) cudaEventDestroy(e);
}

void ReliableCg::iteration(cudaStream_t s, const SellPattern& P, const double* val64, const float* val32,
                           Precond<float>& M, const double* b, double* x, Profiler* prof)
{
    const int n = P.n, nb = div_up(n, RB), nr = red_blocks(n);
    const int* stop = &st_.p->stop;
    {
        const bool pf = prof && prof->on;
        const double bytes = double(P.nent) * (P.has_off16() ? 6.0 : 8.0) + 2.0 * n * 4.0;
        cudaEvent_t ev = nullptr;
        if (pf) prof->begin(s, PK_SPMV32, bytes, &ev);
        if (P.has_off16())
            chain(k_rc_pq<short>, nr, RB, 0, s, n, P.slice_ptr.p, P.off16.p, val32, p_.p, q_.p, st_.p, red_.partial.p,
                red_.counter.p, dview_);
        else
            chain(k_rc_pq<int>, nr, RB, 0, s, n, P.slice_ptr.p, P.col.p, val32, p_.p, q_.p, st_.p, red_.partial.p,
                red_.counter.p, dview_);
        if (pf) prof->end(s, PK_SPMV32, bytes, ev);
    }
    chain(k_rc_update, nr, RB, 0, s, n, x, r_.p, p_.p, q_.p, st_.p, red_.partial.p, red_.counter.p, dview_);
    if (P.has_off16())
        chain(k_rc_true<short>, nr, RB, 0, s, n, P.slice_ptr.p, P.off16.p, val64, x, b, r64_.p, st_.p, red_.partial.p,
            red_.counter.p, dview_);
    else
        chain(k_rc_true<int>, nr, RB, 0, s, n, P.slice_ptr.p, P.col.p, val64, x, b, r64_.p, st_.p, red_.partial.p,
            red_.counter.p, dview_);
    chain(k_rc_rescale, nr, RB, 0, s, n, r64_.p, r_.p, p_.p, st_.p, 0);
    M.apply(s, r_.p, z_.p, stop);
    chain(k_rc_zr, nr, RB, 0, s, n, z_.p, r_.p, st_.p, red_.partial.p, red_.counter.p, 0);
    chain(k_rc_direction, nb, RB, 0, s, n, z_.p, p_.p, st_.p, 0);
}

CgResult ReliableCg::solve(cudaStream_t s, const SellPattern& P, const double* val64, const float* val32,
                           Precond<float>& M, const double* b, double* x, double tol, int maxit, double delta,
                           Profiler* prof)
{
    const int n = P.n;
    ChainPause plain(prof && prof->on);   // events between the kernels time each one
    CgResult res;
    if (n == 0) {
        res.converged = true;
        return res;
    }
    setup(n, s);
    M.set_block_state(nullptr);   // one system: every row works
    const int nb = div_up(n, RB), nr = red_blocks(n);
    RcDev init{};
    init.tol = tol;
    init.maxit = maxit;
    init.delta = delta;
    PORSOL_CUDA(cudaMemcpyAsync(st_.p, &init, sizeof(RcDev), cudaMemcpyHostToDevice, s));
    if (P.has_off16())
        chain(k_rc_init<short>, nr, RB, 0, s, n, P.slice_ptr.p, P.off16.p, val64, x, b, r64_.p, st_.p, red_.partial.p,
            red_.counter.p, dview_);
    else
        chain(k_rc_init<int>, nr, RB, 0, s, n, P.slice_ptr.p, P.col.p, val64, x, b, r64_.p, st_.p, red_.partial.p,
            red_.counter.p, dview_);
    chain(k_rc_rescale, nr, RB, 0, s, n, r64_.p, r_.p, p_.p, st_.p, 1);
    const int* stop = &st_.p->stop;
    M.apply(s, r_.p, z_.p, stop);
    chain(k_rc_zr, nr, RB, 0, s, n, z_.p, r_.p, st_.p, red_.partial.p, red_.counter.p, 1);
    chain(k_rc_direction, nb, RB, 0, s, n, z_.p, p_.p, st_.p, 1);
    PORSOL_CUDA(cudaGetLastError());
    // per-kernel event timing records events inside the V-cycle: no graph capture then
    const bool graphs = !(prof && prof->on);
    const void* key[5] = {&P, val64, val32, (const void*)&M, x};
    bool same = exec_ && key_gen_ == M.generation() && key_[4] == (const void*)b;
    for (int k = 0; k < 4 && same; ++k) same = key_[k] == key[k];
    if (graphs && !same) {
        if (exec_) {
            cudaGraphExecDestroy(exec_);
            exec_ = nullptr;
        }
        cudaGraph_t g;
        const long long l0 = g_launches.load();
        PORSOL_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        iteration(s, P, val64, val32, M, b, x, nullptr);
        PORSOL_CUDA(cudaStreamEndCapture(s, &g));
        nodes_ = g_launches.load() - l0;
        g_launches.fetch_sub(nodes_);
        PORSOL_CUDA(cudaGraphInstantiate(&exec_, g, 0));
        PORSOL_CUDA(cudaGraphDestroy(g));
        for (int k = 0; k < 4; ++k) key_[k] = key[k];
        key_[4] = b;
        key_gen_ = M.generation();
    }
    const int LOOKAHEAD = 2;
    int it = 0;
    bool done = false;
    while (!done) {
        if (it < maxit) {
            if (graphs) {
                PORSOL_CUDA(cudaGraphLaunch(exec_, s));
                g_launches.fetch_add(nodes_);
            } else {
                iteration(s, P, val64, val32, M, b, x, prof);
            }
            PORSOL_CUDA(cudaEventRecord(ev_[it % ev_.size()], s));
            ++it;
        }
        if (it >= LOOKAHEAD || it >= maxit) {
            const int wait_it = (it >= maxit) ? it - 1 : it - LOOKAHEAD;
            PORSOL_CUDA(cudaEventSynchronize(ev_[wait_it % ev_.size()]));
            if (hview_->stop || it >= maxit) {
                if (it >= maxit) PORSOL_CUDA(cudaStreamSynchronize(s));
                done = hview_->stop || it >= maxit;
            }
        }
    }
    RcDev fin{};
    PORSOL_CUDA(cudaMemcpyAsync(&fin, st_.p, sizeof(RcDev), cudaMemcpyDeviceToHost, s));
    PORSOL_CUDA(cudaStreamSynchronize(s));
    nrep_ = fin.nrep;
    res.iterations = fin.iter;
    res.def0 = fin.def0;
    res.def = fin.true_def;
    res.converged = fin.converged != 0;
    res.breakdown = fin.breakdown != 0;
    res.reduction = fin.def0 > 0 ? fin.true_def / fin.def0 : 0.0;
    return res;
}

// ---------------- ILU(0) host side ----------------
void Ilu0::build_levels(const SellPattern& P, cudaStream_t s)
{
    P_ = &P;
    const int n = P.n;
    auto slot = [&](int r, int t) { return (long long)P.h_slice_ptr[r / SELL_C] + (long long)t * SELL_C + r % SELL_C; };
    std::vector<int> lev(n, 0);
    int nl = 0;
    for (int i = 0; i < n; ++i) {
        int l = 0;
        for (int t = 0; t < P.h_rowlen[i]; ++t) {
            const int j = P.h_col[slot(i, t)];
            if (j < i) l = std::max(l, lev[j] + 1);
        }
        lev[i] = l;
        nl = std::max(nl, l + 1);
    }
    auto bucket = [&](const std::vector<int>& lv, int nlev, std::vector<int>& ptr, std::vector<int>& rows, bool rev) {
        ptr.assign(nlev + 1, 0);
        for (int i = 0; i < n; ++i) ptr[lv[i] + 1]++;
        for (int l = 0; l < nlev; ++l) ptr[l + 1] += ptr[l];
        rows.assign(n, 0);
        std::vector<int> f(ptr.begin(), ptr.end() - 1);
        if (!rev)
            for (int i = 0; i < n; ++i) rows[f[lv[i]]++] = i;
        else
            for (int i = n - 1; i >= 0; --i) rows[f[lv[i]]++] = i;
    };
    std::vector<int> lrows, urows;
    bucket(lev, nl, h_lptr_, lrows, false);
    std::vector<int> ulev(n, 0);
    int nu = 0;
    for (int i = n - 1; i >= 0; --i) {
        int l = 0;
        for (int t = 0; t < P.h_rowlen[i]; ++t) {
            const int j = P.h_col[slot(i, t)];
            if (j > i) l = std::max(l, ulev[j] + 1);
        }
        ulev[i] = l;
        nu = std::max(nu, l + 1);
    }
    bucket(ulev, nu, h_uptr_, urows, true);
    lrows_.upload(lrows, s);
    urows_.upload(urows, s);
    PORSOL_CUDA(cudaStreamSynchronize(s));
}

void Ilu0::factor(cudaStream_t s, const SellPattern& P, const double* val)
{
    bump_generation();
    lu_.alloc(P.nent);
    PORSOL_CUDA(cudaMemcpyAsync(lu_.p, val, P.nent * sizeof(double), cudaMemcpyDeviceToDevice, s));
    status_.alloc(1);
    status_.zero(s);
    DBuf<int>& status = status_;
    for (size_t l = 0; l + 1 < h_lptr_.size(); ++l) {
        const int cnt = h_lptr_[l + 1] - h_lptr_[l];
        PORSOL_LAUNCH(k_ilu_factor_level<<<div_up(cnt, 128), 128, 0, s>>>(cnt, lrows_.p + h_lptr_[l], P.slice_ptr.p, P.col.p,
                                                            P.rowlen.p, P.diag.p, lu_.p, status.p));
    }
    PORSOL_CUDA(cudaGetLastError());
    int st = 0;
    PORSOL_CUDA(cudaMemcpyAsync(&st, status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    PORSOL_CUDA(cudaStreamSynchronize(s));
    PORSOL_REQUIRE(st == 0, PORSOL_ERR_NONFINITE, "ILU0: zero or non-finite pivot");
}

void Ilu0::apply(cudaStream_t s, const double* r, double* z, const int* stop)
{
    const SellPattern& P = *P_;
    for (size_t l = 0; l + 1 < h_lptr_.size(); ++l) {
        const int cnt = h_lptr_[l + 1] - h_lptr_[l];
        chain(k_ilu_lower_level, div_up(cnt, 128), 128, 0, s, cnt, lrows_.p + h_lptr_[l], P.slice_ptr.p, P.col.p,
            P.diag.p, lu_.p, r, z, stop);
    }
    for (size_t l = 0; l + 1 < h_uptr_.size(); ++l) {
        const int cnt = h_uptr_[l + 1] - h_uptr_[l];
        chain(k_ilu_upper_level, div_up(cnt, 128), 128, 0, s, cnt, urows_.p + h_uptr_[l], P.slice_ptr.p, P.col.p,
            P.rowlen.p, P.diag.p, lu_.p, z, stop);
    }
    PORSOL_CUDA(cudaGetLastError());
}

// ---------------- helpers ----------------
void device_copy(cudaStream_t s, void* dst, const void* src, size_t bytes)
{
    if (bytes) PORSOL_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, s));
}

template <class TA, class TB>
void convert(cudaStream_t s, long long n, const TA* a, TB* b)
{
    if (n == 0) return;
    PORSOL_LAUNCH(k_convert<TA, TB><<<div_up(n, RB), RB, 0, s>>>(n, a, b));
    PORSOL_CUDA(cudaGetLastError());
}
template void convert<double, float>(cudaStream_t, long long, const double*, float*);
template void convert<float, double>(cudaStream_t, long long, const float*, double*);

void axpy_add(cudaStream_t s, int n, const double* y, double* x)
{
    if (n == 0) return;
    PORSOL_LAUNCH(k_axpy_add<<<div_up(n, RB), RB, 0, s>>>(n, y, x));
    PORSOL_CUDA(cudaGetLastError());
}


void dirichlet_guess(cudaStream_t s, const SellPattern& P, const double* val, const double* b, double* x)
{
    if (P.n == 0) return;
    PORSOL_LAUNCH(k_dirichlet_guess<<<div_up(P.n, RB), RB, 0, s>>>(P.n, P.slice_ptr.p, P.col.p, P.rowlen.p, val, b, x));
    PORSOL_CUDA(cudaGetLastError());
}

template <class T>
double norm2(cudaStream_t s, int n, const T* x, RedScratch& red)
{
    if (n == 0) return 0.0;
    const int nb = red_blocks(n);
    red.ensure(nb + 1, s);
    PORSOL_LAUNCH(k_norm2<T><<<nb, RB, 0, s>>>(n, x, red.partial.p, red.counter.p, red.partial.p + nb));
    PORSOL_CUDA(cudaGetLastError());
    double out = 0.0;
    PORSOL_CUDA(cudaMemcpyAsync(&out, red.partial.p + nb, sizeof(double), cudaMemcpyDeviceToHost, s));
    PORSOL_CUDA(cudaStreamSynchronize(s));
    return std::sqrt(out);
}
template double norm2<double>(cudaStream_t, int, const double*, RedScratch&);
template double norm2<float>(cudaStream_t, int, const float*, RedScratch&);

}  // namespace porsol
