// k_batch.cu -- BatchedPcg: one preconditioned CG per block of a block-diagonal system.
//
// Per iteration (captured into one CUDA graph): q = A p; per block pq_g and lambda_g =
// rholast_g / pq_g; x += lambda p, r -= lambda q; per block ||r_g|| and the stopping test;
// z = M r; per block rho_g = z_g . r_g and beta_g; p = z + beta p.  Block sums are computed by
// one CTA per block over the block's two unknown ranges in a fixed order, so results are
// reproducible.  The CTA of the last block to finish the residual norms counts the active
// blocks and raises the stop flag (device word read by every kernel, mirrored in mapped host
// memory for the host loop).  A block that meets its tolerance, or whose curvature p.Ap is not
// positive, is frozen (lambda = 0).
#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "batch.h"
#include "sell.cuh"

namespace porsol {

namespace {

constexpr int BT = 256;

template <class V>
__device__ __forceinline__ V warp_sum(V v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Threads of the per-block CTAs (one CTA per block sums the block's ranges): a block holds up to
// about 10^5 unknowns, and its CTA alone sets the time of the launch.
constexpr int RT = 1024;

// Sum of a_i * b_i over block g's two ranges in a fixed order; the total is returned in thread 0.
// Thread t keeps four running sums over the elements t + RT (4m + u), u = 0..3, of each range, so
// eight loads are in flight per thread (one running sum put one memory latency on every RT
// elements: 115 us for a 98 k-unknown block).
template <class T>
__device__ double seg_dot(const int* __restrict__ rg, int g, const T* __restrict__ a, const T* __restrict__ b)
{
    __shared__ double ws[RT / 32];
    T v0 = T(0), v1 = T(0), v2 = T(0), v3 = T(0);
    for (int part = 0; part < 2; ++part) {
        const int hi = rg[4 * g + 2 * part + 1];
        int i = rg[4 * g + 2 * part] + threadIdx.x;
        for (; i + 3 * RT < hi; i += 4 * RT) {
            const T a0 = a[i], a1 = a[i + RT], a2 = a[i + 2 * RT], a3 = a[i + 3 * RT];
            const T b0 = b[i], b1 = b[i + RT], b2 = b[i + 2 * RT], b3 = b[i + 3 * RT];
            v0 += a0 * b0;
            v1 += a1 * b1;
            v2 += a2 * b2;
            v3 += a3 * b3;
        }
        for (; i < hi; i += RT) v0 += a[i] * b[i];
    }
    const double w = double(warp_sum<T>((v0 + v1) + (v2 + v3)));
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = w;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < RT / 32; ++k) t += ws[k];
    return t;
}

__device__ __forceinline__ void publish(BatchDev* st, BatchHostView* hv)
{
    hv->iter = st->iter;
    hv->active = st->active;
    hv->breakdown = st->breakdown;
    hv->stop = st->stop;
    __threadfence_system();
}

// After every block has written conv: the last CTA to arrive counts active blocks, updates
// the iteration count and the stop flag.
__device__ void finish_round(int nblk, const int* conv, BatchDev* st, unsigned int* counter, BatchHostView* hv,
                             bool count_iteration)
{
    __shared__ bool last;
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(counter, 1u) == unsigned(nblk - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    int act = 0, brk = 0;
    for (int g = threadIdx.x; g < nblk; g += RT) {
        const int c = ((volatile const int*)conv)[g];
        act += c == 0;
        brk |= c == 2;
    }
    __shared__ int sa[RT / 32], sb[RT / 32];
    const int wa = warp_sum<int>(act), wb = __any_sync(0xffffffffu, brk);
    if ((threadIdx.x & 31) == 0) {
        sa[threadIdx.x >> 5] = wa;
        sb[threadIdx.x >> 5] = wb;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int A = 0, Bk = 0;
        for (int k = 0; k < RT / 32; ++k) {
            A += sa[k];
            Bk |= sb[k];
        }
        if (count_iteration) st->iter += 1;
        st->active = A;
        st->breakdown = Bk;
        st->stop = (A == 0) || st->iter >= st->maxit;
        *counter = 0u;
        publish(st, hv);
    }
}

template <class T>
__global__ void __launch_bounds__(RT) k_b_init(int nblk, const int* __restrict__ rg, const T* __restrict__ r,
                                               double* def0, double* def, int* conv, BatchDev* st,
                                               unsigned int* counter, BatchHostView* hv)
{
    const int g = blockIdx.x;
    const double s = seg_dot<T>(rg, g, r, r);
    if (threadIdx.x == 0) {
        const double d = sqrt(s);
        def0[g] = d;
        def[g] = d;
        conv[g] = !isfinite(d) ? 2 : (d < 1e-30 ? 1 : 0);
    }
    finish_round(nblk, conv, st, counter, hv, false);
}

template <class T>
__global__ void __launch_bounds__(RT) k_b_pq(const int* __restrict__ rg, const T* __restrict__ p,
                                             const T* __restrict__ q, const double* __restrict__ rholast,
                                             int* conv, double* lambda, const BatchDev* st)
{
    if (st->stop) return;
    const int g = blockIdx.x;
    if (conv[g] != 0) {   // frozen block (every thread reads conv[g] before thread 0 may change it)
        if (threadIdx.x == 0) lambda[g] = 0.0;
        return;
    }
    const double s = seg_dot<T>(rg, g, p, q);
    if (threadIdx.x == 0) {
        double l = 0.0;
        if (conv[g] == 0) {
            if (!(s > 0.0) || !isfinite(s)) conv[g] = 2;
            else l = rholast[g] / s;
        }
        lambda[g] = l;
    }
}

template <class T>
__global__ void k_b_update(int n, const int* __restrict__ blk, const double* __restrict__ lambda, T* __restrict__ x,
                           T* __restrict__ r, const T* __restrict__ p, const T* __restrict__ q, const BatchDev* st)
{
    if (st->stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const T l = T(lambda[blk[i]]);
    if (l != T(0)) {
        x[i] += l * p[i];
        r[i] -= l * q[i];
    }
}

template <class T>
__global__ void __launch_bounds__(RT) k_b_rr(int nblk, const int* __restrict__ rg, const T* __restrict__ r,
                                             const double* __restrict__ def0, double* def,
                                             const double* __restrict__ tol, int* conv, BatchDev* st,
                                             unsigned int* counter, BatchHostView* hv)
{
    if (st->stop) return;
    const int g = blockIdx.x;
    const bool live = conv[g] == 0;   // uniform in the CTA: read before thread 0 may change it
    const double s = live ? seg_dot<T>(rg, g, r, r) : 0.0;
    if (threadIdx.x == 0 && live) {
        const double d = sqrt(s);
        def[g] = d;
        if (!isfinite(d)) conv[g] = 2;
        else if (d < tol[g] * def0[g] || d < 1e-30) conv[g] = 1;
    }
    finish_round(nblk, conv, st, counter, hv, true);
}

template <class T>
__global__ void __launch_bounds__(RT) k_b_zr(const int* __restrict__ rg, const T* __restrict__ z,
                                             const T* __restrict__ r, double* rholast, double* beta,
                                             const int* __restrict__ conv, int first, const BatchDev* st)
{
    if (st->stop) return;
    const int g = blockIdx.x;
    if (!first && conv[g] != 0) {   // frozen block: its direction is no longer used
        if (threadIdx.x == 0) beta[g] = 0.0;
        return;
    }
    const double s = seg_dot<T>(rg, g, z, r);
    if (threadIdx.x == 0) {
        const double rl = rholast[g];
        beta[g] = (first || conv[g] != 0 || rl == 0.0) ? 0.0 : s / rl;
        rholast[g] = s;
    }
}

template <class T>
__global__ void k_b_direction(int n, const int* __restrict__ blk, const double* __restrict__ beta,
                              const T* __restrict__ z, T* __restrict__ p, const BatchDev* st)
{
    if (st->stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = z[i] + T(beta[blk[i]]) * p[i];
}

template <class TV, class T>
__global__ void k_b_residual(int n, const int* __restrict__ sp, const int* __restrict__ col,
                             const TV* __restrict__ val, const T* __restrict__ x, const T* __restrict__ b,
                             T* __restrict__ r)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    r[i] = b[i] - sell_dot<T>(sp, col, val, i, [x](int j) { return x[j]; });
}

template <class TV, class T>
__global__ void k_b_spmv(int n, const int* __restrict__ sp, const int* __restrict__ col, const TV* __restrict__ val,
                         const T* __restrict__ p, T* __restrict__ q, const int* __restrict__ blk,
                         const int* __restrict__ conv, const BatchDev* st)
{
    if (st->stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || conv[blk[i]] != 0) return;   // a frozen block's q is not used
    q[i] = sell_dot<T>(sp, col, val, i, [p](int j) { return p[j]; });
}

template <class T>
__global__ void __launch_bounds__(RT) k_b_norms(const int* __restrict__ rg, const T* __restrict__ a,
                                                double* __restrict__ out)
{
    const double s = seg_dot<T>(rg, blockIdx.x, a, a);
    if (threadIdx.x == 0) out[blockIdx.x] = sqrt(s);
}

__global__ void k_b_cast_in(int n, const int* __restrict__ blk, const double* __restrict__ r,
                            const double* __restrict__ sc, float* __restrict__ r32, const int* stop)
{
    if (*stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) r32[i] = float(r[i] * sc[blk[i]]);
}

__global__ void k_b_cast_out(int n, const int* __restrict__ blk, const float* __restrict__ z32,
                             const double* __restrict__ isc, double* __restrict__ z, const int* stop)
{
    if (*stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) z[i] = double(z32[i]) * isc[blk[i]];
}

}  // namespace

void BatchCastPrecond::bind(Precond<float>* inner, const BatchRanges* B, const double* sc, const double* isc)
{
    const float* r0 = r32_.p;
    const float* z0 = z32_.p;
    r32_.alloc(B->n);
    z32_.alloc(B->n);
    // captured graphs hold these pointers: a change of any of them is a new generation
    if (inner != m_ || inner->generation() != inner_gen_ || B != B_ || sc != sc_ || isc != isc_ || r0 != r32_.p ||
        z0 != z32_.p)
        bump_generation();
    m_ = inner;
    B_ = B;
    sc_ = sc;
    isc_ = isc;
    inner_gen_ = inner->generation();
}

void BatchCastPrecond::set_block_state(const int* conv)
{
    if (!m_) return;
    m_->set_block_state(conv);
    if (m_->generation() != inner_gen_) {   // captured graphs hold the inner kernels
        inner_gen_ = m_->generation();
        bump_generation();
    }
}

void BatchCastPrecond::apply(cudaStream_t s, const double* r, double* z, const int* stop)
{
    const int n = B_->n;
    PORSOL_LAUNCH(k_b_cast_in<<<div_up(n, BT), BT, 0, s>>>(n, B_->blk.p, r, sc_, r32_.p, stop));
    m_->apply(s, r32_.p, z32_.p, stop);
    PORSOL_LAUNCH(k_b_cast_out<<<div_up(n, BT), BT, 0, s>>>(n, B_->blk.p, z32_.p, isc_, z, stop));
}

void BatchRanges::build(const std::vector<int>& four, int n_unknowns, cudaStream_t s)
{
    PORSOL_REQUIRE(four.size() % 4 == 0, PORSOL_ERR_BAD_ARG, "batch ranges: four entries per block");
    nblk = int(four.size() / 4);
    n = n_unknowns;
    h = four;
    std::vector<int> b(n, -1);
    for (int g = 0; g < nblk; ++g)
        for (int k = 0; k < 2; ++k) {
            const int r0 = four[4 * g + 2 * k], r1 = four[4 * g + 2 * k + 1];
            PORSOL_REQUIRE(0 <= r0 && r0 <= r1 && r1 <= n, PORSOL_ERR_BAD_ARG, "batch ranges out of bounds");
            for (int i = r0; i < r1; ++i) {
                PORSOL_REQUIRE(b[i] < 0, PORSOL_ERR_BAD_ARG, "batch ranges overlap");
                b[i] = g;
            }
        }
    for (int i = 0; i < n; ++i) PORSOL_REQUIRE(b[i] >= 0, PORSOL_ERR_BAD_ARG, "batch ranges do not cover every unknown");
    ranges.upload(four, s);
    blk.upload(b, s);
}

template <class TV, class T>
void BatchedPcg<TV, T>::setup(int n, int nblk, cudaStream_t s)
{
    if (n != n_) {
        r_.alloc(n);
        z_.alloc(n);
        p_.alloc(n);
        q_.alloc(n);
        n_ = n;
    }
    if (nblk != nblk_) {
        rho_.alloc(nblk);
        rholast_.alloc(nblk);
        lambda_.alloc(nblk);
        beta_.alloc(nblk);
        def0_.alloc(nblk);
        def_.alloc(nblk);
        conv_.alloc(nblk);
        nblk_ = nblk;
    }
    st_.alloc(1);
    if (!counter_.p) {
        counter_.alloc(1);
        counter_.zero(s);
    }
    if (!hview_) {
        PORSOL_CUDA(cudaHostAlloc((void**)&hview_, sizeof(BatchHostView), cudaHostAllocMapped));
        PORSOL_CUDA(cudaHostGetDevicePointer((void**)&dview_, hview_, 0));
    }
    if (ev_.empty()) {
        ev_.resize(4);
        for (auto& e : ev_) PORSOL_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
}

template <class TV, class T>
BatchedPcg<TV, T>::~BatchedPcg()
{
    if (exec_) cudaGraphExecDestroy(exec_);
    if (hview_) cudaFreeHost(hview_);
    for (auto& e : ev_) cudaEventDestroy(e);
}

template <class TV, class T>
void BatchedPcg<TV, T>::iteration(cudaStream_t s, const SellPattern& P, const TV* val, Precond<T>& M,
                                  const BatchRanges& B, T* x, const double* tol)
{
    const int n = P.n, nb = div_up(n, BT), g = B.nblk;
    const int* stop = &st_.p->stop;
    PORSOL_LAUNCH(k_b_spmv<TV, T><<<nb, BT, 0, s>>>(n, P.slice_ptr.p, P.col.p, val, p_.p, q_.p, B.blk.p, conv_.p,
                                                    st_.p));
    PORSOL_LAUNCH(k_b_pq<T><<<g, RT, 0, s>>>(B.ranges.p, p_.p, q_.p, rholast_.p, conv_.p, lambda_.p, st_.p));
    PORSOL_LAUNCH(k_b_update<T><<<nb, BT, 0, s>>>(n, B.blk.p, lambda_.p, x, r_.p, p_.p, q_.p, st_.p));
    PORSOL_LAUNCH(k_b_rr<T><<<g, RT, 0, s>>>(g, B.ranges.p, r_.p, def0_.p, def_.p, tol, conv_.p, st_.p, counter_.p,
                                             dview_));
    M.apply(s, r_.p, z_.p, stop);
    PORSOL_LAUNCH(k_b_zr<T><<<g, RT, 0, s>>>(B.ranges.p, z_.p, r_.p, rholast_.p, beta_.p, conv_.p, 0, st_.p));
    PORSOL_LAUNCH(k_b_direction<T><<<nb, BT, 0, s>>>(n, B.blk.p, beta_.p, z_.p, p_.p, st_.p));
}

template <class TV, class T>
CgResult BatchedPcg<TV, T>::solve(cudaStream_t s, const SellPattern& P, const TV* val, Precond<T>& M,
                                  const BatchRanges& B, const T* b, T* x, const double* tol, int maxit)
{
    const int n = P.n;
    CgResult res;
    PORSOL_REQUIRE(B.n == n && B.nblk > 0, PORSOL_ERR_BAD_ARG, "batched CG: ranges do not match the system");
    setup(n, B.nblk, s);
    // a block-diagonal preconditioner skips the converged blocks' rows (PORSOL_BLOCK_SKIP=0 in the
    // environment: it sweeps every row, with the same results)
    const char* skip_env = std::getenv("PORSOL_BLOCK_SKIP");
    M.set_block_state(skip_env && skip_env[0] == '0' ? nullptr : conv_.p);
    const int nb = div_up(n, BT), g = B.nblk;
    BatchDev init{};
    init.maxit = maxit;
    PORSOL_CUDA(cudaMemcpyAsync(st_.p, &init, sizeof(BatchDev), cudaMemcpyHostToDevice, s));
    p_.zero(s);
    PORSOL_LAUNCH(k_b_residual<TV, T><<<nb, BT, 0, s>>>(n, P.slice_ptr.p, P.col.p, val, x, b, r_.p));
    PORSOL_LAUNCH(k_b_init<T><<<g, RT, 0, s>>>(g, B.ranges.p, r_.p, def0_.p, def_.p, conv_.p, st_.p, counter_.p,
                                               dview_));
    const int* stop = &st_.p->stop;
    M.apply(s, r_.p, z_.p, stop);
    PORSOL_LAUNCH(k_b_zr<T><<<g, RT, 0, s>>>(B.ranges.p, z_.p, r_.p, rholast_.p, beta_.p, conv_.p, 1, st_.p));
    PORSOL_LAUNCH(k_b_direction<T><<<nb, BT, 0, s>>>(n, B.blk.p, beta_.p, z_.p, p_.p, st_.p));
    PORSOL_CUDA(cudaGetLastError());
    const void* key[6] = {&P, val, x, (const void*)&M, (const void*)&B, tol};
    bool same = exec_ && key_gen_ == M.generation();
    for (int k = 0; k < 6 && same; ++k) same = key_[k] == key[k];
    if (!same) {
        if (exec_) {
            cudaGraphExecDestroy(exec_);
            exec_ = nullptr;
        }
        cudaGraph_t gr;
        const long long l0 = g_launches.load();
        PORSOL_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        iteration(s, P, val, M, B, x, tol);
        PORSOL_CUDA(cudaStreamEndCapture(s, &gr));
        nodes_ = g_launches.load() - l0;
        g_launches.fetch_sub(nodes_);
        PORSOL_CUDA(cudaGraphInstantiate(&exec_, gr, 0));
        PORSOL_CUDA(cudaGraphDestroy(gr));
        for (int k = 0; k < 6; ++k) key_[k] = key[k];
        key_gen_ = M.generation();
    }
    // Same host loop as PcgSolver: iterations queued two ahead, stop read from mapped memory.
    const int LOOKAHEAD = 2;
    int it = 0;
    bool done = false;
    while (!done) {
        if (it < maxit) {
            PORSOL_CUDA(cudaGraphLaunch(exec_, s));
            g_launches.fetch_add(nodes_);
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
    res.breakdown = hview_->breakdown != 0;
    res.converged = hview_->active == 0 && !res.breakdown;
    std::vector<double> d0(g), d1(g);
    def0_.download(d0.data(), g, s);
    def_.download(d1.data(), g, s);
    PORSOL_CUDA(cudaStreamSynchronize(s));
    double red = 0.0, s0 = 0.0, s1 = 0.0;
    for (int k = 0; k < g; ++k) {
        if (d0[k] > 0) red = std::max(red, d1[k] / d0[k]);
        s0 += d0[k] * d0[k];
        s1 += d1[k] * d1[k];
    }
    res.reduction = red;
    res.def0 = std::sqrt(s0);
    res.def = std::sqrt(s1);
    return res;
}

template class BatchedPcg<double, double>;

template <class T>
void batch_norms(cudaStream_t s, const BatchRanges& B, const T* a, double* out)
{
    PORSOL_LAUNCH(k_b_norms<T><<<B.nblk, RT, 0, s>>>(B.ranges.p, a, out));
    PORSOL_CUDA(cudaGetLastError());
}
template void batch_norms<double>(cudaStream_t, const BatchRanges&, const double*, double*);
template void batch_norms<float>(cudaStream_t, const BatchRanges&, const float*, double*);

}  // namespace porsol
