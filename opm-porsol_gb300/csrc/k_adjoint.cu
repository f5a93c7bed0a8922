// k_adjoint.cu -- adjoint of the mimetic pressure solve with respect to per-cell
// log-permeability.
//
// The solve of IncompFlowSolverHybrid (IncompFlowSolverHybrid.hpp:658-703) computes face
// pressures pi from  R(pi, k) = sum_c P_c^T (S_c pi_c - b_c) = 0  on the non-Dirichlet face
// unknowns, with the local Schur complement S_c = B - F F^T / L, B = totmob W_c(K),
// F = B 1, L = 1^T B 1, b_c = F g_c / L (buildCellContrib, :1785-1811), and recovers
// p_c = (g_c + F . pi_c) / L and v_c = B (p_c 1 - pi_c) (computePressureAndFluxes, :1672-1730).
// For an objective
//     J = sum_c w_c (p_c - p*_c)^2 + sum_hf u_hf v_hf
// the gradient is  dJ/dtheta_c = dJ/dtheta_c|_pi + mu_c . (dS_c pi_c - db_c)  with the
// adjoint mu solving  A mu = -dJ/dpi  (A = the assembled, symmetric system; mu = 0 on
// Dirichlet faces).  Only the forward solution pi is kept from the forward solve (no Krylov
// history); the adjoint solve reuses the forward preconditioner.
//
// Kernels (thread per cell, packed local matrices in registers, like k_mimetic.cu):
//   k_adjoint_source  J_c and y_c = dJ/dpi_c per half-face
//   k_adjoint_rhs     rhs_i = -sum of y over the half-faces of face i (0 on Dirichlet rows)
//   k_adjoint_grad    per-cell gradient; dB = B for d/d ln k (W is linear in K), or
//                     totmob W(k_a e_a e_a^T) for d/d ln k_a of a diagonal tensor
//   k_sum_blocks/k_sum_final  deterministic two-stage sum of J_c
#include "kernels.h"
#include "mimetic.cuh"
#include "structure.h"

namespace porsol {

namespace {

template <int MAXNF>
__global__ void __launch_bounds__(128) k_adjoint_source(AdjointArgs A)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= A.nc) return;
    constexpr int NPK = MAXNF * (MAXNF + 1) / 2;
    const int nc = A.nc;
    const int f0 = A.facepos[c];
    const int nf = A.facepos[c + 1] - f0;
    double S[NPK];
#pragma unroll
    for (int k = 0; k < NPK; ++k) S[k] = A.sloc[(size_t)k * nc + c];
    double pi[MAXNF], F[MAXNF], u[MAXNF];
#pragma unroll
    for (int i = 0; i < MAXNF; ++i) {
        pi[i] = F[i] = u[i] = 0.0;
        if (i < nf) {
            pi[i] = A.x[A.cf[f0 + i]];
            F[i] = A.F[f0 + i];
            u[i] = A.wv ? A.wv[f0 + i] : 0.0;
        }
    }
    const double Lc = A.L[c], gl = A.g[c] / Lc, p = A.pressure[c];
    const double dev = A.wp ? A.wp[c] * (p - (A.pstar ? A.pstar[c] : 0.0)) : 0.0;
    double jc = dev * (p - (A.pstar ? A.pstar[c] : 0.0));
#pragma unroll
    for (int i = 0; i < MAXNF; ++i) {
        if (i < nf) {
            double spi = 0.0, su = 0.0;
#pragma unroll
            for (int j = 0; j < MAXNF; ++j)
                if (j < nf) {
                    spi += S[pk(i, j)] * pi[j];
                    su += S[pk(i, j)] * u[j];
                }
            // v_i = F_i p - (B pi)_i = -(S pi)_i + F_i g / L  (zero gravity)
            jc += u[i] * (F[i] * gl - spi);
            // dJ/dpi_i: 2 w (p - p*) F_i / L  -  (S u)_i
            A.y[f0 + i] = 2.0 * dev * F[i] / Lc - su;
        }
    }
    A.jc[c] = jc;
}

__global__ void k_adjoint_rhs(int n, const int* __restrict__ rhs_ptr, const int* __restrict__ rhs_ent,
                              const int* __restrict__ kind, const double* __restrict__ y, double* __restrict__ rhs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = 0.0;
    bool dirichlet = false;
    for (int q = rhs_ptr[i]; q < rhs_ptr[i + 1]; ++q) {
        const int e = rhs_ent[q];
        if ((e & 3) != 0) continue;
        const int hf = e >> 2;
        dirichlet = dirichlet || kind[hf] == HK_DIRICHLET;
        v -= y[hf];
    }
    rhs[i] = dirichlet ? 0.0 : v;
}

// Gradient contribution of one derivative direction dB (packed) of cell c.
template <int MAXNF>
__device__ __forceinline__ double cell_gradient(int nf, const double* dB, const double (&pi)[MAXNF],
                                                const double (&mu)[MAXNF], const double (&F)[MAXNF],
                                                const double (&u)[MAXNF], double Lc, double gc, double p, double dev)
{
    double dF[MAXNF];
    double dL = 0.0, Fpi = 0.0, dFpi = 0.0;
#pragma unroll
    for (int i = 0; i < MAXNF; ++i) {
        dF[i] = 0.0;
        if (i < nf) {
            double s = 0.0;
#pragma unroll
            for (int j = 0; j < MAXNF; ++j)
                if (j < nf) s += dB[pk(i, j)];
            dF[i] = s;
            dL += s;
            Fpi += F[i] * pi[i];
            dFpi += s * pi[i];
        }
    }
    const double invL = 1.0 / Lc;
    const double dp = (dFpi - p * dL) * invL;
    double gsum = 2.0 * dev * dp;
#pragma unroll
    for (int i = 0; i < MAXNF; ++i) {
        if (i < nf) {
            double dBpi = 0.0;
#pragma unroll
            for (int j = 0; j < MAXNF; ++j)
                if (j < nf) dBpi += dB[pk(i, j)] * pi[j];
            const double dv = p * dF[i] - dBpi + F[i] * dp;
            const double dSpi = dBpi - (dF[i] * Fpi + F[i] * dFpi) * invL + F[i] * Fpi * dL * invL * invL;
            const double db = gc * (dF[i] - F[i] * dL * invL) * invL;
            gsum += u[i] * dv + mu[i] * (dSpi - db);
        }
    }
    return gsum;
}

template <int MAXNF>
__global__ void __launch_bounds__(128) k_adjoint_grad(AdjointArgs A)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= A.nc) return;
    constexpr int NPK = MAXNF * (MAXNF + 1) / 2;
    const int nc = A.nc;
    const int f0 = A.facepos[c];
    const int nf = A.facepos[c + 1] - f0;
    double pi[MAXNF], mu[MAXNF], F[MAXNF], u[MAXNF];
#pragma unroll
    for (int i = 0; i < MAXNF; ++i) {
        pi[i] = mu[i] = F[i] = u[i] = 0.0;
        if (i < nf) {
            const int hf = f0 + i, d = A.cf[hf];
            pi[i] = A.x[d];
            mu[i] = A.kind[hf] == HK_DIRICHLET ? 0.0 : A.mu[d];
            F[i] = A.F[hf];
            u[i] = A.wv ? A.wv[hf] : 0.0;
        }
    }
    const double Lc = A.L[c], gc = A.g[c], p = A.pressure[c], tm = A.totmob[c];
    const double dev = A.wp ? A.wp[c] * (p - (A.pstar ? A.pstar[c] : 0.0)) : 0.0;
    double dB[NPK];
    if (A.mode == 0) {
#pragma unroll
        for (int k = 0; k < NPK; ++k) dB[k] = A.W[(size_t)k * nc + c] * tm;
        A.grad[c] = cell_gradient<MAXNF>(nf, dB, pi, mu, F, u, Lc, gc, p, dev);
        return;
    }
    const double* K = A.perm + 9 * (size_t)c;
    if (K[1] != 0.0 || K[2] != 0.0 || K[3] != 0.0 || K[5] != 0.0 || K[6] != 0.0 || K[7] != 0.0) {
        atomicOr(A.status, ST_BAD_INDEX);
        return;
    }
    double a[MAXNF], N[MAXNF][3], Q[MAXNF][3];
    if (!cell_frame<MAXNF>(c, f0, nf, A.area, A.fcent, A.fnormal, A.ccent, a, N, Q)) atomicOr(A.status, ST_NONFINITE);
    const double inv_vol = 1.0 / A.cvol[c];
#pragma unroll 1
    for (int ax = 0; ax < 3; ++ax) {
        // totmob W(k_a e_a e_a^T): t = 2 k_a
        const double ka = K[4 * ax];
        const double a1 = tm * ka * inv_vol, a2 = tm * 2.0 * ka * inv_vol;
#pragma unroll
        for (int j = 0; j < MAXNF; ++j)
#pragma unroll
            for (int i = 0; i <= j; ++i) dB[pk(i, j)] = a2 * projected<MAXNF>(i, j, a, Q) + a1 * (N[i][ax] * N[j][ax]);
        A.grad[3 * (size_t)c + ax] = cell_gradient<MAXNF>(nf, dB, pi, mu, F, u, Lc, gc, p, dev);
    }
}

constexpr int SUM_THREADS = 256;

__global__ void __launch_bounds__(SUM_THREADS) k_sum_blocks(int n, const double* __restrict__ x,
                                                            double* __restrict__ partial)
{
    __shared__ double sh[SUM_THREADS / 32];
    double s = 0.0;
    for (int i = blockIdx.x * SUM_THREADS + threadIdx.x; i < n; i += gridDim.x * SUM_THREADS) s += x[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < SUM_THREADS / 32; ++w) t += sh[w];
        partial[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(SUM_THREADS) k_sum_final(int nb, double* __restrict__ partial)
{
    __shared__ double sh[SUM_THREADS / 32];
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += SUM_THREADS) s += partial[b];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < SUM_THREADS / 32; ++w) t += sh[w];
        partial[nb] = t;
    }
}

}  // namespace

void launch_adjoint_source(int maxnf, cudaStream_t s, const AdjointArgs& a)
{
    if (a.nc == 0) return;
    const int bs = 128;
    if (maxnf <= 6) PORSOL_LAUNCH(k_adjoint_source<6><<<div_up(a.nc, bs), bs, 0, s>>>(a));
    else PORSOL_LAUNCH(k_adjoint_source<12><<<div_up(a.nc, bs), bs, 0, s>>>(a));
    PORSOL_CUDA(cudaGetLastError());
}

void launch_adjoint_rhs(cudaStream_t s, int n, const int* rhs_ptr, const int* rhs_ent, const int* kind,
                        const double* y, double* rhs)
{
    if (n == 0) return;
    PORSOL_LAUNCH(k_adjoint_rhs<<<div_up(n, 256), 256, 0, s>>>(n, rhs_ptr, rhs_ent, kind, y, rhs));
    PORSOL_CUDA(cudaGetLastError());
}

void launch_adjoint_grad(int maxnf, cudaStream_t s, const AdjointArgs& a)
{
    if (a.nc == 0) return;
    const int bs = 128;
    if (maxnf <= 6) PORSOL_LAUNCH(k_adjoint_grad<6><<<div_up(a.nc, bs), bs, 0, s>>>(a));
    else PORSOL_LAUNCH(k_adjoint_grad<12><<<div_up(a.nc, bs), bs, 0, s>>>(a));
    PORSOL_CUDA(cudaGetLastError());
}

int sum_scratch_size() { return 1024 + 1; }

void launch_sum(cudaStream_t s, int n, const double* x, double* scratch)
{
    const int nb = std::max(1, std::min(1024, div_up(n, SUM_THREADS)));
    PORSOL_LAUNCH(k_sum_blocks<<<nb, SUM_THREADS, 0, s>>>(n, x, scratch));
    PORSOL_LAUNCH(k_sum_final<<<1, SUM_THREADS, 0, s>>>(nb, scratch));
    PORSOL_CUDA(cudaGetLastError());
}

int sum_result_index(int n) { return std::max(1, std::min(1024, div_up(n, SUM_THREADS))); }

}  // namespace porsol
