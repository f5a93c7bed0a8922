// k_mimetic.cu -- per-cell mimetic kernels: static inner product, local Schur assembly,
// recipe gathers into the global system, flux recovery and flux post-processing.
//
// Thread-per-cell mapping.  Per-cell packed matrices are stored structure-of-arrays
// ([entry][cell]) so that a warp's loads of one entry are one coalesced transaction; the
// nf x nf local matrices live in registers (MAXNF is a compile-time bound: 6 for
// hexahedra, 12 for general cells).
#include "kernels.h"
#include "mimetic.cuh"
#include "structure.h"

namespace porsol {

namespace {

__device__ __forceinline__ void mobilities(const FluidParams& fl, const double* sat, const double* mobdens, int c,
                                           double& totmob, double& md)
{
    if (fl.model == PORSOL_FLUID_COREY2) {
        const double s = sat[c];
        const double m1 = (s * s) / fl.mu1;
        const double m2 = ((1.0 - s) * (1.0 - s)) / fl.mu2;
        totmob = m1 + m2;                       // MimeticIPEvaluator.hpp:308
        md = fl.rho1 * m1 + fl.rho2 * m2;       // :309-310
    } else {
        totmob = sat[c];
        md = mobdens ? mobdens[c] : 0.0;
    }
}

// MimeticIPEvaluator::buildStaticContrib (MimeticIPEvaluator.hpp:201-270): W of every cell
// (cell_frame and projected in mimetic.cuh) and the gravity flux gflux = N K g.
template <int MAXNF>
__global__ void __launch_bounds__(128) k_static_ip(int nc, const int* __restrict__ facepos,
                                                   const double* __restrict__ area, const double* __restrict__ fcent,
                                                   const double* __restrict__ fnormal,
                                                   const double* __restrict__ cvol,
                                                   const double* __restrict__ ccent,
                                                   const double* __restrict__ perm, double g0, double g1,
                                                   double g2, double* __restrict__ W, double* __restrict__ gflux,
                                                   int* status)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int f0 = facepos[c];
    const int nf = facepos[c + 1] - f0;
    if (nf > MAXNF) {
        atomicOr(status, ST_BAD_INDEX);
        return;
    }
    double K[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) K[k] = perm[9 * (size_t)c + k];
    const double Kg0 = K[0] * g0 + K[1] * g1 + K[2] * g2;
    const double Kg1 = K[3] * g0 + K[4] * g1 + K[5] * g2;
    const double Kg2 = K[6] * g0 + K[7] * g1 + K[8] * g2;
    double N[MAXNF][3], Q[MAXNF][3], a[MAXNF];
    if (!cell_frame<MAXNF>(c, f0, nf, area, fcent, fnormal, ccent, a, N, Q))
        atomicOr(status, ST_NONFINITE);   // degenerate cell: the reference asserts here
#pragma unroll
    for (int i = 0; i < MAXNF; ++i)
        if (i < nf) gflux[f0 + i] = N[i][0] * Kg0 + N[i][1] * Kg1 + N[i][2] * Kg2;
    // NK = N K (stored back into N's slot after use is not possible; keep separate)
    double NK[MAXNF][3];
#pragma unroll
    for (int i = 0; i < MAXNF; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) NK[i][j] = N[i][0] * K[j] + N[i][1] * K[3 + j] + N[i][2] * K[6 + j];
    const double t = 6.0 * (K[0] + K[4] + K[8]) / 3.0;
    const double vol = cvol[c];
    const double a1 = 1.0 / vol, a2 = t / vol;
    bool finite = true;
#pragma unroll
    for (int j = 0; j < MAXNF; ++j) {
#pragma unroll
        for (int i = 0; i <= j; ++i) {
            if (j < nf) {
                const double nkn = NK[i][0] * N[j][0] + NK[i][1] * N[j][1] + NK[i][2] * N[j][2];
                const double w = a2 * projected<MAXNF>(i, j, a, Q) + a1 * nkn;
                finite = finite && isfinite(w);
                W[(size_t)pk(i, j) * nc + c] = w;
            }
        }
    }
    if (!finite) atomicOr(status, ST_NONFINITE);
}

// MimeticIPAnisoRelpermEvaluator (MimeticIPAnisoRelpermEvaluator.hpp:207-400), evaluated per
// solve: W = (N (lambda_t K) N^T + 2 tr(lambda_t K) A (I - Q Q^T) A) / |c| with the cell's total
// mobility tensor lambda_t, and the gravity flux N (sum_i rho_i lambda_i) K g.  W is stored
// packed (upper triangle), so lambda_t K must be symmetric (lambda_t commuting with K); a
// non-symmetric product raises ST_BAD_INDEX.
template <int MAXNF>
__global__ void __launch_bounds__(128) k_dynamic_ip_tensor(TensorIpArgs A)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= A.nc) return;
    const int nc = A.nc;
    const int f0 = A.facepos[c];
    const int nf = A.facepos[c + 1] - f0;
    if (nf > MAXNF) {
        atomicOr(A.status, ST_BAD_INDEX);
        return;
    }
    double K[9], Lm[9], LK[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        K[k] = A.perm[9 * (size_t)c + k];
        Lm[k] = A.lam[9 * (size_t)c + k];
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) LK[3 * i + j] = Lm[3 * i] * K[j] + Lm[3 * i + 1] * K[3 + j] + Lm[3 * i + 2] * K[6 + j];
    const double scale = fabs(LK[0]) + fabs(LK[4]) + fabs(LK[8]);
    if (fabs(LK[1] - LK[3]) > 1e-12 * scale || fabs(LK[2] - LK[6]) > 1e-12 * scale ||
        fabs(LK[5] - LK[7]) > 1e-12 * scale)
        atomicOr(A.status, ST_BAD_INDEX);
    double N[MAXNF][3], Q[MAXNF][3], a[MAXNF];
    if (!cell_frame<MAXNF>(c, f0, nf, A.area, A.fcent, A.fnormal, A.ccent, a, N, Q)) atomicOr(A.status, ST_NONFINITE);
    if (A.gravity) {
        const double Kg0 = K[0] * A.g0 + K[1] * A.g1 + K[2] * A.g2;
        const double Kg1 = K[3] * A.g0 + K[4] * A.g1 + K[5] * A.g2;
        const double Kg2 = K[6] * A.g0 + K[7] * A.g1 + K[8] * A.g2;
        const double* R = A.rlam + 9 * (size_t)c;
        const double d0 = R[0] * Kg0 + R[1] * Kg1 + R[2] * Kg2;
        const double d1 = R[3] * Kg0 + R[4] * Kg1 + R[5] * Kg2;
        const double d2 = R[6] * Kg0 + R[7] * Kg1 + R[8] * Kg2;
#pragma unroll
        for (int i = 0; i < MAXNF; ++i)
            if (i < nf) A.gflux[f0 + i] = N[i][0] * d0 + N[i][1] * d1 + N[i][2] * d2;
    }
    double NK[MAXNF][3];
#pragma unroll
    for (int i = 0; i < MAXNF; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) NK[i][j] = N[i][0] * LK[j] + N[i][1] * LK[3 + j] + N[i][2] * LK[6 + j];
    const double t = 6.0 * (LK[0] + LK[4] + LK[8]) / 3.0;
    const double vol = A.cvol[c];
    const double a1 = 1.0 / vol, a2 = t / vol;
    bool finite = true;
#pragma unroll
    for (int j = 0; j < MAXNF; ++j)
#pragma unroll
        for (int i = 0; i <= j; ++i)
            if (j < nf) {
                const double w = a2 * projected<MAXNF>(i, j, a, Q) +
                                 a1 * (NK[i][0] * N[j][0] + NK[i][1] * N[j][1] + NK[i][2] * N[j][2]);
                finite = finite && isfinite(w);
                A.W[(size_t)pk(i, j) * nc + c] = w;
            }
    if (!finite) atomicOr(A.status, ST_NONFINITE);
}

// assembleDynamic for one cell (IncompFlowSolverHybrid.hpp:1325-1382): dynamic scaling
// (computeDynamicParams/getInverseMatrix/gravityFlux, MimeticIPEvaluator.hpp:297-350,
// 540-546), external contributions (setExternalContrib :1736-1779), local Schur
// complement (buildCellContrib :1785-1811) and the per-row right-hand-side pieces of
// addCellContrib (:1817-1901).
template <int MAXNF>
__global__ void __launch_bounds__(128) k_assemble_cells(AssembleArgs A)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= A.nc) return;
    constexpr int NPK = MAXNF * (MAXNF + 1) / 2;
    const int nc = A.nc;
    const int f0 = A.facepos[c];
    const int nf = A.facepos[c + 1] - f0;
    double totmob, md;
    mobilities(A.fluid, A.sat, A.mobdens, c, totmob, md);
    A.totmob[c] = totmob;
    A.mobdens_out[c] = md;
    double S[NPK];
#pragma unroll
    for (int k = 0; k < NPK; ++k) S[k] = A.W[(size_t)k * nc + c] * totmob;
    double F[MAXNF], rl[MAXNF];
    int kd[MAXNF];
    double bv[MAXNF];
    double Lc = 0.0, gsum = 0.0;
#pragma unroll
    for (int j = 0; j < MAXNF; ++j) {
        F[j] = 0.0;
        rl[j] = 0.0;
        kd[j] = 0;
        bv[j] = 0.0;
        if (j < nf) {
            double s = 0.0;
#pragma unroll
            for (int i = 0; i < MAXNF; ++i)
                if (i < nf) s += S[pk(i, j)];
            F[j] = s;
            Lc += s;
            const double gf = A.gravity_zero ? 0.0 : A.gflux[f0 + j] * md;
            gsum += gf;
            kd[j] = A.kind[f0 + j];
            bv[j] = (kd[j] != HK_INTERNAL) ? A.bcval[f0 + j] : 0.0;
            const double h = (kd[j] == HK_NEUMANN) ? bv[j] : 0.0;
            rl[j] = gf - h;
        }
    }
    const double gc = A.src[c] - gsum;
    const double gl = gc / Lc;
    const double al = -1.0 / Lc;
    if (!(Lc > 0.0) || !isfinite(gl)) atomicOr(A.status, ST_NONFINITE);
#pragma unroll
    for (int j = 0; j < MAXNF; ++j) {
        rl[j] = 1.0 * rl[j] + gl * F[j];
#pragma unroll
        for (int i = 0; i <= j; ++i) S[pk(i, j)] = S[pk(i, j)] + F[i] * (al * F[j]);
    }
#pragma unroll
    for (int k = 0; k < NPK; ++k) A.sloc[(size_t)k * nc + c] = S[k];
#pragma unroll
    for (int r = 0; r < MAXNF; ++r) {
        if (r < nf) {
            const size_t hf = f0 + r;
            double rr, pbv = 0.0;
            if (kd[r] == HK_DIRICHLET) {
                rr = S[pk(r, r)] * bv[r];
            } else {
                double acc = 0.0;
#pragma unroll
                for (int cc = 0; cc < MAXNF; ++cc)
                    if (cc < nf && (kd[cc] == HK_DIRICHLET || kd[cc] == HK_PERIODIC_LO))
                        acc -= S[pk(r, cc)] * bv[cc];
                rr = acc + rl[r];
                if (kd[r] == HK_PERIODIC_HI || kd[r] == HK_PERIODIC_LO) pbv = S[pk(r, r)] * bv[r];
            }
            A.rrow[hf] = rr;
            A.pb[hf] = pbv;
            A.F[hf] = F[r];
        }
    }
    A.L[c] = Lc;
    A.g[c] = gc;
}

__global__ void k_gather_slots(long long nent, const int* __restrict__ slot_ptr, const int* __restrict__ slot_ent,
                               const double* __restrict__ sloc, double* __restrict__ val, float* __restrict__ val32)
{
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= nent) return;
    const int b = slot_ptr[k], e = slot_ptr[k + 1];
    double v = 0.0;
    for (int q = b; q < e; ++q) {
        const int x = slot_ent[q];
        v += x >= 0 ? sloc[x] : -sloc[~x];
    }
    val[k] = v;
    if (val32) val32[k] = float(v);
}

__global__ void k_gather_rhs(int n, const int* __restrict__ rhs_ptr, const int* __restrict__ rhs_ent,
                             const double* __restrict__ rrow, const double* __restrict__ pb, double* __restrict__ rhs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = 0.0;
    for (int q = rhs_ptr[i]; q < rhs_ptr[i + 1]; ++q) {
        const int x = rhs_ent[q];
        const int hf = x >> 2, kind = x & 3;
        v += kind == 0 ? rrow[hf] : (kind == 1 ? pb[hf] : -pb[hf]);
    }
    rhs[i] = v;
}

__global__ void k_scale_entry(double* val, const int* diag, int row, double factor, float* val32)
{
    const int k = diag[row];
    val[k] *= factor;
    if (val32) val32[k] = float(val[k]);
}

// computePressureAndFluxes (IncompFlowSolverHybrid.hpp:1672-1730):
//   p_c = (g_c + F . pi_c) / L_c,  v_c = totmob W_c (p_c 1 - pi_c) + mobdens gflux_c.
template <int MAXNF>
__global__ void __launch_bounds__(128) k_recover(RecoverArgs A)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= A.nc) return;
    const int nc = A.nc;
    const int f0 = A.facepos[c];
    const int nf = A.facepos[c + 1] - f0;
    double pi[MAXNF];
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < MAXNF; ++i) {
        pi[i] = 0.0;
        if (i < nf) {
            pi[i] = A.x[A.cf[f0 + i]];
            s += A.F[f0 + i] * pi[i];
        }
    }
    const double p = (A.g[c] + s) / A.L[c];
    A.pressure[c] = p;
#pragma unroll
    for (int i = 0; i < MAXNF; ++i) pi[i] = p - pi[i];
    const double tm = A.totmob[c];
    const double md = A.mobdens[c];
#pragma unroll
    for (int i = 0; i < MAXNF; ++i) {
        if (i < nf) {
            double v = 0.0;
#pragma unroll
            for (int j = 0; j < MAXNF; ++j)
                if (j < nf) v += (A.W[(size_t)pk(i, j) * nc + c] * tm) * pi[j];
            const double gfl = A.gravity_zero ? 0.0 : A.gflux[f0 + i] * md;
            A.outflux[f0 + i] = gfl + v;
        }
    }
}

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* addr, double v)
{
    atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// postProcessFluxes (IncompFlowSolverHybrid.hpp:754-807): the half-face visited first
// gets 0.5 (v1 - v2), the second its negative; returns max |v_old - v_new|.
__global__ void k_post_process(int npairs, const int* __restrict__ pairs, double* __restrict__ outflux,
                               unsigned long long* maxmod)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    double d = 0.0;
    if (k < npairs) {
        const int h1 = pairs[2 * k], h2 = pairs[2 * k + 1];
        const double v1 = outflux[h1], v2 = outflux[h2];
        const double fl = v1 - v2;
        const double n1 = 0.5 * fl, n2 = 0.5 * -1.0 * fl;
        outflux[h1] = n1;
        outflux[h2] = n2;
        d = fmax(fabs(v1 - n1), fabs(v2 - n2));
    }
    // warp max then one atomic per warp
    for (int o = 16; o > 0; o >>= 1) d = fmax(d, __shfl_xor_sync(0xffffffffu, d, o));
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(maxmod, d);
}

// Output fields of SimulatorUtilities.hpp from the solver's own buffers, one thread per cell:
//   velocity  v_c = sum_f outflux_f (x_f - x_c) / |c|         (estimateCellVelocity, :54-82)
//   phase velocities f_w v_c and (1 - f_w) v_c                 (computePhaseVelocities, :144-160)
//   fractional flow f_w = lambda_1 / (lambda_1 + lambda_2)      (Corey-2 model)
//   capillary pressure 1e5 (1 - s)                             (computeCapPressure, :214-225, with
//     ReservoirPropertyCommon_impl.hpp:466-476 when no rock table is given)
__global__ void k_cell_fields(CellFieldArgs A)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= A.nc) return;
    const double x0 = A.ccent[3 * (size_t)c], x1 = A.ccent[3 * (size_t)c + 1], x2 = A.ccent[3 * (size_t)c + 2];
    double v0 = 0.0, v1 = 0.0, v2 = 0.0;
    for (int hf = A.facepos[c]; hf < A.facepos[c + 1]; ++hf) {
        const double f = A.outflux[hf];
        v0 += f * (A.fcent[3 * (size_t)hf] - x0);
        v1 += f * (A.fcent[3 * (size_t)hf + 1] - x1);
        v2 += f * (A.fcent[3 * (size_t)hf + 2] - x2);
    }
    const double iv = 1.0 / A.cvol[c];
    v0 *= iv;
    v1 *= iv;
    v2 *= iv;
    if (A.vel) {
        A.vel[3 * (size_t)c] = v0;
        A.vel[3 * (size_t)c + 1] = v1;
        A.vel[3 * (size_t)c + 2] = v2;
    }
    if (!A.sat) return;
    const double sw = A.sat[c];
    const double m1 = sw * sw / A.mu1, m2 = (1.0 - sw) * (1.0 - sw) / A.mu2;
    const double fw = m1 / (m1 + m2);
    if (A.fw) A.fw[c] = fw;
    if (A.pc) A.pc[c] = 1e5 * (1.0 - sw);
    if (A.vw) {
        A.vw[3 * (size_t)c] = fw * v0;
        A.vw[3 * (size_t)c + 1] = fw * v1;
        A.vw[3 * (size_t)c + 2] = fw * v2;
    }
    if (A.vo) {
        A.vo[3 * (size_t)c] = (1.0 - fw) * v0;
        A.vo[3 * (size_t)c + 1] = (1.0 - fw) * v1;
        A.vo[3 * (size_t)c + 2] = (1.0 - fw) * v2;
    }
}

__global__ void k_mass_balance(int nc, const int* __restrict__ facepos, const double* __restrict__ outflux,
                               const double* __restrict__ src, unsigned long long* out)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double imb = 0.0, sq = 0.0, vm = 0.0;
    if (c < nc) {
        double s = 0.0;
        for (int hf = facepos[c]; hf < facepos[c + 1]; ++hf) {
            s += outflux[hf];
            vm = fmax(vm, fabs(outflux[hf]));
        }
        const double q = src ? src[c] : 0.0;
        imb = fabs(s - q);
        sq = fabs(q);
        if (!isfinite(s)) imb = 1e300;
    }
    for (int o = 16; o > 0; o >>= 1) {
        imb = fmax(imb, __shfl_xor_sync(0xffffffffu, imb, o));
        sq = fmax(sq, __shfl_xor_sync(0xffffffffu, sq, o));
        vm = fmax(vm, __shfl_xor_sync(0xffffffffu, vm, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomic_max_nonneg(&out[0], imb);
        atomic_max_nonneg(&out[1], sq);
        atomic_max_nonneg(&out[2], vm);
    }
}

// Pin unknown r of a consistent singular block: zero row r and column r except the diagonal
// and set rhs_r = 0, so the block solves with pi_r = 0.  For a consistent system this is the
// solution the reference's regularisation S[0][0] *= 2 selects (the doubled row is satisfied
// only with pi_r = 0); pinning keeps the block well conditioned instead of leaving one tiny
// eigenvalue.  Rows of different blocks never couple, so the threads do not interfere.
__global__ void k_pin_rows(int nrows, const int* __restrict__ rows, const int* __restrict__ sp,
                           const int* __restrict__ col, const int* __restrict__ rowlen, double* val, float* val32,
                           double* rhs)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nrows) return;
    const int r = rows[q];
    const int br = sp[r >> 5] + (r & 31);
    for (int t = 0; t < rowlen[r]; ++t) {
        const int k = br + 32 * t;
        const int j = col[k];
        if (j == r) continue;
        val[k] = 0.0;
        if (val32) val32[k] = 0.0f;
        const int bj = sp[j >> 5] + (j & 31);
        for (int u = 0; u < rowlen[j]; ++u) {
            const int kj = bj + 32 * u;
            if (col[kj] == r) {
                val[kj] = 0.0;
                if (val32) val32[kj] = 0.0f;
            }
        }
    }
    rhs[r] = 0.0;
}

// one block per sub-grid: fixed-order sums (deterministic)
__global__ void k_side_fluxes(int ngrids, const int* __restrict__ cellpos, const int* __restrict__ facepos,
                              const int* __restrict__ side, const double* __restrict__ outflux, double* __restrict__ q)
{
    __shared__ double sh[3][256];
    const int g = blockIdx.x;
    if (g >= ngrids) return;
    double acc[3] = {0.0, 0.0, 0.0};
    for (int c = cellpos[g] + threadIdx.x; c < cellpos[g + 1]; c += blockDim.x)
        for (int hf = facepos[c]; hf < facepos[c + 1]; ++hf) {
            const int sd = side[hf];
            if (sd == 2 || sd == 4 || sd == 6) acc[sd / 2 - 1] += outflux[hf];
        }
    for (int i = 0; i < 3; ++i) sh[i][threadIdx.x] = acc[i];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int i = 0; i < 3; ++i) sh[i][threadIdx.x] += sh[i][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 3) q[3 * g + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void k_compare_types(int nb, const int* __restrict__ bhf, const int* __restrict__ bct,
                                const int* __restrict__ cached, int* __restrict__ changed)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < nb && bct[bhf[q]] != cached[q]) *changed = 1;
}

__global__ void k_check_finite(long long n, const double* __restrict__ v, int* status)
{
    bool bad = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        bad |= !isfinite(v[i]);
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(status, ST_NONFINITE);
}

}  // namespace

void launch_static_ip(int maxnf, cudaStream_t s, int nc, const int* facepos, const double* area,
                      const double* fcent, const double* fnormal, const double* cvol, const double* ccent,
                      const double* perm, const double grav[3], double* W, double* gflux, int* status)
{
    if (nc == 0) return;
    const int bs = 128;
    if (maxnf <= 6)
        PORSOL_LAUNCH(k_static_ip<6><<<div_up(nc, bs), bs, 0, s>>>(nc, facepos, area, fcent, fnormal, cvol, ccent, perm, grav[0],
                                                     grav[1], grav[2], W, gflux, status));
    else
        PORSOL_LAUNCH(k_static_ip<12><<<div_up(nc, bs), bs, 0, s>>>(nc, facepos, area, fcent, fnormal, cvol, ccent, perm, grav[0],
                                                      grav[1], grav[2], W, gflux, status));
    PORSOL_CUDA(cudaGetLastError());
}

void launch_dynamic_ip_tensor(int maxnf, cudaStream_t s, const TensorIpArgs& a)
{
    if (a.nc == 0) return;
    const int bs = 128;
    if (maxnf <= 6) PORSOL_LAUNCH(k_dynamic_ip_tensor<6><<<div_up(a.nc, bs), bs, 0, s>>>(a));
    else PORSOL_LAUNCH(k_dynamic_ip_tensor<12><<<div_up(a.nc, bs), bs, 0, s>>>(a));
    PORSOL_CUDA(cudaGetLastError());
}

void launch_assemble_cells(int maxnf, cudaStream_t s, const AssembleArgs& a)
{
    if (a.nc == 0) return;
    const int bs = 128;
    if (maxnf <= 6) PORSOL_LAUNCH(k_assemble_cells<6><<<div_up(a.nc, bs), bs, 0, s>>>(a));
    else PORSOL_LAUNCH(k_assemble_cells<12><<<div_up(a.nc, bs), bs, 0, s>>>(a));
    PORSOL_CUDA(cudaGetLastError());
}

void launch_gather_slots(cudaStream_t s, long long nent, const int* slot_ptr, const int* slot_ent,
                         const double* sloc, double* val, float* val32)
{
    if (nent == 0) return;
    PORSOL_LAUNCH(k_gather_slots<<<div_up(nent, 256), 256, 0, s>>>(nent, slot_ptr, slot_ent, sloc, val, val32));
    PORSOL_CUDA(cudaGetLastError());
}

void launch_gather_rhs(cudaStream_t s, int n, const int* rhs_ptr, const int* rhs_ent, const double* rrow,
                       const double* pb, double* rhs)
{
    if (n == 0) return;
    PORSOL_LAUNCH(k_gather_rhs<<<div_up(n, 256), 256, 0, s>>>(n, rhs_ptr, rhs_ent, rrow, pb, rhs));
    PORSOL_CUDA(cudaGetLastError());
}

__global__ void k_permute(int n, const int* __restrict__ perm, const double* __restrict__ x, double* __restrict__ y,
                          int gather)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    if (gather) y[r] = x[perm[r]];
    else y[perm[r]] = x[r];
}

__global__ void k_gather_values(long long nent, const int* __restrict__ src, const double* __restrict__ val,
                                double* __restrict__ out)
{
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= nent) return;
    const int j = src[k];
    out[k] = j >= 0 ? val[j] : 0.0;
}

void launch_permute(cudaStream_t s, int n, const int* perm, const double* x, double* y, bool gather)
{
    if (n <= 0) return;
    PORSOL_LAUNCH(k_permute<<<div_up(n, 256), 256, 0, s>>>(n, perm, x, y, gather ? 1 : 0));
    PORSOL_CUDA(cudaGetLastError());
}

void launch_gather_values(cudaStream_t s, long long nent, const int* src, const double* val, double* val_ref)
{
    if (nent <= 0) return;
    PORSOL_LAUNCH(k_gather_values<<<div_up(nent, 256), 256, 0, s>>>(nent, src, val, val_ref));
    PORSOL_CUDA(cudaGetLastError());
}

void launch_scale_entry(cudaStream_t s, double* val, const int* diag, int row, double factor, float* val32)
{
    PORSOL_LAUNCH(k_scale_entry<<<1, 1, 0, s>>>(val, diag, row, factor, val32));
    PORSOL_CUDA(cudaGetLastError());
}

void launch_recover(int maxnf, cudaStream_t s, const RecoverArgs& a)
{
    if (a.nc == 0) return;
    const int bs = 128;
    if (maxnf <= 6) PORSOL_LAUNCH(k_recover<6><<<div_up(a.nc, bs), bs, 0, s>>>(a));
    else PORSOL_LAUNCH(k_recover<12><<<div_up(a.nc, bs), bs, 0, s>>>(a));
    PORSOL_CUDA(cudaGetLastError());
}

void launch_post_process(cudaStream_t s, int npairs, const int* pairs, double* outflux,
                         unsigned long long* maxmod_bits)
{
    if (npairs == 0) return;
    PORSOL_LAUNCH(k_post_process<<<div_up(npairs, 256), 256, 0, s>>>(npairs, pairs, outflux, maxmod_bits));
    PORSOL_CUDA(cudaGetLastError());
}

void launch_mass_balance(cudaStream_t s, int nc, const int* facepos, const double* outflux, const double* src,
                         unsigned long long* out3)
{
    if (nc == 0) return;
    PORSOL_LAUNCH(k_mass_balance<<<div_up(nc, 256), 256, 0, s>>>(nc, facepos, outflux, src, out3));
    PORSOL_CUDA(cudaGetLastError());
}

void launch_cell_fields(cudaStream_t s, const CellFieldArgs& a)
{
    if (a.nc == 0) return;
    PORSOL_LAUNCH(k_cell_fields<<<div_up(a.nc, 256), 256, 0, s>>>(a));
    PORSOL_CUDA(cudaGetLastError());
}

void launch_pin_rows(cudaStream_t s, int nrows, const int* rows, const int* sp, const int* col, const int* rowlen,
                     double* val, float* val32, double* rhs)
{
    if (nrows == 0) return;
    PORSOL_LAUNCH(k_pin_rows<<<div_up(nrows, 256), 256, 0, s>>>(nrows, rows, sp, col, rowlen, val, val32, rhs));
    PORSOL_CUDA(cudaGetLastError());
}

void launch_side_fluxes(cudaStream_t s, int ngrids, const int* cellpos, const int* facepos, const int* side,
                        const double* outflux, double* q)
{
    if (ngrids == 0) return;
    PORSOL_LAUNCH(k_side_fluxes<<<ngrids, 256, 0, s>>>(ngrids, cellpos, facepos, side, outflux, q));
    PORSOL_CUDA(cudaGetLastError());
}

void launch_compare_types(cudaStream_t s, int nb, const int* bhf, const int* bct, const int* cached, int* changed)
{
    if (nb == 0) return;
    PORSOL_LAUNCH(k_compare_types<<<div_up(nb, 256), 256, 0, s>>>(nb, bhf, bct, cached, changed));
    PORSOL_CUDA(cudaGetLastError());
}

void launch_check_finite(cudaStream_t s, long long n, const double* v, int* status)
{
    if (n == 0) return;
    PORSOL_LAUNCH(k_check_finite<<<std::min(div_up(n, 256), 152 * 8), 256, 0, s>>>(n, v, status));
    PORSOL_CUDA(cudaGetLastError());
}

}  // namespace porsol
