// k_transport.cu -- explicit upstream saturation transport (EulerUpstream) on the GPU.
//
// Reference: EulerUpstream::transportSolve / computeCflTime / smallTimeStep /
// checkAndPossiblyClampSat (euler/EulerUpstream_impl.hpp:153-385), the residual of
// EulerUpstreamResidual (euler/EulerUpstreamResidual_impl.hpp:101-300, 475-547) and the
// CFL estimates of cfl_calculator (euler/CflCalculator.hpp:55-170), for the scalar
// two-phase model of ReservoirPropertyCapillary: with rock tables (RockJfunc, rock.cuh) or
// without (kr1 = s^2, kr2 = (1-s)^2, pc = 1e5 (1-s); ReservoirPropertyCapillary_impl.hpp:
// 118-170, ReservoirPropertyCommon_impl.hpp:466-476).  Kernels are instantiated for both
// (template flag TAB), so the table-free path keeps its closed-form arithmetic.
//
// Layout: every face that contributes is one "face entry" (the reference visits each
// internal/periodic face once, from the lower cell index, and every Dirichlet boundary
// face).  All saturation-independent per-face factors (gravity driving force G, capillary
// geometry factor, n.n) are computed once per transportSolve.  A sub-step with gravity or
// capillarity is two kernels: face entries compute dS, then each cell gathers its entries' dS
// in a fixed order (no atomics, deterministic) and updates its saturation with the range check.
// A viscous-only sub-step is one cell kernel that evaluates its entries' terms itself.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <sstream>

#include "kernels.h"
#include "porsol_internal.h"
#include "structure.h"
#include "transport.h"

using namespace porsol;

namespace {

constexpr int TB = 256;

// UpdateForCell::operator() for one face (EulerUpstreamResidual_impl.hpp:101-291), scalar
// mobilities evaluated in the upstream cell (the boundary cell on Dirichlet faces)
template <bool TAB>
__global__ void k_face_dS(int nfe, const FaceEntry* __restrict__ fe, const double* __restrict__ sat,
                          const double* __restrict__ flux, TrParams p, RockView R, double* __restrict__ dS,
                          const int* __restrict__ status)
{
    if (*status) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nfe) return;
    const FaceEntry e = fe[k];
    const double s0 = sat[e.c0];
    const double s1 = e.dirichlet ? e.satbc : sat[e.c1];
    const double q = flux[e.hf];
    const double G = p.grav ? e.G : 0.0;
    const int triv = G >= 0.0 ? 0 : 1;
    const double sup = (q >= 0.0) ? s0 : s1;
    const int cup = (q >= 0.0) ? e.c0 : e.c1;
    double m[2];
    m[triv] = mobp<TAB>(triv, cup, sup, p, R);
    const double signG = triv == 0 ? -1.0 : 1.0;
    const double gnt = signG * m[triv] * G;
    const double supn = (q + gnt >= 0.0) ? s0 : s1;
    const int cupn = (q + gnt >= 0.0) ? e.c0 : e.c1;
    const int nt = 1 - triv;
    m[nt] = mobp<TAB>(nt, cupn, supn, p, R);
    const double mtinv = 1.0 / (m[0] + m[1]);
    double d = 0.0;
    if (p.visc) d += m[0] * mtinv * q * e.nn;
    if (p.grav && !e.dirichlet) d += m[0] * mtinv * m[1] * G;
    if (p.cap && e.capf != 0.0) {
        const double as = 0.5 * (s0 + s1);
        double a1, a2, cp0, cp1;
        if (TAB) {
            // mobilities at the mean saturation averaged over both cells' rocks (:226-236)
            a1 = 0.5 * (mobp<TAB>(0, e.c0, as, p, R) + mobp<TAB>(0, e.c1, as, p, R));
            a2 = 0.5 * (mobp<TAB>(1, e.c0, as, p, R) + mobp<TAB>(1, e.c1, as, p, R));
            cp0 = rock_pc(R, e.c0, s0);
            cp1 = rock_pc(R, e.c1, s1);
        } else {
            a1 = mob1(as, p.mu1);
            a2 = mob2(as, p.mu2);
            cp0 = 1e5 * (1.0 - s0);
            cp1 = 1e5 * (1.0 - s1);
        }
        d += a1 * (1.0 / (a1 + a2)) * a2 * e.capf * (cp1 - cp0);
    }
    dS[k] = d;
}

// Fractional flow lambda_1 / (lambda_1 + lambda_2), evaluated with the same operations as the
// viscous term of k_face_dS (m1 * (1 / (m1 + m2))), so the viscous-only sub-step is bitwise equal.
template <bool TAB>
__device__ __forceinline__ double frac1(int c, double s, const TrParams& p, const RockView& R)
{
    const double m0 = mobp<TAB>(0, c, s, p, R), m1 = mobp<TAB>(1, c, s, p, R);
    return m0 * (1.0 / (m0 + m1));
}

template <bool TAB>
__global__ void k_frac_init(int nc, const double* __restrict__ sat, TrParams p, RockView R, double* __restrict__ frac)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < nc) frac[c] = frac1<TAB>(c, sat[c], p, R);
}

// Fractional flow of each Dirichlet entry's boundary saturation, in its cell's rock
template <bool TAB>
__global__ void k_frac_bc(int nfe, const FaceEntry* __restrict__ fe, TrParams p, RockView R, double* __restrict__ fbc)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nfe && fe[k].dirichlet) fbc[k] = frac1<TAB>(fe[k].c0, fe[k].satbc, p, R);
}

// One viscous-only sub-step (no gravity driving force, no capillary term) as a single cell
// kernel.  Both phase mobilities of a face come from the same upstream cell, so its term is
// f(s_up) q n.n with the fractional flow f precomputed per cell (one FP64 division per cell, not
// per face), q the flux of the lower cell's half-face.  Every cell evaluates the terms of its own
// entries in its gather order, then updates as k_cell_update; an entry's term is evaluated by
// both its cells with the same operations, (f q) (+-n.n) = +-(f q n.n) exactly, so each cell
// sums exactly what a face-entry pass followed by the gather would give, without the per-entry
// array written and read back or a second launch per sub-step.  Fractional flows are read from
// frac_in and the updated cell's written to frac_out (a neighbour may still read the old value).
template <bool TAB>
__global__ void k_visc_substep(int nc, const int* __restrict__ cptr, const int* __restrict__ va,
                               const int* __restrict__ vb, const int* __restrict__ vhf,
                               const double* __restrict__ vcoef, const double* __restrict__ flux,
                               const double* __restrict__ frac_in, const double* __restrict__ fbc,
                               const double* __restrict__ inj, const double* __restrict__ ipv, TrParams p, RockView R,
                               double dt, int check, int clamp, double* __restrict__ sat,
                               double* __restrict__ frac_out, int* status)
{
    if (*status) return;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    double r = 0.0;
    for (int q = cptr[c]; q < cptr[c + 1]; ++q) {
        const double qf = flux[vhf[q]];
        const int b = vb[q];
        double f;
        if (qf >= 0.0) f = frac_in[va[q]];
        else f = b >= 0 ? frac_in[b] : fbc[~b];
        r += (f * qf) * vcoef[q];
    }
    const double s = sat[c];
    if (inj) {
        double rate = inj[c];
        if (rate < 0.0) {
            const double l1 = mobp<TAB>(0, c, s, p, R), l2 = mobp<TAB>(1, c, s, p, R);
            rate *= l1 / (l1 + l2);
        }
        r += rate;
    }
    double sn = s + (dt * r) * ipv[c];
    if (check || clamp) {
        if (sn > 1.0 || sn < 0.0) {
            if (clamp) sn = fmax(fmin(sn, 1.0), 0.0);
            else if (sn > 1.001 || sn < -0.001) atomicOr(status, ST_SAT_RANGE);
        }
    }
    if (!isfinite(sn)) atomicOr(status, ST_NONFINITE);
    sat[c] = sn;
    frac_out[c] = frac1<TAB>(c, sn, p, R);
}

// residual gather + smallTimeStep update + checkAndPossiblyClampSat
template <bool TAB>
__global__ void k_cell_update(int nc, const int* __restrict__ cptr, const int* __restrict__ cent,
                              const double* __restrict__ dS, const double* __restrict__ inj,
                              const double* __restrict__ ipv, TrParams p, RockView R, double dt, int check,
                              int clamp, double* __restrict__ sat, int* status)
{
    if (*status) return;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    double r = 0.0;
    for (int q = cptr[c]; q < cptr[c + 1]; ++q) {
        const int x = cent[q];
        r += x >= 0 ? dS[x] : -dS[~x];
    }
    const double s = sat[c];
    if (inj) {
        double rate = inj[c];
        if (rate < 0.0) {
            const double l1 = mobp<TAB>(0, c, s, p, R), l2 = mobp<TAB>(1, c, s, p, R);
            rate *= l1 / (l1 + l2);
        }
        r += rate;
    }
    // ipv = 1 / pore volume, precomputed at init: one FP64 division per cell and sub-step saved
    // (the update differs from s + dt r / pv by at most one rounding of the increment)
    double sn = s + (dt * r) * ipv[c];
    if (check || clamp) {
        if (sn > 1.0 || sn < 0.0) {
            if (clamp) sn = fmax(fmin(sn, 1.0), 0.0);
            else if (sn > 1.001 || sn < -0.001) atomicOr(status, ST_SAT_RANGE);
        }
    }
    if (!isfinite(sn)) atomicOr(status, ST_NONFINITE);
    sat[c] = sn;
}

// findCFLtimeVelocity (CflCalculator.hpp:55-88) and findCFLtimeGravity (:91-139) per cell
__global__ void k_cfl_cells(int nc, const int* __restrict__ facepos, const double* __restrict__ flux,
                            const double* __restrict__ gflux_hf, const double* __restrict__ vol,
                            const double* __restrict__ poro, double fac_v, double fac_g, int do_v, int do_g,
                            double* __restrict__ part, int* status)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double dv = 1e100, dg = 1e100;
    if (c < nc) {
        double fp = 0.0, fn = 0.0, fg = 0.0;
        for (int hf = facepos[c]; hf < facepos[c + 1]; ++hf) {
            const double f = flux[hf];
            if (f > 0) fp += f;
            else fn -= f;
            if (do_g) {
                const double g = gflux_hf[hf];
                if (g > 0) fg += g;
            }
        }
        if (do_v) {
            dv = (fac_v * vol[c] * poro[c]) / fmax(fn, fp);
            if (dv == 0.0) atomicOr(status, ST_CFL_ZERO);
        }
        if (do_g) dg = (fac_g * vol[c] * poro[c]) / fg;
    }
    if (!(dv >= 0.0)) dv = 1e300;   // NaN never wins the comparison in the reference
    if (!(dg >= 0.0)) dg = 1e300;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        dv = fmin(dv, __shfl_xor_sync(0xffffffffu, dv, o));
        dg = fmin(dg, __shfl_xor_sync(0xffffffffu, dg, o));
    }
    // block minimum, written to the block's slot (a second launch takes the minimum of the slots:
    // one global atomic per block on a single address serialised about 150 us at 1 M cells)
    __shared__ double sv[TB / 32], sg[TB / 32];
    if ((threadIdx.x & 31) == 0) {
        sv[threadIdx.x >> 5] = dv;
        sg[threadIdx.x >> 5] = dg;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < TB / 32; ++w) {
            dv = fmin(dv, sv[w]);
            dg = fmin(dg, sg[w]);
        }
        part[2 * blockIdx.x] = dv;
        part[2 * blockIdx.x + 1] = dg;
    }
}

// Minimum over the per-block slots of k_cfl_cells and 1e100 (order-independent: the result is exact).
__global__ void __launch_bounds__(1024) k_cfl_final(int nblocks, const double* __restrict__ part,
                                                    unsigned long long* __restrict__ out)
{
    __shared__ double sv[32], sg[32];
    double dv = 1e100, dg = 1e100;   // the initial bound of findCFLtimeVelocity / findCFLtimeGravity
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
        dv = fmin(dv, part[2 * b]);
        dg = fmin(dg, part[2 * b + 1]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        dv = fmin(dv, __shfl_xor_sync(0xffffffffu, dv, o));
        dg = fmin(dg, __shfl_xor_sync(0xffffffffu, dg, o));
    }
    if ((threadIdx.x & 31) == 0) {
        sv[threadIdx.x >> 5] = dv;
        sg[threadIdx.x >> 5] = dg;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < int(blockDim.x >> 5); ++w) {
            dv = fmin(dv, sv[w]);
            dg = fmin(dg, sg[w]);
        }
        out[0] = (unsigned long long)__double_as_longlong(dv);
        out[1] = (unsigned long long)__double_as_longlong(dg);
    }
}

}  // namespace

namespace {

// ReservoirPropertyCapillary::computeSingleRockCflFactors (ReservoirPropertyCapillary_impl.hpp:
// 213-250): 257-point sampling of the fractional flow, the gravity flow function and, with a
// rock table (rock >= 0), the capillary-pressure derivative at min_perm I and max_poro.
void single_rock_cfl(double mu1, double mu2, const RockView* R, int rock, double min_perm, double max_poro,
                     double* out)
{
    const int N = 257;
    const double delta = 1.0 / double(N - 1);
    int a = 0, n = 0;
    if (rock >= 0) {
        a = R->pos[rock];
        n = R->pos[rock + 1] - a;
    }
    auto ff = [&](double s, double& f1, double& fg) {
        double l1, l2;
        if (rock < 0) {
            l1 = (s * s) / mu1;
            l2 = ((1 - s) * (1 - s)) / mu2;
        } else {
            l1 = tab_value(R->s + a, R->krw + a, n, s) / mu1;
            l2 = tab_value(R->s + a, R->kro + a, n, s) / mu2;
        }
        f1 = l1 / (l1 + l2);
        fg = l1 * l2 / (l1 + l2);
    };
    // RockJfunc::capPressDeriv (common/RockJfunc.hpp:110-123) for perm = min_perm I
    auto dpc = [&](double s) {
        const double d = tab_slope(R->s + a, R->J + a, n, s);
        return R->jscale ? d * R->sct / std::sqrt(3 * min_perm / (3 * max_poro)) : d;
    };
    double last1, lastg, md1 = -1e100, mdg = -1e100;
    ff(0.0, last1, lastg);
    double maxffg = lastg;
    double mdpc = rock < 0 ? 0.0 : std::fabs(dpc(0.0));
    for (int i = 1; i < N; ++i) {
        const double s = double(i) * delta;
        double f1, fg;
        ff(s, f1, fg);
        md1 = std::max(md1, std::fabs(f1 - last1) / delta);
        mdg = std::max(mdg, std::fabs(fg - lastg) / delta);
        maxffg = std::max(maxffg, fg);
        if (rock >= 0) mdpc = std::max(mdpc, std::fabs(dpc(s)));
        last1 = f1;
        lastg = fg;
    }
    out[0] = 1.0 / md1;
    out[1] = 1.0 / mdg;
    out[2] = maxffg * mdpc;   // 0 without a rock table
}

}  // namespace

namespace porsol {

void launch_face_dS(cudaStream_t s, int nfe, const FaceEntry* fe, const double* sat, const double* flux,
                    const TrParams& p, const RockView& R, double* dS, const int* status)
{
    if (R.nrock > 0) PORSOL_LAUNCH(k_face_dS<true><<<div_up(nfe, TB), TB, 0, s>>>(nfe, fe, sat, flux, p, R, dS, status));
    else PORSOL_LAUNCH(k_face_dS<false><<<div_up(nfe, TB), TB, 0, s>>>(nfe, fe, sat, flux, p, R, dS, status));
}

}  // namespace porsol

// ReservoirPropertyCapillary::computeCflFactors (ReservoirPropertyCapillary_impl.hpp:255-282):
// per rock the smallest mean diagonal permeability and the largest porosity of its cells, the
// most restrictive factors over the rocks; then findCFLtimeCapillary (CflCalculator.hpp:
// 143-170), which depends on geometry, permeability and that factor only.
void porsol_transport::compute_cfl_factors()
{
    const double mu1 = fluid.viscosity1, mu2 = fluid.viscosity2;
    dt_capillary = 1e100;
    if (rock_h.nrock == 0) {
        single_rock_cfl(mu1, mu2, nullptr, -1, 0.0, 0.0, fac);
        return;
    }
    const int nr = rock_h.nrock, nc = g.nc;
    std::vector<double> min_perm(nr, 1e100), max_poro(nr, 0.0);
    for (int c = 0; c < nc; ++c) {
        const int r = rk_cell_h[c];
        const double* K = &perm[9 * size_t(c)];
        min_perm[r] = std::min(min_perm[r], (K[0] + K[4] + K[8]) / 3.0);
        max_poro[r] = std::max(max_poro[r], poro[c]);
    }
    fac[0] = 1e100;
    fac[1] = 1e100;
    fac[2] = 0.0;
    for (int r = 0; r < nr; ++r) {
        double f[3];
        single_rock_cfl(mu1, mu2, &rock_h, r, min_perm[r], max_poro[r], f);
        fac[0] = std::min(fac[0], f[0]);
        fac[1] = std::min(fac[1], f[1]);
        fac[2] = std::max(fac[2], f[2]);
    }
    double dt = 1e100;
    for (int c = 0; c < nc; ++c)
        for (int f = g.facepos[c]; f < g.facepos[c + 1]; ++f) {
            double Kl[9];
            const int c1 = g.nb[f];
            for (int k = 0; k < 9; ++k)
                Kl[k] = g.boundary(f) ? perm[9 * size_t(c) + k]
                                      : 0.5 * (perm[9 * size_t(c) + k] + perm[9 * size_t(c1) + k]);
            // inverse3x3 (MatrixInverse.hpp:85) by cofactors
            const double det = Kl[0] * (Kl[4] * Kl[8] - Kl[5] * Kl[7]) - Kl[1] * (Kl[3] * Kl[8] - Kl[5] * Kl[6]) +
                               Kl[2] * (Kl[3] * Kl[7] - Kl[4] * Kl[6]);
            double Ki[9];
            Ki[0] = (Kl[4] * Kl[8] - Kl[5] * Kl[7]) / det;
            Ki[1] = (Kl[2] * Kl[7] - Kl[1] * Kl[8]) / det;
            Ki[2] = (Kl[1] * Kl[5] - Kl[2] * Kl[4]) / det;
            Ki[3] = (Kl[5] * Kl[6] - Kl[3] * Kl[8]) / det;
            Ki[4] = (Kl[0] * Kl[8] - Kl[2] * Kl[6]) / det;
            Ki[5] = (Kl[2] * Kl[3] - Kl[0] * Kl[5]) / det;
            Ki[6] = (Kl[3] * Kl[7] - Kl[4] * Kl[6]) / det;
            Ki[7] = (Kl[1] * Kl[6] - Kl[0] * Kl[7]) / det;
            Ki[8] = (Kl[0] * Kl[4] - Kl[1] * Kl[3]) / det;
            double x[3];
            for (int d = 0; d < 3; ++d) x[d] = g.fcent[3 * size_t(f) + d] - g.ccent[3 * size_t(c) + d];
            double sc = 0.0;
            for (int i = 0; i < 3; ++i) sc += x[i] * (Ki[3 * i] * x[0] + Ki[3 * i + 1] * x[1] + Ki[3 * i + 2] * x[2]);
            dt = std::min(dt, sc / fac[2]);
        }
    dt_capillary = dt;
}

void porsol_transport::set_rock_tables(const porsol_rock_tables* rt)
{
    PORSOL_REQUIRE(ready, PORSOL_ERR_STATE, "transport solver not initialised");
    if (!rt) {
        rock = RockView{};
        rock_h = RockView{};
        compute_cfl_factors();
        return;
    }
    const int nr = rt->num_rocks, nc = g.nc;
    PORSOL_REQUIRE(nr >= 1 && rt->table_pos && rt->s && rt->krw && rt->kro && rt->jfunc && rt->cell_rock,
                   PORSOL_ERR_BAD_ARG, "rock tables: no rock or null array");
    PORSOL_REQUIRE(rt->table_pos[0] == 0, PORSOL_ERR_BAD_ARG, "rock tables: table_pos[0] must be 0");
    for (int r = 0; r < nr; ++r)
        PORSOL_REQUIRE(rt->table_pos[r + 1] > rt->table_pos[r], PORSOL_ERR_BAD_ARG, "rock tables: empty table");
    PORSOL_REQUIRE(!rt->use_jfunction_scaling || (std::isfinite(rt->sigma_cos_theta) && rt->sigma_cos_theta != 0.0),
                   PORSOL_ERR_BAD_ARG, "rock tables: sigma cos(theta) must be finite and non-zero");
    const int m = rt->table_pos[nr];
    rk_pos_h.assign(rt->table_pos, rt->table_pos + nr + 1);
    rk_s_h.assign(rt->s, rt->s + m);
    rk_krw_h.assign(rt->krw, rt->krw + m);
    rk_kro_h.assign(rt->kro, rt->kro + m);
    rk_J_h.assign(rt->jfunc, rt->jfunc + m);
    rk_Jx_h.resize(m);
    rk_sy_h.resize(m);
    for (int r = 0; r < nr; ++r) {
        const int a = rk_pos_h[r], b = rk_pos_h[r + 1];
        for (int k = a; k < b; ++k)
            PORSOL_REQUIRE(std::isfinite(rk_s_h[k]) && std::isfinite(rk_krw_h[k]) && std::isfinite(rk_kro_h[k]) &&
                               std::isfinite(rk_J_h[k]),
                           PORSOL_ERR_BAD_ARG, "rock tables: non-finite entry");
        for (int k = a + 1; k < b; ++k)
            PORSOL_REQUIRE(rk_s_h[k] >= rk_s_h[k - 1], PORSOL_ERR_BAD_ARG, "rock tables: saturations must increase");
        // the reader's fix-ups (RockJfunc.hpp:200-207)
        rk_krw_h[a] = 0.0;
        rk_kro_h[b - 1] = 0.0;
        const bool inc = rk_J_h[b - 1] >= rk_J_h[a];
        for (int k = a + 1; k < b; ++k)
            PORSOL_REQUIRE(inc ? rk_J_h[k] >= rk_J_h[k - 1] : rk_J_h[k] <= rk_J_h[k - 1], PORSOL_ERR_BAD_ARG,
                           "rock tables: J must be monotone");
        for (int k = 0; k < b - a; ++k) {
            const int src = inc ? a + k : b - 1 - k;
            rk_Jx_h[a + k] = rk_J_h[src];
            rk_sy_h[a + k] = rk_s_h[src];
        }
    }
    rk_cell_h.assign(rt->cell_rock, rt->cell_rock + nc);
    for (int c = 0; c < nc; ++c)
        PORSOL_REQUIRE(rk_cell_h[c] >= 0 && rk_cell_h[c] < nr, PORSOL_ERR_BAD_ARG, "rock tables: rock index out of range");
    rk_skp_h.resize(nc);
    for (int c = 0; c < nc; ++c) {
        const double* K = &perm[9 * size_t(c)];
        rk_skp_h[c] = std::sqrt((K[0] + K[4] + K[8]) / (3 * poro[c]));
    }
    cudaStream_t s = stream;
    rk_pos.upload(rk_pos_h, s);
    rk_s.upload(rk_s_h, s);
    rk_krw.upload(rk_krw_h, s);
    rk_kro.upload(rk_kro_h, s);
    rk_J.upload(rk_J_h, s);
    rk_Jx.upload(rk_Jx_h, s);
    rk_sy.upload(rk_sy_h, s);
    rk_cell.upload(rk_cell_h, s);
    rk_skp.upload(rk_skp_h, s);
    PORSOL_CUDA(cudaStreamSynchronize(s));
    auto view = [&](bool dev) {
        RockView v;
        v.nrock = nr;
        v.pos = dev ? rk_pos.p : rk_pos_h.data();
        v.s = dev ? rk_s.p : rk_s_h.data();
        v.krw = dev ? rk_krw.p : rk_krw_h.data();
        v.kro = dev ? rk_kro.p : rk_kro_h.data();
        v.J = dev ? rk_J.p : rk_J_h.data();
        v.Jx = dev ? rk_Jx.p : rk_Jx_h.data();
        v.sy = dev ? rk_sy.p : rk_sy_h.data();
        v.cell = dev ? rk_cell.p : rk_cell_h.data();
        v.skp = dev ? rk_skp.p : rk_skp_h.data();
        v.jscale = rt->use_jfunction_scaling ? 1 : 0;
        v.sct = rt->sigma_cos_theta;
        return v;
    };
    rock = view(true);
    rock_h = view(false);
    compute_cfl_factors();
}

void porsol_transport::init(const porsol_grid* grid, const double* K, const double* phi, const porsol_fluid* fl,
                            const int* stype, const double* sval, const int* partner,
                            const porsol_transport_opts* opts)
{
    ready = false;
    PORSOL_REQUIRE(K && phi && fl && stype && sval, PORSOL_ERR_BAD_ARG, "transport init: null argument");
    PORSOL_REQUIRE(grid && grid->num_cells > 0, PORSOL_ERR_BAD_ARG, "grid: no cells");
    PORSOL_REQUIRE(fl->model == PORSOL_FLUID_COREY2, PORSOL_ERR_BAD_ARG,
                   "transport needs the two-phase Corey-2 fluid model");
    g.copy_from(grid);
    const int nc = g.nc, nhf = g.nhf;
    perm.assign(K, K + 9 * size_t(nc));
    poro.assign(phi, phi + nc);
    st.assign(stype, stype + nhf);
    sv.assign(sval, sval + nhf);
    pbid.assign(nhf, 0);
    if (partner) pbid.assign(partner, partner + nhf);
    fluid = *fl;
    porsol_transport_opts_default(&o);
    if (opts) o = *opts;
    rock = RockView{};   // a new grid drops earlier rock tables
    rock_h = RockView{};
    compute_cfl_factors();
    hf_cell.resize(nhf);
    int maxbid = 0;
    for (int c = 0; c < nc; ++c)
        for (int hf = g.facepos[c]; hf < g.facepos[c + 1]; ++hf) {
            hf_cell[hf] = c;
            maxbid = std::max(maxbid, g.bid[hf]);
        }
    bid_to_face.assign(maxbid + 1, -1);
    for (int hf = 0; hf < nhf; ++hf)
        if (g.boundary(hf) && st[hf] == PORSOL_BC_PERIODIC) bid_to_face[g.bid[hf]] = hf;
    for (int hf = 0; hf < nhf; ++hf)
        if (g.boundary(hf) && st[hf] != PORSOL_BC_PERIODIC)
            PORSOL_REQUIRE(st[hf] == PORSOL_BC_DIRICHLET, PORSOL_ERR_BAD_ARG,
                           "saturation boundary conditions must be Dirichlet or periodic");
    cudaStream_t s = stream;
    std::vector<double> pv(nc);
    for (int c = 0; c < nc; ++c) pv[c] = g.cvol[c] * poro[c];   // initObj (EulerUpstream_impl.hpp:120-129)
    std::vector<double> ip(nc);
    for (int c = 0; c < nc; ++c) ip[c] = 1.0 / pv[c];
    ipv.upload(ip, s);
    vol.upload(g.cvol, s);
    poro_d.upload(poro, s);
    facepos.upload(g.facepos, s);
    status.alloc(1);
    status.zero(s);
    red.alloc(2);
    grav_cached[0] = grav_cached[1] = grav_cached[2] = NAN;
    const double zero[3] = {0.0, 0.0, 0.0};
    build_entries(zero);   // face tables for zero gravity; transportSolve rebuilds only for another vector
    PORSOL_CUDA(cudaStreamSynchronize(s));
    ready = true;
}

// Build face entries for a gravity vector (G depends on it).  Host work, cached per gravity.
void porsol_transport::build_entries(const double* grav)
{
    const int nc = g.nc, nhf = g.nhf;
    const double gv[3] = {grav ? grav[0] : 0.0, grav ? grav[1] : 0.0, grav ? grav[2] : 0.0};
    if (gv[0] == grav_cached[0] && gv[1] == grav_cached[1] && gv[2] == grav_cached[2]) return;
    const double drho = fluid.density1 - fluid.density2;
    fe_h.clear();
    std::vector<std::vector<int>> cl(nc);
    std::vector<double> ghf(nhf, 0.0);
    for (int c0 = 0; c0 < nc; ++c0) {
        for (int f = g.facepos[c0]; f < g.facepos[c0 + 1]; ++f) {
            // gravity CFL flux per half-face (CflCalculator.hpp:100-131)
            {
                const int c1 = g.nb[f];
                double Kl[9];
                for (int k = 0; k < 9; ++k)
                    Kl[k] = g.boundary(f) ? perm[9 * size_t(c0) + k]
                                          : 0.5 * (perm[9 * size_t(c0) + k] + perm[9 * size_t(c1) + k]);
                const double* n = &g.fnormal[3 * size_t(f)];
                double gf = 0.0;
                for (int k = 0; k < 3; ++k)
                    for (int q = 0; q < 3; ++q) gf += n[q] * (Kl[3 * q + k] * gv[k] * drho);
                ghf[f] = gf * g.area[f];
            }
            int c1, nbface = f, dir = 0;
            double sbc = 0.0;
            if (g.boundary(f)) {
                if (st[f] == PORSOL_BC_PERIODIC) {
                    const int pb = pbid[f];
                    PORSOL_REQUIRE(pb >= 0 && pb < int(bid_to_face.size()) && bid_to_face[pb] >= 0,
                                   PORSOL_ERR_BAD_ARG, "periodic saturation partner not found");
                    nbface = bid_to_face[pb];
                    c1 = hf_cell[nbface];
                    if (c0 > c1) continue;
                } else {
                    c1 = c0;
                    dir = 1;
                    sbc = sv[f];
                }
            } else {
                c1 = g.nb[f];
                if (c0 > c1) continue;
            }
            FaceEntry e{};
            e.c0 = c0;
            e.c1 = c1;
            e.hf = f;
            e.dirichlet = dir;
            e.satbc = sbc;
            const double* n = &g.fnormal[3 * size_t(f)];
            const double A = g.area[f];
            double Kav[9];
            for (int k = 0; k < 9; ++k) Kav[k] = 0.5 * (perm[9 * size_t(c0) + k] + perm[9 * size_t(c1) + k]);
            double gi[3];
            for (int i = 0; i < 3; ++i)
                gi[i] = (Kav[3 * i] * gv[0] + Kav[3 * i + 1] * gv[1] + Kav[3 * i + 2] * gv[2]) * drho;
            e.G = A * (n[0] * gi[0] + n[1] * gi[1] + n[2] * gi[2]);
            e.nn = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
            // capillary geometry (estimateCapPressureGradient, EulerUpstreamResidual_impl.hpp:512-547)
            e.capf = 0.0;
            if (!(g.boundary(f) && st[f] != PORSOL_BC_PERIODIC)) {
                const int nb = g.boundary(f) ? hf_cell[nbface] : g.nb[f];
                double d0 = 0, d1 = 0, r[3], nr = 0;
                for (int d = 0; d < 3; ++d) {
                    const double a = g.ccent[3 * size_t(c0) + d] - g.fcent[3 * size_t(f) + d];
                    const double b = g.ccent[3 * size_t(nb) + d] - g.fcent[3 * size_t(nbface) + d];
                    d0 += a * a;
                    d1 += b * b;
                    r[d] = g.ccent[3 * size_t(nb) + d] - g.fcent[3 * size_t(nbface) + d] + g.fcent[3 * size_t(f) + d] -
                           g.ccent[3 * size_t(c0) + d];
                    nr += r[d] * r[d];
                }
                nr = std::sqrt(nr);
                const double inv = 1.0 / (std::sqrt(d0) + std::sqrt(d1));
                double kr[3];
                for (int i = 0; i < 3; ++i) kr[i] = Kav[3 * i] * r[0] / nr + Kav[3 * i + 1] * r[1] / nr + Kav[3 * i + 2] * r[2] / nr;
                e.capf = A * (n[0] * kr[0] + n[1] * kr[1] + n[2] * kr[2]) * inv;
            }
            const int k = int(fe_h.size());
            fe_h.push_back(e);
            cl[c0].push_back(~k);
            if (c1 != c0) cl[c1].push_back(k);
        }
    }
    std::vector<int> cp(nc + 1, 0), ce;
    for (int c = 0; c < nc; ++c) cp[c + 1] = cp[c] + int(cl[c].size());
    ce.reserve(cp[nc]);
    for (int c = 0; c < nc; ++c) ce.insert(ce.end(), cl[c].begin(), cl[c].end());
    // the same entries seen from each cell, for the single-kernel viscous sub-step
    std::vector<int> va(ce.size()), vb(ce.size()), vh(ce.size());
    std::vector<double> vc(ce.size());
    for (size_t q = 0; q < ce.size(); ++q) {
        const int x = ce[q], k = x >= 0 ? x : ~x;
        const FaceEntry& e = fe_h[size_t(k)];
        va[q] = e.c0;
        vb[q] = e.dirichlet ? ~k : e.c1;
        vh[q] = e.hf;
        vc[q] = x >= 0 ? e.nn : -e.nn;
    }
    any_gravity = false;
    for (const FaceEntry& e : fe_h) any_gravity = any_gravity || e.G != 0.0;
    cudaStream_t s = stream;
    fe.upload(fe_h, s);
    cptr.upload(cp, s);
    cent.upload(ce, s);
    ve_a.upload(va, s);
    ve_b.upload(vb, s);
    ve_hf.upload(vh, s);
    ve_coef.upload(vc, s);
    gflux_hf.upload(ghf, s);
    dS.alloc(std::max<size_t>(fe_h.size(), 1));
    PORSOL_CUDA(cudaStreamSynchronize(s));
    grav_cached[0] = gv[0];
    grav_cached[1] = gv[1];
    grav_cached[2] = gv[2];
}

void porsol_transport::solve(double* sat, double time, const double* grav, const double* flux, const double* inj,
                             porsol_transport_stats* stats, bool dev)
{
    NvtxRange range("porsol transportSolve");
    PORSOL_REQUIRE(ready, PORSOL_ERR_STATE, "transport solver not initialised");
    PORSOL_REQUIRE(sat && flux, PORSOL_ERR_BAD_ARG, "transportSolve: null argument");
    build_entries(grav);
    const int nc = g.nc, nhf = g.nhf;
    cudaStream_t s = stream;
    double* d_sat;
    const double *d_flux, *d_inj = nullptr;
    if (dev) {
        d_sat = sat;
        d_flux = flux;
        d_inj = inj;
    } else {
        in_sat.upload(sat, nc, s);
        d_sat = in_sat.p;
        in_flux.upload(flux, nhf, s);
        d_flux = in_flux.p;
        if (inj) {
            in_inj.upload(inj, nc, s);
            d_inj = in_inj.p;
        }
    }
    const double gv[3] = {grav ? grav[0] : 0.0, grav ? grav[1] : 0.0, grav ? grav[2] : 0.0};
    // computeCflTime (EulerUpstream_impl.hpp:265-331)
    double dtv = 1e99, dtg = 1e99, dtc = 1e99;
    const int do_v = o.method_viscous && o.use_cfl_viscous;
    const int do_g = o.method_gravity && o.use_cfl_gravity;
    const int do_c = o.method_capillary && o.use_cfl_capillary;
    if (do_v || do_g) {
        const int nbk = div_up(nc, TB);
        cfl_part.alloc(2 * size_t(nbk));
        PORSOL_LAUNCH(k_cfl_cells<<<nbk, TB, 0, s>>>(nc, facepos.p, d_flux, gflux_hf.p, vol.p, poro_d.p, fac[0], fac[1],
                                                  do_v, do_g, cfl_part.p, status.p));
        PORSOL_LAUNCH(k_cfl_final<<<1, 1024, 0, s>>>(nbk, cfl_part.p, red.p));
        PORSOL_CUDA(cudaGetLastError());
        unsigned long long out[2];
        int stt = 0;
        PORSOL_CUDA(cudaMemcpyAsync(out, red.p, sizeof(out), cudaMemcpyDeviceToHost, s));
        PORSOL_CUDA(cudaMemcpyAsync(&stt, status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        PORSOL_CUDA(cudaStreamSynchronize(s));
        if (stt & ST_CFL_ZERO) {
            status.zero(s);
            throw Error(PORSOL_ERR_CFL, "Cfl computation gave dt = 0.0");
        }
        double v[2];
        std::memcpy(v, out, sizeof(v));
        if (do_v) dtv = v[0];
        if (do_g) dtg = v[1];
    }
    if (do_c) {
        // findCFLtimeCapillary (CflCalculator.hpp:143-170) depends on the geometry and the rock
        // tables only (computed when they are set); without tables cflFactorCapillary is zero,
        // every local bound is +inf and the estimate keeps its initial value 1e100.
        dtc = dt_capillary;
    }
    (void)gv;
    const double cfl_dt = std::min(std::min(dtv, dtg), dtc) * o.courant_number;
    int n;
    if (cfl_dt > time) {
        n = o.minimum_small_steps;
    } else {
        const double steps = std::min<double>(std::ceil(time / cfl_dt), double(std::numeric_limits<int>::max()));
        n = int(steps);
        n = std::max(n, o.minimum_small_steps);
        n = std::min(n, o.maximum_small_steps);
    }
    double dt = time / n;
    sat0.alloc(nc);
    PORSOL_CUDA(cudaMemcpyAsync(sat0.p, d_sat, nc * sizeof(double), cudaMemcpyDeviceToDevice, s));
    const TrParams p = params(o.method_viscous, o.method_gravity, o.method_capillary);
    const bool tab = rock.nrock > 0;
    const int nfe = int(fe_h.size());
    // viscous-only sub-steps use the per-cell fractional flow (same arithmetic, fewer FP64 ops)
    const bool visc_only = o.method_viscous && !o.method_capillary && (!o.method_gravity || !any_gravity);
    if (visc_only) {
        frac.alloc(nc);
        frac2.alloc(nc);
        fbc.alloc(std::max(nfe, 1));
        if (nfe) {
            if (tab) PORSOL_LAUNCH(k_frac_bc<true><<<div_up(nfe, TB), TB, 0, s>>>(nfe, fe.p, p, rock, fbc.p));
            else PORSOL_LAUNCH(k_frac_bc<false><<<div_up(nfe, TB), TB, 0, s>>>(nfe, fe.p, p, rock, fbc.p));
        }
    }
    int repeats = 0;
    const int max_repeats = 10;
    while (true) {
        if (visc_only) {
            if (tab) PORSOL_LAUNCH(k_frac_init<true><<<div_up(nc, TB), TB, 0, s>>>(nc, d_sat, p, rock, frac.p));
            else PORSOL_LAUNCH(k_frac_init<false><<<div_up(nc, TB), TB, 0, s>>>(nc, d_sat, p, rock, frac.p));
            for (int q = 0; q < n; ++q) {
                const double* fin = (q & 1) ? frac2.p : frac.p;
                double* fout = (q & 1) ? frac.p : frac2.p;
                if (tab)
                    PORSOL_LAUNCH(k_visc_substep<true><<<div_up(nc, TB), TB, 0, s>>>(
                        nc, cptr.p, ve_a.p, ve_b.p, ve_hf.p, ve_coef.p, d_flux, fin, fbc.p, d_inj, ipv.p, p, rock, dt,
                        o.check_sat, o.clamp_sat, d_sat, fout, status.p));
                else
                    PORSOL_LAUNCH(k_visc_substep<false><<<div_up(nc, TB), TB, 0, s>>>(
                        nc, cptr.p, ve_a.p, ve_b.p, ve_hf.p, ve_coef.p, d_flux, fin, fbc.p, d_inj, ipv.p, p, rock, dt,
                        o.check_sat, o.clamp_sat, d_sat, fout, status.p));
                if ((q & 255) == 255) PORSOL_CUDA(cudaGetLastError());
            }
        }
        for (int q = 0; q < (visc_only ? 0 : n); ++q) {
            if (nfe) launch_face_dS(s, nfe, fe.p, d_sat, d_flux, p, rock, dS.p, status.p);
            if (tab)
                PORSOL_LAUNCH(k_cell_update<true><<<div_up(nc, TB), TB, 0, s>>>(
                    nc, cptr.p, cent.p, dS.p, d_inj, ipv.p, p, rock, dt, o.check_sat, o.clamp_sat, d_sat, status.p));
            else
                PORSOL_LAUNCH(k_cell_update<false><<<div_up(nc, TB), TB, 0, s>>>(
                    nc, cptr.p, cent.p, dS.p, d_inj, ipv.p, p, rock, dt, o.check_sat, o.clamp_sat, d_sat, status.p));
            if ((q & 255) == 255) PORSOL_CUDA(cudaGetLastError());
        }
        PORSOL_CUDA(cudaGetLastError());
        int stt = 0;
        PORSOL_CUDA(cudaMemcpyAsync(&stt, status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        PORSOL_CUDA(cudaStreamSynchronize(s));
        if (stt == 0) break;
        status.zero(s);
        if (stt & ST_NONFINITE) throw Error(PORSOL_ERR_NONFINITE, "non-finite saturation in transport");
        ++repeats;
        if (repeats > max_repeats) {
            PORSOL_CUDA(cudaMemcpyAsync(d_sat, sat0.p, nc * sizeof(double), cudaMemcpyDeviceToDevice, s));
            PORSOL_CUDA(cudaStreamSynchronize(s));
            throw Error(PORSOL_ERR_SAT_RANGE, "Saturation out of range in EulerUpstream");
        }
        n *= 2;   // "Transport failed, retrying with more steps." (EulerUpstream_impl.hpp:200-211)
        dt = time / n;
        PORSOL_CUDA(cudaMemcpyAsync(d_sat, sat0.p, nc * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
    if (!dev) {
        PORSOL_CUDA(cudaMemcpyAsync(sat, d_sat, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
        PORSOL_CUDA(cudaStreamSynchronize(s));
    }
    if (stats) {
        stats->small_steps = n;
        stats->repeats = repeats;
        stats->cfl_dt = cfl_dt;
    }
}


extern "C" {

void porsol_transport_opts_default(porsol_transport_opts* o)
{
    if (!o) return;
    o->courant_number = 0.5;
    o->method_viscous = o->method_gravity = o->method_capillary = 1;
    o->use_cfl_viscous = o->use_cfl_gravity = o->use_cfl_capillary = 1;
    o->minimum_small_steps = 1;
    o->maximum_small_steps = 10000;
    o->check_sat = 1;
    o->clamp_sat = 0;
}

int porsol_transport_create(porsol_transport** out)
{
    if (!out) return PORSOL_ERR_BAD_ARG;
    *out = nullptr;
    auto* t = new (std::nothrow) porsol_transport();
    if (!t) return PORSOL_ERR_BAD_ARG;
    if (cudaGetDevice(&t->device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete t;
        return PORSOL_ERR_CUDA;
    }
    *out = t;
    return PORSOL_OK;
}

void porsol_transport_destroy(porsol_transport* t)
{
    if (!t) return;
    cudaSetDevice(t->device);
    cudaStreamSynchronize(t->stream);
    cudaStream_t s = t->stream;
    delete t;
    cudaStreamDestroy(s);
}

const char* porsol_transport_last_error(const porsol_transport* t) { return t ? t->err.c_str() : "null handle"; }

int porsol_transport_init(porsol_transport* t, const porsol_grid* grid, const double* perm, const double* poro,
                          const porsol_fluid* fluid, const int* st, const double* sv, const int* partner,
                          const porsol_transport_opts* opts)
{
    return tguard(t, [&] { t->init(grid, perm, poro, fluid, st, sv, partner, opts); });
}

int porsol_transport_solve(porsol_transport* t, double* sat, double time, const double* grav, const double* outflux,
                           const double* injection, porsol_transport_stats* stats)
{
    return tguard(t, [&] { t->solve(sat, time, grav, outflux, injection, stats, false); });
}

int porsol_transport_solve_device(porsol_transport* t, double* sat, double time, const double* grav,
                                  const double* outflux, const double* injection, porsol_transport_stats* stats)
{
    return tguard(t, [&] { t->solve(sat, time, grav, outflux, injection, stats, true); });
}

int porsol_transport_set_options(porsol_transport* t, const porsol_transport_opts* opts)
{
    return tguard(t, [&] {
        PORSOL_REQUIRE(opts, PORSOL_ERR_BAD_ARG, "transport options: null argument");
        t->o = *opts;
    });
}

int porsol_transport_set_rock_tables(porsol_transport* t, const porsol_rock_tables* rocks)
{
    return tguard(t, [&] { t->set_rock_tables(rocks); });
}

}  // extern "C"
