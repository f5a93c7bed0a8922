// k_capillary.cu -- ImplicitCapillarity::transportSolve on the GPU.
//
// Reference: euler/ImplicitCapillarity_impl.hpp:138-247 with
// euler/MatchSaturatedVolumeFunctor.hpp:49-112.  One step is: capillary mobilities per cell,
// the viscous/gravity upstream residual of the transport solver as source, one pressure solve
// (the pressure handle's assembly, AMG/ILU0 CG and recovery) for the capillary pressure, then a
// scalar root search for the constant shift of the capillary pressure that keeps the
// pore-volume-weighted saturation.  Every evaluation of that function is one per-cell kernel
// (inverse capillary-pressure curve) and a deterministic sum; only the scalar crosses to the
// host.
//
// The root search restates the published methods the reference takes from opm-core's
// RootFinders (not part of the reference tree): a bracket search that steps away from 0 by
// the capillary-pressure range, alternating sides and doubling the step until the sign changes
// (at most 100 trials), then false position with the Pegasus modification (Dowell & Jarratt,
// BIT 12 (1972) 503-508), stopping at |f| <= 1e-12, at most 40 iterations (:205-210).
#include <algorithm>
#include <cmath>
#include <vector>

#include "kernels.h"
#include "solver.h"
#include "transport.h"

using namespace porsol;

namespace {

constexpr int TB = 256;
constexpr int MINMAX_BLOCKS = 1024;

// lambda_1 (1 / (lambda_1 + lambda_2)) lambda_2, at least 1e-10 (:148-165)
template <bool TAB>
__global__ void k_cap_mob(int nc, const double* __restrict__ sat, TrParams p, RockView R, double* __restrict__ mob)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const double s = sat[c];
    const double m1 = mobp<TAB>(0, c, s, p, R), m2 = mobp<TAB>(1, c, s, p, R);
    mob[c] = fmax((m1 * (1.0 / (m1 + m2))) * m2, 1e-10);
}

// computeResidual without the capillary term (:176-183), negated: per cell the ordered gather
// of the face terms plus the source (producers scaled by the fractional flow)
template <bool TAB>
__global__ void k_cap_source(int nc, const int* __restrict__ cptr, const int* __restrict__ cent,
                             const double* __restrict__ dS, const double* __restrict__ inj,
                             const double* __restrict__ sat, TrParams p, RockView R, double* __restrict__ src)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    double r = 0.0;
    for (int q = cptr[c]; q < cptr[c + 1]; ++q) {
        const int x = cent[q];
        r += x >= 0 ? dS[x] : -dS[~x];
    }
    if (inj) {
        double rate = inj[c];
        if (rate < 0.0) {
            const double s = sat[c];
            const double l1 = mobp<TAB>(0, c, s, p, R), l2 = mobp<TAB>(1, c, s, p, R);
            rate *= l1 / (l1 + l2);
        }
        r += rate;
    }
    src[c] = -r;
}

// periodic flow conditions get a zero jump (:168-174); other values are kept
__global__ void k_cap_bcv(int nhf, const int* __restrict__ bct, const double* __restrict__ bcv, double* __restrict__ out)
{
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h < nhf) out[h] = bct[h] == PORSOL_BC_PERIODIC ? 0.0 : bcv[h];
}

// pore volume and pore-volume-weighted saturation per cell (poreSatVolumes, :49-63)
__global__ void k_cap_volumes(int nc, const double* __restrict__ vol, const double* __restrict__ poro,
                              const double* __restrict__ sat, double* __restrict__ pv, double* __restrict__ pvs)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const double v = vol[c] * poro[c];
    pv[c] = v;
    pvs[c] = v * sat[c];
}

// MatchSaturatedVolumeFunctor::computeSaturations at shift dp (:88-109); without rock tables
// saturationFromCapillaryPressure is 0 (ReservoirPropertyCommon_impl.hpp:518-528)
template <bool TAB>
__global__ void k_cap_sat(int nc, const double* __restrict__ pc, double dp, RockView R, const double* __restrict__ vol,
                          const double* __restrict__ poro, double* __restrict__ snew, double* __restrict__ pvs)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const double s = TAB ? rock_sat(R, c, pc[c] + dp) : 0.0;
    snew[c] = s;
    pvs[c] = (vol[c] * poro[c]) * s;
}

// per-block minimum and maximum (grid-stride), finished on the host
__global__ void k_minmax(int n, const double* __restrict__ x, double* __restrict__ part)
{
    double lo = 1e300, hi = -1e300;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        lo = fmin(lo, x[i]);
        hi = fmax(hi, x[i]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    __shared__ double sl[TB / 32], sh[TB / 32];
    if ((threadIdx.x & 31) == 0) {
        sl[threadIdx.x >> 5] = lo;
        sh[threadIdx.x >> 5] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < TB / 32; ++w) {
            lo = fmin(lo, sl[w]);
            hi = fmax(hi, sh[w]);
        }
        part[2 * blockIdx.x] = lo;
        part[2 * blockIdx.x + 1] = hi;
    }
}

// relaxation (:213-217) and checkAndPossiblyClampSat (:234-247), into snew
__global__ void k_cap_update(int nc, const double* __restrict__ sat, double* __restrict__ snew, double w, int check,
                             int clamp, int* status)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    double s = (1.0 - w) * sat[c] + w * snew[c];
    if (check || clamp) {
        if (s > 1.0 || s < 0.0) {
            if (clamp) s = fmax(fmin(s, 1.0), 0.0);
            else if (s > 1.001 || s < -0.001) atomicOr(status, ST_SAT_RANGE);
        }
    }
    if (!isfinite(s)) atomicOr(status, ST_NONFINITE);
    snew[c] = s;
}

}  // namespace

void porsol_transport::capillary_solve(porsol_solver* P, double* sat, const double* grav, const double* flux,
                                       const double* inj, const int* bct, const double* bcv,
                                       const porsol_capillary_opts* opts_in, porsol_capillary_stats* stats, bool dev)
{
    NvtxRange range("porsol ImplicitCapillarity step");
    PORSOL_REQUIRE(ready, PORSOL_ERR_STATE, "transport solver not initialised");
    PORSOL_REQUIRE(P && sat && flux && bct && bcv, PORSOL_ERR_BAD_ARG, "capillary solve: null argument");
    P->require_structure();
    PORSOL_REQUIRE(P->ip_valid, PORSOL_ERR_STATE, "capillary solve: the pressure solver has no inner products");
    PORSOL_REQUIRE(P->S.g.nc == g.nc && P->S.g.nhf == g.nhf, PORSOL_ERR_BAD_ARG,
                   "capillary solve: pressure and transport solvers are on different grids");
    PORSOL_REQUIRE(P->gravity_zero, PORSOL_ERR_BAD_ARG,
                   "capillary solve: the pressure solver must hold zero-gravity inner products");
    porsol_capillary_opts o;
    porsol_capillary_opts_default(&o);
    if (opts_in) o = *opts_in;
    build_entries(grav);
    const int nc = g.nc, nhf = g.nhf;
    cudaStream_t s = stream;
    const double* d_sat;
    const double *d_flux, *d_inj = nullptr, *d_bcv;
    const int* d_bct;
    if (dev) {
        d_sat = sat;
        d_flux = flux;
        d_inj = inj;
        d_bct = bct;
        d_bcv = bcv;
    } else {
        cap_sat.upload(sat, nc, s);
        d_sat = cap_sat.p;
        cap_flux.upload(flux, nhf, s);
        d_flux = cap_flux.p;
        if (inj) {
            cap_inj.upload(inj, nc, s);
            d_inj = cap_inj.p;
        }
        cap_bct.upload(bct, nhf, s);
        d_bct = cap_bct.p;
        cap_bcvin.upload(bcv, nhf, s);   // the copy with zeroed periodic jumps goes to cap_bcv
        d_bcv = cap_bcvin.p;
    }
    const bool tab = rock.nrock > 0;
    const TrParams p = params(o.method_viscous, o.method_gravity, 0);
    cap_mob.alloc(nc);
    cap_src.alloc(nc);
    cap_bcv.alloc(nhf);
    if (tab) PORSOL_LAUNCH(k_cap_mob<true><<<div_up(nc, TB), TB, 0, s>>>(nc, d_sat, p, rock, cap_mob.p));
    else PORSOL_LAUNCH(k_cap_mob<false><<<div_up(nc, TB), TB, 0, s>>>(nc, d_sat, p, rock, cap_mob.p));
    const int nfe = int(fe_h.size());
    if (nfe) launch_face_dS(s, nfe, fe.p, d_sat, d_flux, p, rock, dS.p, status.p);
    if (tab)
        PORSOL_LAUNCH(k_cap_source<true><<<div_up(nc, TB), TB, 0, s>>>(nc, cptr.p, cent.p, dS.p, d_inj, d_sat, p, rock,
                                                                     cap_src.p));
    else
        PORSOL_LAUNCH(k_cap_source<false><<<div_up(nc, TB), TB, 0, s>>>(nc, cptr.p, cent.p, dS.p, d_inj, d_sat, p, rock,
                                                                      cap_src.p));
    PORSOL_LAUNCH(k_cap_bcv<<<div_up(nhf, TB), TB, 0, s>>>(nhf, d_bct, d_bcv, cap_bcv.p));
    PORSOL_CUDA(cudaGetLastError());
    PORSOL_CUDA(cudaStreamSynchronize(s));

    // the capillary pressure: fixed mobilities, phase densities (1, 0) (:186-193,
    // ReservoirPropertyFixedMobility.hpp:55-74); gravity is zero in the pressure handle
    porsol_fluid fl{PORSOL_FLUID_CELLWISE, 1.0, 1.0, 0.0, 0.0};
    porsol_solve_opts po;
    porsol_solve_opts_default(&po);
    po.residual_tolerance = o.residual_tolerance;
    po.linsolver_verbosity = o.linsolver_verbosity;
    po.linsolver_type = o.linsolver_type;
    po.precision = o.precision;
    porsol_solve_stats pst{};
    P->solve(&fl, cap_mob.p, cap_mob.p, d_bct, cap_bcv.p, cap_src.p, &po, &pst, true);
    PORSOL_CUDA(cudaStreamSynchronize(P->stream));
    const double* pc = P->pressure.p;

    // range of the capillary pressure (:200-204)
    const int nb = std::max(1, std::min(MINMAX_BLOCKS, div_up(nc, TB)));
    cap_part.alloc(2 * size_t(nb));
    PORSOL_LAUNCH(k_minmax<<<nb, TB, 0, s>>>(nc, pc, cap_part.p));
    std::vector<double> part(2 * size_t(nb));
    cap_part.download(part.data(), part.size(), s);
    // pore volume and the original saturation volume (the functor's constructor, :73-84)
    cap_snew.alloc(nc);
    cap_pvs.alloc(nc);
    cap_sum.alloc(sum_scratch_size());
    const int ri = sum_result_index(nc);
    PORSOL_LAUNCH(k_cap_volumes<<<div_up(nc, TB), TB, 0, s>>>(nc, vol.p, poro_d.p, d_sat, cap_snew.p, cap_pvs.p));
    double pv_sum = 0.0, sv0 = 0.0;
    launch_sum(s, nc, cap_snew.p, cap_sum.p);
    PORSOL_CUDA(cudaMemcpyAsync(&pv_sum, cap_sum.p + ri, sizeof(double), cudaMemcpyDeviceToHost, s));
    launch_sum(s, nc, cap_pvs.p, cap_sum.p);
    PORSOL_CUDA(cudaMemcpyAsync(&sv0, cap_sum.p + ri, sizeof(double), cudaMemcpyDeviceToHost, s));
    PORSOL_CUDA(cudaStreamSynchronize(s));
    double lo = 1e300, hi = -1e300;
    for (int b = 0; b < nb; ++b) {
        lo = std::min(lo, part[2 * b]);
        hi = std::max(hi, part[2 * b + 1]);
    }

    int evals = 0;
    auto fun = [&](double dp) {
        ++evals;
        if (tab)
            PORSOL_LAUNCH(k_cap_sat<true><<<div_up(nc, TB), TB, 0, s>>>(nc, pc, dp, rock, vol.p, poro_d.p, cap_snew.p,
                                                                      cap_pvs.p));
        else
            PORSOL_LAUNCH(k_cap_sat<false><<<div_up(nc, TB), TB, 0, s>>>(nc, pc, dp, rock, vol.p, poro_d.p, cap_snew.p,
                                                                       cap_pvs.p));
        launch_sum(s, nc, cap_pvs.p, cap_sum.p);
        double sv = 0.0;
        PORSOL_CUDA(cudaMemcpyAsync(&sv, cap_sum.p + ri, sizeof(double), cudaMemcpyDeviceToHost, s));
        PORSOL_CUDA(cudaStreamSynchronize(s));
        return (sv - sv0) / pv_sum;
    };
    // bracket search from 0 with step max - min (:205)
    const char* nobracket = "ImplicitCapillarity: no sign change of the saturation-volume mismatch found";
    double a, b;
    {
        const double x0 = 0.0, f0 = fun(x0);
        double step = hi - lo;
        bool found = false;
        for (int i = 0; i < 100 && !found; ++i) {
            const double x = x0 + step;
            if (f0 * fun(x) <= 0.0) {
                a = std::min(x0, x);
                b = std::max(x0, x);
                found = true;
            }
            step = -2.0 * step;
        }
        PORSOL_REQUIRE(found, PORSOL_ERR_NOT_CONVERGED, nobracket);
    }
    // regula falsi, Pegasus variant (:206-210)
    const int max_iter = 40;
    const double tol = 1e-12;
    int iters = 0;
    double shift;
    {
        double x0 = a, f0 = fun(x0);
        bool done = std::fabs(f0) <= tol;
        shift = x0;
        double x1 = b, f1 = 0.0;
        if (!done) {
            f1 = fun(x1);
            done = std::fabs(f1) <= tol;
            shift = x1;
        }
        if (!done) {
            PORSOL_REQUIRE(f0 * f1 <= 0.0, PORSOL_ERR_NOT_CONVERGED, nobracket);
            for (int it = 1; it <= max_iter && !done; ++it) {
                const double x = x1 - f1 * (x1 - x0) / (f1 - f0);
                const double fx = fun(x);
                iters = it;
                shift = x;
                if (std::fabs(fx) <= tol) {
                    done = true;
                    break;
                }
                if ((fx < 0.0) != (f1 < 0.0)) {
                    x0 = x1;
                    f0 = f1;
                } else {
                    f0 *= f1 / (f1 + fx);
                }
                x1 = x;
                f1 = fx;
            }
            PORSOL_REQUIRE(done, PORSOL_ERR_NOT_CONVERGED,
                           "ImplicitCapillarity: regula falsi did not converge in 40 iterations");
        }
    }
    // cap_snew holds the saturations of the last evaluation (functor.lastSaturations(), :212)
    PORSOL_LAUNCH(k_cap_update<<<div_up(nc, TB), TB, 0, s>>>(nc, d_sat, cap_snew.p, o.update_relaxation, o.check_sat,
                                                          o.clamp_sat, status.p));
    PORSOL_CUDA(cudaGetLastError());
    int stt = 0;
    PORSOL_CUDA(cudaMemcpyAsync(&stt, status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    PORSOL_CUDA(cudaStreamSynchronize(s));
    if (stt) {
        status.zero(s);
        PORSOL_CUDA(cudaStreamSynchronize(s));
        if (stt & ST_NONFINITE) throw Error(PORSOL_ERR_NONFINITE, "non-finite saturation in ImplicitCapillarity");
        throw Error(PORSOL_ERR_SAT_RANGE, "Saturation out of range in ImplicitCapillarity");
    }
    if (dev)
        PORSOL_CUDA(cudaMemcpyAsync(sat, cap_snew.p, nc * sizeof(double), cudaMemcpyDeviceToDevice, s));
    else
        PORSOL_CUDA(cudaMemcpyAsync(sat, cap_snew.p, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
    PORSOL_CUDA(cudaStreamSynchronize(s));
    if (stats) {
        stats->shift = shift;
        stats->root_iterations = iters;
        stats->evaluations = evals;
        stats->pressure = pst;
    }
}

extern "C" {

void porsol_capillary_opts_default(porsol_capillary_opts* o)
{
    if (!o) return;
    o->method_viscous = 1;
    o->method_gravity = 1;
    o->check_sat = 1;
    o->clamp_sat = 0;
    o->residual_tolerance = 1e-8;
    o->linsolver_verbosity = 1;
    o->linsolver_type = 1;
    o->update_relaxation = 1.0;
    o->precision = PORSOL_FP64;
}

int porsol_capillary_solve(porsol_transport* t, porsol_solver* p, double* sat, const double* grav,
                           const double* outflux, const double* injection, const int* hf_flow_type,
                           const double* hf_flow_value, const porsol_capillary_opts* opts,
                           porsol_capillary_stats* stats)
{
    return tguard(t, [&] {
        t->capillary_solve(p, sat, grav, outflux, injection, hf_flow_type, hf_flow_value, opts, stats, false);
    });
}

int porsol_capillary_solve_device(porsol_transport* t, porsol_solver* p, double* sat, const double* grav,
                                  const double* outflux, const double* injection, const int* hf_flow_type,
                                  const double* hf_flow_value, const porsol_capillary_opts* opts,
                                  porsol_capillary_stats* stats)
{
    return tguard(t, [&] {
        t->capillary_solve(p, sat, grav, outflux, injection, hf_flow_type, hf_flow_value, opts, stats, true);
    });
}

}  // extern "C"
