// transport.h -- the transport-solver handle behind the C ABI (EulerUpstream, and the
// ImplicitCapillarity step that reuses its residual and rock tables).
#pragma once

#include <vector>

#include "porsol_internal.h"
#include "rock.cuh"
#include "structure.h"

namespace porsol {

struct FaceEntry {
    int c0, c1, hf;     // cells (c1 == c0 on Dirichlet faces) and the half-face of c0
    int dirichlet;
    double satbc;       // Dirichlet saturation
    double G;           // A n . (Kavg g) (rho1 - rho2)
    double capf;        // A n . (Kavg e) / (d0 + d1), e the unit centre-to-centre direction
    double nn;          // n . n
};

struct TrParams {
    double mu1, mu2;   // reciprocal viscosities 1/mu1, 1/mu2
    int visc, grav, cap;
};

// kr_i / mu_i with the reciprocal viscosities precomputed (FP64 division is a multi-FMA
// sequence on this GPU; the products differ from the quotients by at most one rounding)
__device__ __forceinline__ double mob1(double s, double imu1) { return (s * s) * imu1; }
__device__ __forceinline__ double mob2(double s, double imu2) { return ((1.0 - s) * (1.0 - s)) * imu2; }

// mobility of phase 0/1 of cell c: the rock table of the cell (TAB) or Corey-2
template <bool TAB>
__device__ __forceinline__ double mobp(int phase, int c, double s, const TrParams& p, const RockView& R)
{
    if (TAB) return rock_kr(R, phase, c, s) * (phase == 0 ? p.mu1 : p.mu2);
    return phase == 0 ? mob1(s, p.mu1) : mob2(s, p.mu2);
}

// dS of every face entry (UpdateForCell::operator(), EulerUpstreamResidual_impl.hpp:101-291)
void launch_face_dS(cudaStream_t s, int nfe, const FaceEntry* fe, const double* sat, const double* flux,
                    const TrParams& p, const RockView& R, double* dS, const int* status);

}  // namespace porsol

struct porsol_transport {
    cudaStream_t stream = nullptr;
    int device = 0;
    std::string err;
    bool ready = false;
    porsol::HostGrid g;
    std::vector<double> perm, poro;
    std::vector<int> st;
    std::vector<double> sv;
    std::vector<int> pbid;
    porsol_fluid fluid{};
    porsol_transport_opts o{};
    double fac[3] = {0, 0, 0};
    std::vector<int> bid_to_face;   // last periodic half-face with each bid
    std::vector<int> hf_cell;
    std::vector<porsol::FaceEntry> fe_h;
    double grav_cached[3] = {NAN, NAN, NAN};
    porsol::DBuf<porsol::FaceEntry> fe;
    porsol::DBuf<int> cptr, cent, facepos, status;
    porsol::DBuf<double> ipv, vol, poro_d, dS, sat0, gflux_hf, in_sat, in_flux, in_inj, frac;
    // the viscous-only sub-step as one cell kernel: each cell's entries in its gather order (lower
    // cell, other cell or ~entry for Dirichlet faces, flux half-face, +-n.n), the fractional flow
    // of the Dirichlet entries, and a second fractional-flow buffer (read one, write the other)
    porsol::DBuf<int> ve_a, ve_b, ve_hf;
    porsol::DBuf<double> ve_coef, fbc, frac2;
    bool any_gravity = false;   // some face entry has a non-zero gravity driving force
    porsol::DBuf<unsigned long long> red;
    porsol::DBuf<double> cfl_part;   // per-block minima of the CFL bounds

    // rock tables (porsol_transport_set_rock_tables); rock.nrock == 0 without
    porsol::RockView rock;            // device pointers
    porsol::RockView rock_h;          // the same tables on the host (CFL factors)
    std::vector<int> rk_pos_h, rk_cell_h;
    std::vector<double> rk_s_h, rk_krw_h, rk_kro_h, rk_J_h, rk_Jx_h, rk_sy_h, rk_skp_h;
    porsol::DBuf<int> rk_pos, rk_cell;
    porsol::DBuf<double> rk_s, rk_krw, rk_kro, rk_J, rk_Jx, rk_sy, rk_skp;
    double dt_capillary = 1e100;      // findCFLtimeCapillary (geometry and rock only)

    // ImplicitCapillarity scratch
    porsol::DBuf<double> cap_mob, cap_src, cap_snew, cap_pvs, cap_sum, cap_part, cap_bcv, cap_bcvin, cap_sat, cap_flux,
        cap_inj;
    porsol::DBuf<int> cap_bct;

    void init(const porsol_grid* grid, const double* K, const double* phi, const porsol_fluid* fl, const int* stype,
              const double* sval, const int* partner, const porsol_transport_opts* opts);
    void set_rock_tables(const porsol_rock_tables* rt);
    void compute_cfl_factors();
    void build_entries(const double* grav);
    porsol::TrParams params(int visc, int grav, int cap) const
    {
        return porsol::TrParams{1.0 / fluid.viscosity1, 1.0 / fluid.viscosity2, visc, grav, cap};
    }
    void solve(double* sat, double time, const double* grav, const double* flux, const double* inj,
               porsol_transport_stats* stats, bool dev);
    void capillary_solve(porsol_solver* p, double* sat, const double* grav, const double* flux, const double* inj,
                         const int* bct, const double* bcv, const porsol_capillary_opts* opts,
                         porsol_capillary_stats* stats, bool dev);
};

// C-ABI guard of the transport handle: exceptions become status codes and the error text.
template <class F>
int tguard(porsol_transport* t, F&& f)
{
    if (!t) return PORSOL_ERR_BAD_ARG;
    try {
        PORSOL_CUDA(cudaSetDevice(t->device));
        f();
        t->err.clear();
        return PORSOL_OK;
    } catch (const porsol::Error& e) {
        t->err = e.what();
        return e.code;
    } catch (const std::exception& e) {
        t->err = e.what();
        return PORSOL_ERR_BAD_ARG;
    }
}
