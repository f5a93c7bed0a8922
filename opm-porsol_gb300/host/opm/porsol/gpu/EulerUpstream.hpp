// EulerUpstream.hpp -- GB300 drop-in for Opm::EulerUpstream (explicit upstream transport).
//
// Same class template, constructors and methods as the reference
// (opm/porsol/euler/EulerUpstream.hpp:60-110, EulerUpstream_impl.hpp:95-218).  The
// parameter object of init() is any type with getDefault(key, default) -- the reference's
// Opm::parameter::ParameterGroup works unchanged, and so does the plain Params struct
// below.  The transport runs on the GPU through porsol_transport_* (include/porsol_gpu.h).
//
// The reservoir-properties concept consumed is that of ReservoirPropertyCapillary
// (ReservoirPropertyCapillary_impl.hpp:118-170): permeability(c), porosity(c),
// viscosityFirstPhase/SecondPhase(), densityFirstPhase/SecondPhase() (ReservoirPropertyCommon.hpp),
// with kr1 = s^2, kr2 = (1-s)^2 until setRockTables() hands over the RockJfunc tables.
#ifndef OPM_PORSOL_GPU_EULERUPSTREAM_HPP
#define OPM_PORSOL_GPU_EULERUPSTREAM_HPP

#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "GridFlattener.hpp"
#include "RockTables.hpp"
#include "porsol_gpu.h"

namespace Opm {
namespace gpu {

// Plain stand-in for Opm::parameter::ParameterGroup with the same getDefault() call.
struct Params {
    porsol_transport_opts o;
    Params() { porsol_transport_opts_default(&o); }
    double getDefault(const std::string& key, double def) const
    {
        if (key == "courant_number") return o.courant_number;
        return def;
    }
    int getDefault(const std::string& key, int def) const
    {
        if (key == "minimum_small_steps") return o.minimum_small_steps;
        if (key == "maximum_small_steps") return o.maximum_small_steps;
        return def;
    }
    bool getDefault(const std::string& key, bool def) const
    {
        if (key == "method_viscous") return o.method_viscous;
        if (key == "method_gravity") return o.method_gravity;
        if (key == "method_capillary") return o.method_capillary;
        if (key == "use_cfl_viscous") return o.use_cfl_viscous;
        if (key == "use_cfl_gravity") return o.use_cfl_gravity;
        if (key == "use_cfl_capillary") return o.use_cfl_capillary;
        if (key == "check_sat") return o.check_sat;
        if (key == "clamp_sat") return o.clamp_sat;
        return def;
    }
};

template <class GridInterface, class ReservoirProperties, class BoundaryConditions>
class EulerUpstream {
public:
    EulerUpstream() { create(); }
    EulerUpstream(const GridInterface& g, const ReservoirProperties& r, const BoundaryConditions& b)
    {
        create();
        initObj(g, r, b);
    }
    ~EulerUpstream() { porsol_transport_destroy(t_); }
    EulerUpstream(const EulerUpstream&) = delete;
    EulerUpstream& operator=(const EulerUpstream&) = delete;

    // EulerUpstream_impl.hpp:95-108 -- same keys and defaults
    template <class ParamGroup>
    void init(const ParamGroup& param)
    {
        o_.courant_number = param.getDefault("courant_number", o_.courant_number);
        o_.method_viscous = param.getDefault("method_viscous", bool(o_.method_viscous));
        o_.method_gravity = param.getDefault("method_gravity", bool(o_.method_gravity));
        o_.method_capillary = param.getDefault("method_capillary", bool(o_.method_capillary));
        o_.use_cfl_viscous = param.getDefault("use_cfl_viscous", bool(o_.use_cfl_viscous));
        o_.use_cfl_gravity = param.getDefault("use_cfl_gravity", bool(o_.use_cfl_gravity));
        o_.use_cfl_capillary = param.getDefault("use_cfl_capillary", bool(o_.use_cfl_capillary));
        o_.minimum_small_steps = param.getDefault("minimum_small_steps", o_.minimum_small_steps);
        o_.maximum_small_steps = param.getDefault("maximum_small_steps", o_.maximum_small_steps);
        o_.check_sat = param.getDefault("check_sat", bool(o_.check_sat));
        o_.clamp_sat = param.getDefault("clamp_sat", bool(o_.clamp_sat));
        if (ready_) check(porsol_transport_set_options(t_, &o_));
    }
    template <class ParamGroup>
    void init(const ParamGroup& param, const GridInterface& g, const ReservoirProperties& r,
              const BoundaryConditions& b)
    {
        init(param);
        initObj(g, r, b);
    }

    // EulerUpstream_impl.hpp:120-129 with EulerUpstreamResidual::initFinal
    void initObj(const GridInterface& g, const ReservoirProperties& r, const BoundaryConditions& b)
    {
        grid_ = flattenGrid(g);
        const int nc = grid_.numCells(), nhf = grid_.numHalfFaces();
        std::vector<double> K(9 * size_t(nc)), poro(nc);
        for (int p = 0; p < nc; ++p) {
            const int ci = grid_.index_of_position[p];
            const auto k = r.permeability(ci);
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) K[9 * size_t(p) + 3 * i + j] = k(i, j);
            poro[p] = r.porosity(ci);
        }
        std::vector<int> st(nhf, PORSOL_BC_DIRICHLET), partner(nhf, 0);
        std::vector<double> sv(nhf, 1.0);
        typedef typename GridInterface::CellIterator CI;
        typedef typename CI::FaceIterator FI;
        int hf = 0;
        for (CI c = g.cellbegin(); c != g.cellend(); ++c)
            for (FI f = c->facebegin(); f != c->faceend(); ++f, ++hf) {
                if (!f->boundary()) continue;
                const auto& sc = b.satCond(*f);
                if (sc.isPeriodic()) {
                    st[hf] = PORSOL_BC_PERIODIC;
                    partner[hf] = b.getPeriodicPartner(f->boundaryId());
                } else {
                    st[hf] = PORSOL_BC_DIRICHLET;
                    sv[hf] = sc.saturation();
                }
            }
        porsol_fluid fl{PORSOL_FLUID_COREY2, r.viscosityFirstPhase(), r.viscositySecondPhase(),
                        r.densityFirstPhase(), r.densitySecondPhase()};
        const porsol_grid v = grid_.view();
        check(porsol_transport_init(t_, &v, K.data(), poro.data(), &fl, st.data(), sv.data(), partner.data(), &o_));
        ready_ = true;
    }

    // EulerUpstream_impl.hpp:132-139
    void display()
    {
        std::cout << std::endl;
        std::cout << "Displaying some members of EulerUpstream" << std::endl;
        std::cout << std::endl;
        std::cout << "courant_number = " << o_.courant_number << std::endl;
    }

    // EulerUpstream_impl.hpp:143-147 (takes effect for the next transportSolve)
    void setCourantNumber(double cn)
    {
        o_.courant_number = cn;
        if (ready_) check(porsol_transport_set_options(t_, &o_));
    }

    // ReservoirPropertyCapillary with rock tables: table mobilities and capillary pressure,
    // per-rock CFL factors (call after initObj; an empty table list returns to Corey-2)
    void setRockTables(const RockTables& rt)
    {
        if (rt.rocks.empty()) check(porsol_transport_set_rock_tables(t_, nullptr));
        else check(Opm::gpu::setRockTables(t_, grid_, rt));
    }

    porsol_transport* handle() const { return t_; }
    const FlatGrid& flatGrid() const { return grid_; }

    // EulerUpstream_impl.hpp:153-218.  PressureSolution is any type with outflux(face);
    // a FlowSolution of Opm::gpu::IncompFlowSolverHybrid is read straight from device memory.
    template <class PressureSolution, class SparseVec>
    void transportSolve(std::vector<double>& saturation, const double time,
                        const typename GridInterface::Vector& gravity, const PressureSolution& pressure_sol,
                        const SparseVec& injection_rates) const
    {
        const int nc = grid_.numCells(), nhf = grid_.numHalfFaces();
        std::vector<double> s = grid_.toPositions(saturation);
        std::vector<double> inj(nc, 0.0);
        for (int p = 0; p < nc; ++p) inj[p] = injection_rates.element(grid_.index_of_position[p]);
        std::vector<double> flux(nhf);
        fluxes(pressure_sol, flux);
        const double g[3] = {gravity[0], gravity[1], gravity[2]};
        porsol_transport_stats st{};
        check(porsol_transport_solve(t_, s.data(), time, g, flux.data(), inj.data(), &st));
        last_ = st;
        grid_.fromPositions(s, saturation);
    }

    // sub-steps, retries and CFL step of the last transportSolve (GPU extension)
    const porsol_transport_stats& lastStats() const { return last_; }

private:
    porsol_transport* t_ = nullptr;
    porsol_transport_opts o_{};
    bool ready_ = false;
    mutable porsol_transport_stats last_{};
    FlatGrid grid_;

    void create()
    {
        throwOnError(porsol_transport_create(&t_), "porsol_transport_create failed (no CUDA device?)");
        porsol_transport_opts_default(&o_);
    }
    void check(int rc) const
    {
        if (rc != PORSOL_OK) throw std::runtime_error(porsol_transport_last_error(t_));
    }
    template <class PressureSolution>
    void fluxes(const PressureSolution& ps, std::vector<double>& flux) const
    {
        for (int hf = 0; hf < grid_.numHalfFaces(); ++hf) flux[hf] = ps.outflux(hf);
    }
};

}  // namespace gpu
}  // namespace Opm

#endif
