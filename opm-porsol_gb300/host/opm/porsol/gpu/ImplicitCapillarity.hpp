// ImplicitCapillarity.hpp -- GB300 drop-in for Opm::ImplicitCapillarity (steady capillary
// redistribution of the saturation, the "ImplicitCap" transport of SimulatorTraits).
//
// Same class template, constructors and methods as the reference
// (opm/porsol/euler/ImplicitCapillarity.hpp:52-129, ImplicitCapillarity_impl.hpp:57-247).  The
// residual, rock tables and boundary data live in an Opm::gpu::EulerUpstream (the reference's
// EulerUpstreamResidual member), the capillary pressure is solved by an
// Opm::gpu::IncompFlowSolverHybrid initialised with zero gravity (its psolver_), and one call of
// porsol_capillary_solve (include/porsol_gpu.h) runs the whole step on the GPU.  The RockJfunc
// tables are handed over with setRockTables() (RockTables.hpp): without them the inverse
// capillary-pressure curve is 0, as in the reference, and no shift can be found.
#ifndef OPM_PORSOL_GPU_IMPLICITCAPILLARITY_HPP
#define OPM_PORSOL_GPU_IMPLICITCAPILLARITY_HPP

#include <stdexcept>
#include <string>
#include <vector>

#include "EulerUpstream.hpp"
#include "GridFlattener.hpp"
#include "IncompFlowSolverHybrid.hpp"
#include "RockTables.hpp"
#include "porsol_gpu.h"

namespace Opm {
namespace gpu {

template <class GridInterface, class ReservoirProperties, class BoundaryConditions,
          template <class, class> class InnerProd>
class ImplicitCapillarity {
public:
    typedef IncompFlowSolverHybrid<GridInterface, ReservoirProperties, BoundaryConditions, InnerProd> PressureSolver;

    ImplicitCapillarity() { porsol_capillary_opts_default(&o_); }
    ImplicitCapillarity(const GridInterface& g, const ReservoirProperties& r, const BoundaryConditions& b)
    {
        porsol_capillary_opts_default(&o_);
        initObj(g, r, b);
    }

    // ImplicitCapillarity_impl.hpp:91-101 -- same keys and defaults
    template <class ParamGroup>
    void init(const ParamGroup& param)
    {
        o_.method_viscous = param.getDefault("method_viscous", bool(o_.method_viscous));
        o_.method_gravity = param.getDefault("method_gravity", bool(o_.method_gravity));
        o_.check_sat = param.getDefault("check_sat", bool(o_.check_sat));
        o_.clamp_sat = param.getDefault("clamp_sat", bool(o_.clamp_sat));
        o_.residual_tolerance = param.getDefault("residual_tolerance", o_.residual_tolerance);
        o_.linsolver_verbosity = param.getDefault("linsolver_verbosity", o_.linsolver_verbosity);
        o_.linsolver_type = param.getDefault("linsolver_type", o_.linsolver_type);
        o_.update_relaxation = param.getDefault("update_relaxation", o_.update_relaxation);
    }
    template <class ParamGroup>
    void init(const ParamGroup& param, const GridInterface& g, const ReservoirProperties& r,
              const BoundaryConditions& b)
    {
        init(param);
        initObj(g, r, b);
    }

    // ImplicitCapillarity_impl.hpp:109-117: the residual object and psolver_.init(g, r, 0, b)
    void initObj(const GridInterface& g, const ReservoirProperties& r, const BoundaryConditions& b)
    {
        residual_.initObj(g, r, b);
        typename GridInterface::Vector grav;
        for (int d = 0; d < 3; ++d) grav[d] = 0.0;
        psolver_.init(g, r, grav, b);
        pgrid_ = &g;
        pbc_ = &b;
    }

    void setRockTables(const RockTables& rt) { residual_.setRockTables(rt); }
    // precision of the capillary pressure solve (PORSOL_FP64 or PORSOL_MIXED)
    void setPrecision(int precision) { o_.precision = precision; }

    // ImplicitCapillarity_impl.hpp:138-226 (time is unused, as in the reference)
    template <class PressureSolution, class SparseVec>
    void transportSolve(std::vector<double>& saturation, const double /*time*/,
                        const typename GridInterface::Vector& gravity, const PressureSolution& pressure_sol,
                        const SparseVec& injection_rates) const
    {
        if (!pgrid_) throw std::runtime_error("ImplicitCapillarity: initObj was not called");
        const FlatGrid& fg = residual_.flatGrid();
        const int nc = fg.numCells(), nhf = fg.numHalfFaces();
        std::vector<double> s = fg.toPositions(saturation);
        std::vector<double> inj(nc, 0.0);
        for (int p = 0; p < nc; ++p) inj[p] = injection_rates.element(fg.index_of_position[p]);
        std::vector<double> flux(nhf);
        for (int hf = 0; hf < nhf; ++hf) flux[hf] = pressure_sol.outflux(hf);
        std::vector<int> bct, partner;
        std::vector<double> bcv;
        flattenFlowBC(*pgrid_, fg, *pbc_, bct, bcv, partner);
        const double g[3] = {gravity[0], gravity[1], gravity[2]};
        porsol_capillary_stats st{};
        const int rc = porsol_capillary_solve(residual_.handle(), psolver_.handle(), s.data(), g, flux.data(),
                                              inj.data(), bct.data(), bcv.data(), &o_, &st);
        if (rc != PORSOL_OK) throw std::runtime_error(porsol_transport_last_error(residual_.handle()));
        last_ = st;
        fg.fromPositions(s, saturation);
    }

    // shift of the capillary pressure and iteration counts of the last transportSolve
    const porsol_capillary_stats& lastStats() const { return last_; }

private:
    EulerUpstream<GridInterface, ReservoirProperties, BoundaryConditions> residual_;
    mutable PressureSolver psolver_;
    const GridInterface* pgrid_ = nullptr;
    const BoundaryConditions* pbc_ = nullptr;
    porsol_capillary_opts o_{};
    mutable porsol_capillary_stats last_{};
};

}  // namespace gpu
}  // namespace Opm

#endif
