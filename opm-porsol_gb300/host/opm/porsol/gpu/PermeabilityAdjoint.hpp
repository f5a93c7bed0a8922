// PermeabilityAdjoint.hpp -- forward/backward pair for the permeability gradient of the
// mimetic pressure solve (a GPU extension: the reference has no adjoint).
//
//   J = sum_c w_c (p_c - p*_c)^2 + sum_hf u_hf v_hf
//
// forward() runs IncompFlowSolverHybrid::solve with the reference's arguments and returns J
// (porsol_objective_value); backward() returns dJ/d ln k per cell (porsol_adjoint_gradient:
// one adjoint solve with the forward's matrix and preconditioner, then the per-cell gradient).
// Cell data are keyed by Cell::index(), half-face weights by the FlowSolution half-face index
// (FlowSolution::outflux(int hf)); empty vectors mean zero.  Zero gravity, no periodic faces
// and at least one Dirichlet face are required (std::runtime_error otherwise).
#ifndef OPM_PORSOL_GPU_PERMEABILITYADJOINT_HPP
#define OPM_PORSOL_GPU_PERMEABILITYADJOINT_HPP

#include <stdexcept>
#include <vector>

#include "porsol_gpu.h"

namespace Opm {
namespace gpu {

template <class FlowSolver>
class PermeabilityAdjoint {
public:
    explicit PermeabilityAdjoint(FlowSolver& solver) : s_(solver) {}

    void setObjective(const std::vector<double>& cell_weight, const std::vector<double>& cell_target,
                      const std::vector<double>& hf_weight)
    {
        w_ = cell_weight;
        t_ = cell_target;
        u_ = hf_weight;
    }

    template <class FluidInterface, class BCInterface>
    double forward(const FluidInterface& fl, const std::vector<double>& sat, const BCInterface& bc,
                   const std::vector<double>& src, double residual_tolerance = 1e-8, int linsolver_verbosity = 1,
                   int linsolver_type = 1, bool same_matrix = false, int linsolver_maxit = 0,
                   double prolongate_factor = 1.6, int smooth_steps = 1)
    {
        s_.solve(fl, sat, bc, src, residual_tolerance, linsolver_verbosity, linsolver_type, same_matrix,
                 linsolver_maxit, prolongate_factor, smooth_steps);
        return objective();
    }

    // J of the solver's current solution
    double objective()
    {
        porsol_objective o = view();
        double J = 0.0;
        check(porsol_objective_value(s_.handle(), &o, &J));
        return J;
    }

    // dJ/d ln k_c (K_c -> s K_c), keyed by Cell::index(); with axes = true, 3 values per cell
    // (d/d ln k_x, k_y, k_z of diagonal tensors) at [3 c + a].
    std::vector<double> backward(bool axes = false)
    {
        porsol_objective o = view();
        const FlatGrid& g = s_.flatGrid();
        const int nc = g.numCells(), na = axes ? 3 : 1;
        std::vector<double> byPos(size_t(na) * nc), out(size_t(na) * nc);
        check(porsol_adjoint_gradient(s_.handle(), &o, axes ? PORSOL_GRAD_LOGK_AXES : PORSOL_GRAD_LOGK, nullptr,
                                      &J_, byPos.data(), &stats_));
        for (int p = 0; p < nc; ++p)
            for (int a = 0; a < na; ++a) out[size_t(na) * g.index_of_position[p] + a] = byPos[size_t(na) * p + a];
        return out;
    }

    double lastObjective() const { return J_; }
    const porsol_solve_stats& lastStats() const { return stats_; }

private:
    FlowSolver& s_;
    std::vector<double> w_, t_, u_, wp_, tp_;
    double J_ = 0.0;
    porsol_solve_stats stats_{};

    porsol_objective view()
    {
        const FlatGrid& g = s_.flatGrid();
        wp_ = w_.empty() ? std::vector<double>() : g.toPositions(w_);
        tp_ = t_.empty() ? std::vector<double>() : g.toPositions(t_);
        if (!u_.empty() && int(u_.size()) != g.numHalfFaces())
            throw std::runtime_error("PermeabilityAdjoint: one half-face weight per half-face expected");
        porsol_objective o;
        o.cell_weight = wp_.empty() ? nullptr : wp_.data();
        o.cell_target = tp_.empty() ? nullptr : tp_.data();
        o.hf_weight = u_.empty() ? nullptr : u_.data();
        return o;
    }
    void check(int rc) const
    {
        if (rc != PORSOL_OK) throw std::runtime_error(porsol_last_error(s_.handle()));
    }
};

}  // namespace gpu
}  // namespace Opm

#endif
