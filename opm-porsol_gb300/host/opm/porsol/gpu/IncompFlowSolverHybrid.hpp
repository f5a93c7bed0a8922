// IncompFlowSolverHybrid.hpp -- GB300 drop-in for Opm::IncompFlowSolverHybrid.
//
// Same template parameters, method names, argument order and defaults as the reference
// (opm/porsol/mimetic/IncompFlowSolverHybrid.hpp:362-366, 477-831), so code written
// against the reference (SimulatorBase, SimulatorTester, ImplicitCapillarity, the
// examples) compiles unchanged when it names Opm::gpu::IncompFlowSolverHybrid instead.
// The work is done on the GPU through the C ABI of include/porsol_gpu.h:
//   init / initSystemStructure  -> porsol_init_system_structure (face DOFs, sparsity)
//   computeInnerProducts        -> porsol_compute_inner_products (MimeticIPEvaluator)
//   solve                       -> porsol_solve (assembly, ILU0-CG or AMG-CG, recovery)
//   postProcessFluxes           -> porsol_post_process_fluxes
//   getSolution                 -> porsol_get_solution (FlowSolution mirror on the host)
// The InnerProduct template argument is accepted for source compatibility; the GPU
// evaluates the MimeticIPEvaluator inner product (the only one on this path).
// Errors come back as std::runtime_error with the reference's message text.
#ifndef OPM_PORSOL_GPU_INCOMPFLOWSOLVERHYBRID_HPP
#define OPM_PORSOL_GPU_INCOMPFLOWSOLVERHYBRID_HPP

#include <array>
#include <iostream>
#include <cmath>
#include <fstream>
#include <iterator>
#include <ostream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "GridFlattener.hpp"
#include "porsol_gpu.h"

namespace Opm {
namespace gpu {

// InnerProduct tag for the tensor-mobility evaluator (MimeticIPAnisoRelpermEvaluator,
// mimetic/MimeticIPAnisoRelpermEvaluator.hpp): with it, solve() asks the fluid for phase
// mobility tensors, fl.phaseMobility(phase, cell, s, m) with m a Mat3, and the GPU rebuilds the
// inner products from lambda_t K on every solve (PORSOL_FLUID_TENSOR).
template <class GridIF, class RockIF>
class MimeticIPAnisoRelpermEvaluator {};

// 3x3 matrix handed to FluidInterface::phaseMobility: m(i, j), column-major storage like the
// reference's SharedFortranMatrix.
struct Mat3 {
    double a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double& operator()(int i, int j) { return a[i + 3 * j]; }
    double operator()(int i, int j) const { return a[i + 3 * j]; }
    int numRows() const { return 3; }
    int numCols() const { return 3; }
    double* data() { return a; }
};

template <class GridInterface, class RockInterface, class BCInterface,
          template <class GridIF, class RockIF> class InnerProduct>
class IncompFlowSolverHybrid {
    typedef typename GridInterface::Scalar Scalar;

public:
    // FlowSolution (IncompFlowSolverHybrid.hpp:382-447): cell pressure and outward
    // half-face fluxes, mirrored on the host after every solve / postProcessFluxes.
    class FlowSolution {
    public:
        typedef typename GridInterface::CellIterator CI;
        typedef typename CI::FaceIterator FI;
        friend class IncompFlowSolverHybrid;

        Scalar pressure(const CI& c) const { return pressure_[grid_->position[c->index()]]; }
        Scalar outflux(const FI& f) const { return outflux_[grid_->halfFace(f->cellIndex(), f->localIndex())]; }
        Scalar outflux(int hf) const { return outflux_[hf]; }
        // GPU extension: device pointer of the half-face fluxes (valid until the next solve)
        const double* deviceOutflux() const { return d_outflux_; }

    private:
        const FlatGrid* grid_ = nullptr;
        std::vector<Scalar> pressure_;
        std::vector<Scalar> outflux_;
        const double* d_outflux_ = nullptr;
        void clear()
        {
            pressure_.clear();
            outflux_.clear();
            d_outflux_ = nullptr;
        }
    };
    typedef const FlowSolution& SolutionType;

    IncompFlowSolverHybrid()
    {
        porsol_solver* h = nullptr;
        throwOnError(porsol_create(&h), "porsol_create failed (no CUDA device?)");
        h_ = h;
        porsol_solve_opts_default(&extra_);
    }
    ~IncompFlowSolverHybrid() { porsol_destroy(h_); }
    IncompFlowSolverHybrid(const IncompFlowSolverHybrid&) = delete;
    IncompFlowSolverHybrid& operator=(const IncompFlowSolverHybrid&) = delete;

    // IncompFlowSolverHybrid.hpp:477-488
    template <class Point>
    void init(const GridInterface& g, const RockInterface& r, const Point& grav, const BCInterface& bc)
    {
        clear();
        if (g.numberOfCells() > 0) {
            initSystemStructure(g, bc);
            computeInnerProducts(r, grav);
        }
    }

    // IncompFlowSolverHybrid.hpp:498-516
    void clear()
    {
        check(porsol_clear(h_));
        pgrid_ = nullptr;
        flowSolution_.clear();
    }

    // IncompFlowSolverHybrid.hpp:534-545
    void initSystemStructure(const GridInterface& g, const BCInterface& bc)
    {
        pgrid_ = &g;
        grid_ = flattenGrid(g);
        flattenFlowBC(g, grid_, bc, bct_, bcv_, partner_);
        const porsol_grid v = grid_.view();
        check(porsol_init_system_structure(h_, &v, bct_.data(), partner_.data()));
        flowSolution_.grid_ = &grid_;
    }

    // IncompFlowSolverHybrid.hpp:565-578 (MimeticIPEvaluator::buildStaticContrib)
    template <class Point>
    void computeInnerProducts(const RockInterface& r, const Point& grav)
    {
        const int nc = grid_.numCells();
        std::vector<double> K(9 * size_t(nc));
        for (int p = 0; p < nc; ++p) {
            const auto k = r.permeability(grid_.index_of_position[p]);
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) K[9 * size_t(p) + 3 * i + j] = k(i, j);
        }
        const double g[3] = {grav[0], grav[1], grav[2]};
        check(porsol_compute_inner_products(h_, K.data(), g));
    }
    // The name used by the reference's commented callers (common/SimulatorBase.hpp:211).
    template <class Point>
    void assembleStatic(const RockInterface& r, const Point& grav) { computeInnerProducts(r, grav); }

    // IncompFlowSolverHybrid.hpp:658-703
    template <class FluidInterface>
    void solve(const FluidInterface& fl, const std::vector<double>& sat, const BCInterface& bc,
               const std::vector<double>& src, double residual_tolerance = 1e-8, int linsolver_verbosity = 1,
               int linsolver_type = 1, bool same_matrix = false, int linsolver_maxit = 0,
               double prolongate_factor = 1.6, int smooth_steps = 1)
    {
        if constexpr (std::is_same<InnerProduct<GridInterface, RockInterface>,
                                   MimeticIPAnisoRelpermEvaluator<GridInterface, RockInterface>>::value) {
            solveTensor(fl, sat, bc, src, residual_tolerance, linsolver_verbosity, linsolver_type, same_matrix,
                        linsolver_maxit, prolongate_factor, smooth_steps);
        } else {
            solveScalar(fl, sat, bc, src, residual_tolerance, linsolver_verbosity, linsolver_type, same_matrix,
                        linsolver_maxit, prolongate_factor, smooth_steps);
        }
    }

private:
    template <class FluidInterface>
    void solveScalar(const FluidInterface& fl, const std::vector<double>& sat, const BCInterface& bc,
                     const std::vector<double>& src, double residual_tolerance, int linsolver_verbosity,
                     int linsolver_type, bool same_matrix, int linsolver_maxit, double prolongate_factor,
                     int smooth_steps)
    {
        const int nc = grid_.numCells();
        // FluidInterface::phaseMobilities / phaseDensities per cell
        // (MimeticIPEvaluator::computeDynamicParams, MimeticIPEvaluator.hpp:297-311)
        std::vector<double> totmob(nc), mobdens(nc), srcp(nc);
        for (int p = 0; p < nc; ++p) {
            const int ci = grid_.index_of_position[p];
            std::array<double, FluidInterface::NumberOfPhases> mob, rho;
            fl.phaseMobilities(ci, sat[ci], mob);
            fl.phaseDensities(ci, rho);
            double tm = 0.0, md = 0.0;
            for (int k = 0; k < FluidInterface::NumberOfPhases; ++k) {
                tm += mob[k];
                md += rho[k] * mob[k];
            }
            totmob[p] = tm;
            mobdens[p] = md;
            srcp[p] = src[ci];
        }
        flattenFlowBC(*pgrid_, grid_, bc, bct_, bcv_, partner_);
        porsol_fluid f{PORSOL_FLUID_CELLWISE, 1.0, 1.0, 0.0, 0.0};
        porsol_solve_opts o = extra_;
        o.residual_tolerance = residual_tolerance;
        o.linsolver_verbosity = linsolver_verbosity;
        o.linsolver_type = linsolver_type;
        o.same_matrix = same_matrix ? 1 : 0;
        o.linsolver_maxit = linsolver_maxit;
        o.prolongate_factor = prolongate_factor;
        o.smooth_steps = smooth_steps;
        check(porsol_solve(h_, &f, totmob.data(), mobdens.data(), bct_.data(), bcv_.data(), srcp.data(), &o,
                           &stats_));
        report(linsolver_verbosity);
        fetchSolution();
    }

public:
    // IncompFlowSolverHybrid.hpp:754-807
    double postProcessFluxes()
    {
        double m = 0.0;
        check(porsol_post_process_fluxes(h_, &m));
        fetchSolution();
        return m;
    }

    // IncompFlowSolverHybrid.hpp:818-831
    SolutionType getSolution() { return flowSolution_; }

    // IncompFlowSolverHybrid.hpp:849-871
    template <typename charT, class traits>
    void printStats(std::basic_ostream<charT, traits>& os)
    {
        int n = 0, nnz = 0, mx = 0, ni = 0;
        check(porsol_num_dofs(h_, &n, &nnz, &mx, &ni));
        os << "IncompFlowSolverHybrid<> (GB300):\n"
           << "\tMaximum number of cell faces = " << mx << '\n'
           << "\tNumber of internal faces     = " << ni << '\n'
           << "\tTotal number of faces        = " << n << '\n'
           << "\tNon-zeros of S               = " << nnz << '\n';
    }

    // IncompFlowSolverHybrid.hpp:895-905: the assembled system of the last solve (before the
    // pure-Neumann regularisation) as prefix + "-mat.dat" (one "row col value" line per stored
    // entry, 1-based, the coordinate format of dune-istl's writeMatrixToMatlab) and
    // prefix + "-rhs.dat" (one value per line, 15 digits, scientific with sign, as the reference).
    void printSystem(const std::string& prefix)
    {
        int n = 0, nnz = 0, mx = 0, ni = 0;
        check(porsol_num_dofs(h_, &n, &nnz, &mx, &ni));
        std::vector<int> cf(grid_.numHalfFaces()), rp(n + 1), ci(nnz), pp(n);
        std::vector<double> val(nnz), rhs(n);
        check(porsol_get_structure(h_, cf.data(), rp.data(), ci.data(), pp.data()));
        check(porsol_get_system(h_, val.data(), rhs.data()));
        std::ofstream mat((prefix + "-mat.dat").c_str());
        mat.precision(15);
        mat.setf(std::ios::scientific);
        for (int i = 0; i < n; ++i)
            for (int k = rp[i]; k < rp[i + 1]; ++k) mat << i + 1 << ' ' << ci[k] + 1 << ' ' << val[k] << '\n';
        std::ofstream r((prefix + "-rhs.dat").c_str());
        r.precision(15);
        r.setf(std::ios::scientific | std::ios::showpos);
        std::copy(rhs.begin(), rhs.end(), std::ostream_iterator<double>(r, "\n"));
        if (!mat || !r) throw std::runtime_error("printSystem: could not write " + prefix + "-mat.dat / -rhs.dat");
    }

    // ---- GPU extensions (no counterpart in the reference) ----
    // PORSOL_FP64 (default, the plain drop-in) or PORSOL_MIXED (FP32 AMG hierarchy under FP32 CG
    // recurrences with an FP64 solution and FP64 residual replacements).
    void setPrecision(int mode) { extra_.precision = mode; }
    const porsol_solve_stats& lastStats() const { return stats_; }
    porsol_solver* handle() const { return h_; }
    const FlatGrid& flatGrid() const { return grid_; }

private:
    // linsolver_verbosity > 0: the summary line the reference's CG solver prints
    // (dune-istl CGSolver with verbose >= 1: convergence rate, time, time per iteration, iterations)
    void report(int verbosity) const
    {
        if (verbosity <= 0) return;
        const int it = stats_.iterations;
        const double T = 1e-3 * stats_.ms_krylov;
        const double rate = it > 0 && stats_.reduction > 0 ? std::pow(stats_.reduction, 1.0 / it) : 0.0;
        std::cout << "=== rate=" << rate << ", T=" << T << ", TIT=" << (it > 0 ? T / it : 0.0) << ", IT=" << it
                  << std::endl;
    }

    porsol_solver* h_ = nullptr;
    const GridInterface* pgrid_ = nullptr;
    FlatGrid grid_;
    std::vector<int> bct_, partner_;
    std::vector<double> bcv_;
    porsol_solve_opts extra_;
    porsol_solve_stats stats_{};
    FlowSolution flowSolution_;

    void check(int rc) const
    {
        if (rc != PORSOL_OK) throw std::runtime_error(porsol_last_error(h_));
    }
    // MimeticIPAnisoRelpermEvaluator::computeDynamicParams (MimeticIPAnisoRelpermEvaluator.hpp:
    // 297-330): lambda_t = sum_i lambda_i and sum_i rho_i lambda_i per cell, row-major.
    template <class FluidInterface>
    void solveTensor(const FluidInterface& fl, const std::vector<double>& sat, const BCInterface& bc,
                     const std::vector<double>& src, double residual_tolerance, int linsolver_verbosity,
                     int linsolver_type, bool same_matrix, int linsolver_maxit, double prolongate_factor,
                     int smooth_steps)
    {
        const int nc = grid_.numCells();
        std::vector<double> lam(9 * size_t(nc), 0.0), rlam(9 * size_t(nc), 0.0), srcp(nc);
        for (int p = 0; p < nc; ++p) {
            const int ci = grid_.index_of_position[p];
            std::array<double, FluidInterface::NumberOfPhases> rho;
            fl.phaseDensities(ci, rho);
            for (int ph = 0; ph < FluidInterface::NumberOfPhases; ++ph) {
                Mat3 m;
                fl.phaseMobility(ph, ci, sat[ci], m);
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) {
                        lam[9 * size_t(p) + 3 * i + j] += m(i, j);
                        rlam[9 * size_t(p) + 3 * i + j] += rho[ph] * m(i, j);
                    }
            }
            srcp[p] = src[ci];
        }
        flattenFlowBC(*pgrid_, grid_, bc, bct_, bcv_, partner_);
        porsol_fluid f{PORSOL_FLUID_TENSOR, 1.0, 1.0, 0.0, 0.0};
        porsol_solve_opts o = extra_;
        o.residual_tolerance = residual_tolerance;
        o.linsolver_verbosity = linsolver_verbosity;
        o.linsolver_type = linsolver_type;
        o.same_matrix = same_matrix ? 1 : 0;
        o.linsolver_maxit = linsolver_maxit;
        o.prolongate_factor = prolongate_factor;
        o.smooth_steps = smooth_steps;
        check(porsol_solve(h_, &f, lam.data(), rlam.data(), bct_.data(), bcv_.data(), srcp.data(), &o, &stats_));
        report(linsolver_verbosity);
        fetchSolution();
    }
    void fetchSolution()
    {
        const int nc = grid_.numCells(), nhf = grid_.numHalfFaces();
        flowSolution_.pressure_.resize(nc);
        flowSolution_.outflux_.resize(nhf);
        check(porsol_get_solution(h_, flowSolution_.pressure_.data(), flowSolution_.outflux_.data(), nullptr));
        const double* dv = nullptr;
        check(porsol_get_solution_device(h_, nullptr, &dv, nullptr));
        flowSolution_.d_outflux_ = dv;
        flowSolution_.grid_ = &grid_;
    }
};

}  // namespace gpu
}  // namespace Opm

#endif
