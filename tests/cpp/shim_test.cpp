// shim_test.cpp -- compiles and drives the C++ drop-in (Opm::gpu::IncompFlowSolverHybrid,
// Opm::gpu::EulerUpstream) through minimal classes that model the reference's concepts:
// GridInterfaceEuler (cells/faces), a rock with permeability()/porosity() and fluid
// properties, BasicBoundaryConditions (flowCond/satCond/getPeriodicPartner), a fluid with
// phaseMobilities()/phaseDensities() and SparseVector::element().
//
// Checks: a linear pressure field is reproduced exactly (mimetic consistency), for both
// linsolver_type 0 (ILU0-CG) and 1 (AMG-CG); postProcessFluxes leaves antisymmetric twin
// fluxes; transportSolve conserves water volume; the ImplicitCapillarity step conserves the
// saturation volume.  Prints "OK" on success.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <vector>

#include "opm/porsol/gpu/EulerUpstream.hpp"
#include "opm/porsol/gpu/ImplicitCapillarity.hpp"
#include "opm/porsol/gpu/IncompFlowSolverHybrid.hpp"
#include "opm/porsol/gpu/PermeabilityAdjoint.hpp"

namespace mock {

struct Vec {
    double v[3] = {0, 0, 0};
    enum { dimension = 3 };
    double& operator[](int i) { return v[i]; }
    double operator[](int i) const { return v[i]; }
};

struct Cart {
    int nx, ny, nz;
    double h[3];
    int nc() const { return nx * ny * nz; }
};

struct Face {
    const Cart* g;
    int c, lf;
    typedef Vec Vector;
    int ijk(int d) const { return d == 0 ? c % g->nx : d == 1 ? (c / g->nx) % g->ny : c / (g->nx * g->ny); }
    int axis() const { return lf / 2; }
    int sign() const { return (lf % 2) ? 1 : -1; }
    bool boundary() const
    {
        const int n[3] = {g->nx, g->ny, g->nz};
        const int x = ijk(axis());
        return sign() < 0 ? x == 0 : x == n[axis()] - 1;
    }
    int boundaryId() const { return boundary() ? lf + 1 : 0; }
    int cellIndex() const { return c; }
    int localIndex() const { return lf; }
    int neighbourCellIndex() const
    {
        const int st[3] = {1, g->nx, g->nx * g->ny};
        return boundary() ? -999 : c + sign() * st[axis()];
    }
    double area() const
    {
        const int a = axis();
        return a == 0 ? g->h[1] * g->h[2] : a == 1 ? g->h[0] * g->h[2] : g->h[0] * g->h[1];
    }
    Vec centroid() const
    {
        Vec x;
        for (int d = 0; d < 3; ++d) x[d] = (ijk(d) + 0.5) * g->h[d];
        x[axis()] += sign() * 0.5 * g->h[axis()];
        return x;
    }
    Vec normal() const
    {
        Vec n;
        n[axis()] = sign();
        return n;
    }
};

struct FaceIterator : Face {
    typedef Vec Vector;
    const FaceIterator* operator->() const { return this; }
    const Face& operator*() const { return *this; }
    FaceIterator& operator++()
    {
        ++lf;
        return *this;
    }
    bool operator!=(const FaceIterator& o) const { return lf != o.lf || c != o.c; }
    bool operator==(const FaceIterator& o) const { return !(*this != o); }
};

struct CellIterator {
    const Cart* g;
    int c;
    typedef Vec Vector;
    typedef mock::FaceIterator FaceIterator;
    const CellIterator* operator->() const { return this; }
    CellIterator& operator++()
    {
        ++c;
        return *this;
    }
    bool operator!=(const CellIterator& o) const { return c != o.c; }
    int index() const { return c; }
    double volume() const { return g->h[0] * g->h[1] * g->h[2]; }
    Vec centroid() const
    {
        Vec x;
        const int ijk[3] = {c % g->nx, (c / g->nx) % g->ny, c / (g->nx * g->ny)};
        for (int d = 0; d < 3; ++d) x[d] = (ijk[d] + 0.5) * g->h[d];
        return x;
    }
    FaceIterator facebegin() const { return FaceIterator{{g, c, 0}}; }
    FaceIterator faceend() const { return FaceIterator{{g, c, 6}}; }
};

struct GridInterface {
    Cart g;
    typedef double Scalar;
    typedef mock::CellIterator CellIterator;
    typedef Vec Vector;
    enum { Dimension = 3 };
    int numberOfCells() const { return g.nc(); }
    CellIterator cellbegin() const { return CellIterator{&g, 0}; }
    CellIterator cellend() const { return CellIterator{&g, g.nc()}; }
};

struct Tensor {
    double k[9];
    double operator()(int i, int j) const { return k[3 * i + j]; }
};

struct Rock {
    std::vector<Tensor> K;
    std::vector<double> phi;
    Tensor permeability(int c) const { return K[c]; }
    double porosity(int c) const { return phi[c]; }
    double viscosityFirstPhase() const { return 1e-3; }
    double viscositySecondPhase() const { return 5e-3; }
    double densityFirstPhase() const { return 1000.0; }
    double densitySecondPhase() const { return 850.0; }
};

struct Fluid {
    enum { NumberOfPhases = 2 };
    template <class V>
    void phaseMobilities(int, double s, V& mob) const
    {
        mob[0] = s * s / 1e-3;
        mob[1] = (1 - s) * (1 - s) / 5e-3;
    }
    template <class V>
    void phaseDensities(int, V& rho) const
    {
        rho[0] = 1000.0;
        rho[1] = 850.0;
    }
};

// phase mobility tensors, diagonal (they commute with the diagonal K of the test)
struct TensorFluid {
    enum { NumberOfPhases = 2 };
    template <class M>
    void phaseMobility(int phase, int, double s, M& m) const
    {
        const double k = phase == 0 ? s * s / 1e-3 : (1 - s) * (1 - s) / 5e-3;
        m(0, 0) = k;
        m(1, 1) = 0.5 * k;
        m(2, 2) = 2.0 * k;
    }
    template <class V>
    void phaseDensities(int, V& rho) const
    {
        rho[0] = 1000.0;
        rho[1] = 850.0;
    }
};

struct FlowBC {
    int type = PORSOL_BC_NEUMANN;
    double value = 0.0;
    bool isDirichlet() const { return type == PORSOL_BC_DIRICHLET; }
    bool isNeumann() const { return type == PORSOL_BC_NEUMANN; }
    bool isPeriodic() const { return type == PORSOL_BC_PERIODIC; }
    double pressure() const { return value; }
    double outflux() const { return value; }
    double pressureDifference() const { return value; }
};
struct SatBC {
    bool isPeriodic() const { return false; }
    double saturation() const { return 1.0; }
};

// Dirichlet values of a linear field on every boundary face
struct LinearBC {
    double a[3];
    FlowBC flowCond(const Face& f) const
    {
        const Vec x = f.centroid();
        FlowBC b;
        b.type = PORSOL_BC_DIRICHLET;
        b.value = a[0] * x[0] + a[1] * x[1] + a[2] * x[2];
        return b;
    }
    SatBC satCond(const Face&) const { return SatBC(); }
    int getPeriodicPartner(int) const { return 0; }
};

struct Sparse {
    std::vector<double> v;
    double element(int i) const { return v[i]; }
};

template <class G, class R>
struct NoInnerProduct {};

}  // namespace mock

int main()
{
    using namespace mock;
    GridInterface g{{8, 6, 5, {0.125, 1.0 / 6, 0.2}}};
    const int nc = g.numberOfCells();
    Rock r;
    r.K.resize(nc);
    r.phi.assign(nc, 0.25);
    // A linear pressure field is the discrete solution only for a spatially constant K
    // (flux continuity); anisotropic but uniform here.
    for (int c = 0; c < nc; ++c) {
        const double k = 1e-13;
        r.K[c] = Tensor{{k, 0, 0, 0, 0.7 * k, 0, 0, 0, 0.3 * k}};
    }
    const LinearBC bc{{2.0, -1.0, 0.5}};
    Fluid fl;
    std::vector<double> sat(nc, 0.3), src(nc, 0.0);
    Vec grav;
    typedef Opm::gpu::IncompFlowSolverHybrid<GridInterface, Rock, LinearBC, NoInnerProduct> Solver;
    for (int type = 0; type < 2; ++type) {
        Solver s;
        s.init(g, r, grav, bc);
        s.solve(fl, sat, bc, src, 1e-13, 0, type);
        Solver::SolutionType sol = s.getSolution();
        double err = 0.0;
        for (CellIterator c = g.cellbegin(); c != g.cellend(); ++c) {
            const Vec x = c->centroid();
            const double u = 2.0 * x[0] - 1.0 * x[1] + 0.5 * x[2];
            err = std::fmax(err, std::fabs(sol.pressure(c) - u));
        }
        if (err > 1e-9) {
            std::printf("linear field error %g (type %d)\n", err, type);
            return 1;
        }
        const double mm = s.postProcessFluxes();
        if (!(mm >= 0.0)) return 1;
        // antisymmetric twin fluxes after post-processing
        for (CellIterator c = g.cellbegin(); c != g.cellend(); ++c)
            for (FaceIterator f = c->facebegin(); f != c->faceend(); ++f) {
                if (f->boundary()) continue;
                const FaceIterator tw{{&g.g, f->neighbourCellIndex(), f->localIndex() ^ 1}};
                if (std::fabs(s.getSolution().outflux(f) + s.getSolution().outflux(tw)) > 1e-25) {
                    std::printf("twin fluxes differ\n");
                    return 1;
                }
            }
        s.printStats(std::cout);
        // printSystem: one line per stored entry and one per unknown, the diagonal positive
        s.printSystem("/tmp/porsol_shim_system");
        std::ifstream mat("/tmp/porsol_shim_system-mat.dat"), rhs("/tmp/porsol_shim_system-rhs.dat");
        long long lines = 0, diag_ok = 0, rlines = 0;
        int i, j;
        double v;
        while (mat >> i >> j >> v) {
            ++lines;
            if (i == j && v > 0) ++diag_ok;
        }
        while (rhs >> v) ++rlines;
        int n = 0, nnz = 0, mx = 0, ni = 0;
        porsol_num_dofs(s.handle(), &n, &nnz, &mx, &ni);
        if (lines != nnz || diag_ok != n || rlines != n) {
            std::printf("printSystem: %lld entries (%d), %lld positive diagonals, %lld rhs lines (%d)\n", lines, nnz,
                        diag_ok, rlines, n);
            return 1;
        }
    }
    // tensor mobilities (the anisotropic-relperm inner product): still exact for a linear field
    {
        typedef Opm::gpu::IncompFlowSolverHybrid<GridInterface, Rock, LinearBC, Opm::gpu::MimeticIPAnisoRelpermEvaluator>
            TSolver;
        TSolver ts;
        ts.init(g, r, grav, bc);
        ts.solve(TensorFluid(), sat, bc, src, 1e-13, 0, 1);
        double err = 0.0;
        for (CellIterator c = g.cellbegin(); c != g.cellend(); ++c) {
            const Vec x = c->centroid();
            err = std::fmax(err, std::fabs(ts.getSolution().pressure(c) - (2.0 * x[0] - 1.0 * x[1] + 0.5 * x[2])));
        }
        if (err > 1e-9) {
            std::printf("tensor mobility: linear field error %g\n", err);
            return 1;
        }
    }
    // transport: p = -x drives water in through x- only (no normal flux elsewhere)
    const LinearBC bcx{{-1.0, 0.0, 0.0}};
    Solver s;
    s.init(g, r, grav, bcx);
    std::vector<double> s0(nc, 0.0);
    s.solve(fl, s0, bcx, src, 1e-12, 1, 1);   // verbosity 1: the CG summary line
    s.postProcessFluxes();
    Opm::gpu::Params prm;
    prm.o.method_capillary = 0;
    Opm::gpu::EulerUpstream<GridInterface, Rock, LinearBC> tr;
    tr.init(prm, g, r, bcx);
    Sparse inj{std::vector<double>(nc, 0.0)};
    std::vector<double> sw = s0;
    double qin = 0.0, pv = 0.0;
    for (CellIterator c = g.cellbegin(); c != g.cellend(); ++c) {
        pv += c->volume() * r.porosity(c->index());
        for (FaceIterator f = c->facebegin(); f != c->faceend(); ++f)
            if (f->boundary() && s.getSolution().outflux(f) < 0) qin -= s.getSolution().outflux(f);
    }
    const double T = 0.01 * pv / qin;
    // setCourantNumber after init applies to the next transportSolve: half the Courant number,
    // twice the sub-steps (up to the rounding of the step count)
    {
        std::vector<double> s1 = s0, s2 = s0;
        tr.transportSolve(s1, 4 * T, grav, s.getSolution(), inj);
        const int n1 = tr.lastStats().small_steps;
        tr.setCourantNumber(0.25);
        tr.transportSolve(s2, 4 * T, grav, s.getSolution(), inj);
        const int n2 = tr.lastStats().small_steps;
        tr.setCourantNumber(0.5);
        if (n2 < 2 * n1 - 1 || n2 > 2 * n1 + 1) {
            std::printf("setCourantNumber: %d sub-steps at 0.5, %d at 0.25\n", n1, n2);
            return 1;
        }
    }
    tr.transportSolve(sw, T, grav, s.getSolution(), inj);
    double water = 0.0, smin = 1, smax = 0;
    for (int c = 0; c < nc; ++c) {
        water += sw[c] * 0.25 * g.g.h[0] * g.g.h[1] * g.g.h[2];
        smin = std::fmin(smin, sw[c]);
        smax = std::fmax(smax, sw[c]);
    }
    // the x- faces inject water (SatBC s = 1); after 1% of a pore volume almost none has
    // left through x+ (upstream weighting smears the front over a few cells)
    if (water > qin * T * (1 + 1e-9) || water < qin * T * (1 - 1e-3) || smin < -1e-12 || smax > 1 + 1e-12) {
        std::printf("transport mass balance %g vs %g\n", water, qin * T);
        return 1;
    }
    // ImplicitCapillarity with one RockJfunc table: the step keeps the saturation volume and
    // stays inside the table's [s_min, s_max]
    {
        Opm::gpu::RockTables rt;
        Opm::gpu::RockTable tab;
        for (int i = 0; i <= 16; ++i) {
            const double s = 0.1 + 0.05 * i, se = (s - 0.1) / 0.8;
            tab.s.push_back(s);
            tab.krw.push_back(se * se);
            tab.kro.push_back((1 - se) * (1 - se));
            tab.J.push_back(2.0 * (1 - se) * (1 - se) + 0.05 * (1 - se));
        }
        rt.rocks.push_back(tab);
        rt.cell_rock.assign(nc, 0);
        rt.sigma_cos_theta = 1e-6;
        Opm::gpu::ImplicitCapillarity<GridInterface, Rock, LinearBC, NoInnerProduct> cap(g, r, bcx);
        cap.setRockTables(rt);
        std::vector<double> sc(nc);
        double v0 = 0.0;
        for (int c = 0; c < nc; ++c) {
            sc[c] = 0.3 + 0.4 * sw[c];
            v0 += sc[c];
        }
        cap.transportSolve(sc, T, grav, s.getSolution(), inj);
        double v1 = 0.0, lo = 1, hi = 0;
        for (int c = 0; c < nc; ++c) {
            v1 += sc[c];
            lo = std::fmin(lo, sc[c]);
            hi = std::fmax(hi, sc[c]);
        }
        if (std::fabs(v1 - v0) > 1e-10 * v0 || lo < 0.1 || hi > 0.9 || cap.lastStats().root_iterations <= 0) {
            std::printf("capillary step: volume %g vs %g, range [%g, %g]\n", v1, v0, lo, hi);
            return 1;
        }
    }
    // forward/backward pair: J = sum of squared mismatches at three cells + scaled outflux at x+
    {
        Rock r2 = r;
        for (int c = 0; c < nc; ++c) {
            const double k = 1e-13 * std::exp(0.7 * std::sin(1.3 * c));
            r2.K[c] = Tensor{{k, 0, 0, 0, 0.5 * k, 0, 0, 0, 0.2 * k}};
        }
        Solver sa;
        sa.init(g, r2, grav, bcx);
        Opm::gpu::PermeabilityAdjoint<Solver> adj(sa);
        std::vector<double> w(nc, 0.0), tgt(nc, -0.4), u(sa.flatGrid().numHalfFaces(), 0.0);
        w[5] = w[77] = w[150] = 1.0;
        for (CellIterator c = g.cellbegin(); c != g.cellend(); ++c)
            for (FaceIterator f = c->facebegin(); f != c->faceend(); ++f)
                if (f->boundary() && f->centroid()[0] > 1.0 - 1e-12) u[sa.flatGrid().halfFace(c->index(), f->localIndex())] = 1e12;
        adj.setObjective(w, tgt, u);
        const double J = adj.forward(fl, s0, bcx, src, 1e-14, 0, 1);
        double Jh = 0.0;
        for (CellIterator c = g.cellbegin(); c != g.cellend(); ++c) {
            const double d = sa.getSolution().pressure(c) - tgt[c->index()];
            Jh += w[c->index()] * d * d;
            for (FaceIterator f = c->facebegin(); f != c->faceend(); ++f)
                Jh += u[sa.flatGrid().halfFace(c->index(), f->localIndex())] * sa.getSolution().outflux(f);
        }
        if (std::fabs(J - Jh) > 1e-12 * std::fabs(J)) {
            std::printf("objective %.17g vs %.17g\n", J, Jh);
            return 1;
        }
        const std::vector<double> grad = adj.backward();
        const std::vector<double> g3 = adj.backward(true);
        for (int c = 0; c < nc; ++c)
            if (std::fabs(g3[3 * c] + g3[3 * c + 1] + g3[3 * c + 2] - grad[c]) > 1e-10 * std::fabs(grad[77]) + 1e-300) {
                std::printf("axis gradients do not sum to the scale gradient at %d\n", c);
                return 1;
            }
        const double h = 1e-4;
        double Jpm[2];
        for (int k = 0; k < 2; ++k) {
            Rock rp = r2;
            for (int q = 0; q < 9; ++q) rp.K[77].k[q] *= std::exp(k == 0 ? h : -h);
            sa.computeInnerProducts(rp, grav);
            Jpm[k] = adj.forward(fl, s0, bcx, src, 1e-14, 0, 1);
        }
        const double fd = (Jpm[0] - Jpm[1]) / (2 * h);
        if (std::fabs(fd - grad[77]) > 1e-6 * std::fabs(fd)) {
            std::printf("adjoint %.12g vs finite difference %.12g\n", grad[77], fd);
            return 1;
        }
    }
    std::printf("OK\n");
    return 0;
}
