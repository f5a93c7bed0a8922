// GridFlattener.hpp -- walks a GridInterface once and produces the flat arrays of
// porsol_grid (include/porsol_gpu.h).
//
// The concept consumed is the reference's GridInterfaceEuler (GridInterfaceEuler.hpp):
// cellbegin()/cellend(), Cell::index()/volume()/centroid()/facebegin()/faceend(),
// Face::area()/centroid()/normal()/boundary()/boundaryId()/neighbourCellIndex()/
// cellIndex()/localIndex().  Cells are stored in iteration order (the reference's
// cellno_ numbering, IncompFlowSolverHybrid.hpp:968-979); cell data keyed by
// Cell::index() is permuted through `position`.
#ifndef OPM_PORSOL_GPU_GRIDFLATTENER_HPP
#define OPM_PORSOL_GPU_GRIDFLATTENER_HPP

#include <stdexcept>
#include <string>
#include <vector>

#include "porsol_gpu.h"

namespace Opm {
namespace gpu {

struct FlatGrid {
    std::vector<int> facepos, neighbour, bid, index_of_position, position;
    std::vector<double> area, centroid, normal, volume, ccentroid;
    bool identity = true;   // iteration order == index order

    int numCells() const { return int(volume.size()); }
    int numHalfFaces() const { return facepos.empty() ? 0 : facepos.back(); }

    porsol_grid view() const
    {
        porsol_grid g;
        g.num_cells = numCells();
        g.cell_facepos = facepos.data();
        g.hf_neighbour = neighbour.data();
        g.hf_bid = bid.data();
        g.hf_area = area.data();
        g.hf_centroid = centroid.data();
        g.hf_normal = normal.data();
        g.cell_volume = volume.data();
        g.cell_centroid = ccentroid.data();
        return g;
    }

    // half-face index of (cell position, local face index)
    int halfFace(int cell_index, int local) const { return facepos[position[cell_index]] + local; }

    template <class V>
    std::vector<double> toPositions(const V& by_index) const
    {
        std::vector<double> out(numCells());
        for (int p = 0; p < numCells(); ++p) out[p] = by_index[index_of_position[p]];
        return out;
    }
    template <class V>
    void fromPositions(const std::vector<double>& by_pos, V& by_index) const
    {
        for (int p = 0; p < numCells(); ++p) by_index[index_of_position[p]] = by_pos[p];
    }
};

template <class GridInterface>
FlatGrid flattenGrid(const GridInterface& g)
{
    typedef typename GridInterface::CellIterator CI;
    typedef typename CI::FaceIterator FI;
    FlatGrid fg;
    const int nc = g.numberOfCells();
    fg.position.assign(nc, -1);
    fg.index_of_position.reserve(nc);
    int p = 0;
    for (CI c = g.cellbegin(); c != g.cellend(); ++c, ++p) {
        const int ci = c->index();
        if (ci < 0 || ci >= nc || fg.position[ci] != -1)
            throw std::runtime_error("grid: cell indices are not a permutation of 0..numberOfCells()-1");
        fg.position[ci] = p;
        fg.index_of_position.push_back(ci);
        if (ci != p) fg.identity = false;
    }
    fg.facepos.push_back(0);
    for (CI c = g.cellbegin(); c != g.cellend(); ++c) {
        fg.volume.push_back(c->volume());
        const typename CI::Vector cc = c->centroid();
        for (int d = 0; d < 3; ++d) fg.ccentroid.push_back(cc[d]);
        int nf = 0;
        for (FI f = c->facebegin(); f != c->faceend(); ++f, ++nf) {
            if (f->localIndex() != nf) throw std::runtime_error("grid: faces not visited in local order");
            fg.neighbour.push_back(f->boundary() ? -1 : fg.position[f->neighbourCellIndex()]);
            fg.bid.push_back(f->boundary() ? f->boundaryId() : 0);
            fg.area.push_back(f->area());
            const typename FI::Vector fc = f->centroid();
            const typename FI::Vector fn = f->normal();
            for (int d = 0; d < 3; ++d) {
                fg.centroid.push_back(fc[d]);
                fg.normal.push_back(fn[d]);
            }
        }
        fg.facepos.push_back(fg.facepos.back() + nf);
    }
    return fg;
}

// FlowBC of every boundary half-face (BCInterface::flowCond(face), BoundaryConditions.hpp:121-171):
// type, value and, for periodic faces, getPeriodicPartner(boundaryId()).
template <class GridInterface, class BCInterface>
void flattenFlowBC(const GridInterface& g, const FlatGrid& fg, const BCInterface& bc, std::vector<int>& type,
                   std::vector<double>& value, std::vector<int>& partner)
{
    typedef typename GridInterface::CellIterator CI;
    typedef typename CI::FaceIterator FI;
    const int nhf = fg.numHalfFaces();
    type.assign(nhf, PORSOL_BC_NEUMANN);
    value.assign(nhf, 0.0);
    partner.assign(nhf, 0);
    int hf = 0;
    for (CI c = g.cellbegin(); c != g.cellend(); ++c)
        for (FI f = c->facebegin(); f != c->faceend(); ++f, ++hf) {
            if (!f->boundary()) continue;
            const auto& fc = bc.flowCond(*f);
            if (fc.isDirichlet()) {
                type[hf] = PORSOL_BC_DIRICHLET;
                value[hf] = fc.pressure();
            } else if (fc.isPeriodic()) {
                type[hf] = PORSOL_BC_PERIODIC;
                value[hf] = fc.pressureDifference();
                partner[hf] = bc.getPeriodicPartner(f->boundaryId());
            } else {
                type[hf] = PORSOL_BC_NEUMANN;
                value[hf] = fc.outflux();
            }
        }
}

inline void throwOnError(int rc, const char* what)
{
    if (rc != PORSOL_OK) throw std::runtime_error(what ? std::string(what) : std::string("porsol error"));
}

}  // namespace gpu
}  // namespace Opm

#endif
