// RockTables.hpp -- RockJfunc tables (opm/porsol/common/RockJfunc.hpp:63-216) for the GB300
// transport and ImplicitCapillarity shims.
//
// The reference's ReservoirPropertyCapillary reads its RockJfunc tables from files
// (ReservoirPropertyCommon::readRocks, ReservoirPropertyCommon_impl.hpp:785-805) and keeps them
// private, so the shims take them explicitly: one table per rock in the file's column order
// (s, krw, kro, J) and the rock of every cell keyed by Cell::index() (cell_to_rock_, 0-based).
#ifndef OPM_PORSOL_GPU_ROCKTABLES_HPP
#define OPM_PORSOL_GPU_ROCKTABLES_HPP

#include <stdexcept>
#include <vector>

#include "GridFlattener.hpp"
#include "porsol_gpu.h"

namespace Opm {
namespace gpu {

struct RockTable {
    std::vector<double> s, krw, kro, J;
};

struct RockTables {
    std::vector<RockTable> rocks;
    std::vector<int> cell_rock;          // by Cell::index()
    bool use_jfunction_scaling = true;   // RockJfunc::setUseJfunctionScaling
    double sigma_cos_theta = 1.0;        // RockJfunc::setSigmaAndTheta: sigma cos(theta)
};

// Hand the tables to a transport handle (cells permuted to the flat grid's iteration order).
// Throws std::invalid_argument on ragged columns or a cell map of the wrong size.
inline int setRockTables(porsol_transport* t, const FlatGrid& fg, const RockTables& rt)
{
    std::vector<int> pos(1, 0), cell(fg.numCells());
    std::vector<double> s, krw, kro, J;
    for (const RockTable& r : rt.rocks) {
        if (r.krw.size() != r.s.size() || r.kro.size() != r.s.size() || r.J.size() != r.s.size())
            throw std::invalid_argument("rock table columns differ in length");
        s.insert(s.end(), r.s.begin(), r.s.end());
        krw.insert(krw.end(), r.krw.begin(), r.krw.end());
        kro.insert(kro.end(), r.kro.begin(), r.kro.end());
        J.insert(J.end(), r.J.begin(), r.J.end());
        pos.push_back(int(s.size()));
    }
    if (int(rt.cell_rock.size()) != fg.numCells()) throw std::invalid_argument("cell_rock needs one rock per cell");
    for (int p = 0; p < fg.numCells(); ++p) cell[p] = rt.cell_rock[fg.index_of_position[p]];
    porsol_rock_tables v{int(rt.rocks.size()), pos.data(), s.data(), krw.data(), kro.data(), J.data(), cell.data(),
                         rt.use_jfunction_scaling ? 1 : 0, rt.sigma_cos_theta};
    return porsol_transport_set_rock_tables(t, &v);
}

}  // namespace gpu
}  // namespace Opm

#endif
