// structure.cpp -- face-DOF enumeration, periodic pairing, sparsity and assembly recipe.
//
// Restates IncompFlowSolverHybrid::enumerateGridDof / enumerateBCDof
// (IncompFlowSolverHybrid.hpp:956-1110), allocateConnections / setConnections
// (:1115-1319) and the write pattern of addCellContrib (:1817-1901).  The numbering is
// the reference's: internal faces in order of first discovery by the cell iteration,
// then boundary faces in cell order.  The reference's std::find over the discovering
// cell's new faces is replaced by a scan of that cell's half-faces (same result: the
// first half-face of the earlier cell that points at the later one).
#include "structure.h"

#include <algorithm>
#include <numeric>

namespace porsol {

void HostGrid::copy_from(const porsol_grid* grid)
{
    PORSOL_REQUIRE(grid && grid->num_cells >= 0, PORSOL_ERR_BAD_ARG, "grid: null or negative cell count");
    nc = grid->num_cells;
    PORSOL_REQUIRE(grid->cell_facepos && grid->hf_neighbour && grid->hf_bid && grid->hf_area &&
                       grid->hf_centroid && grid->hf_normal && grid->cell_volume && grid->cell_centroid,
                   PORSOL_ERR_BAD_ARG, "grid: null array");
    facepos.assign(grid->cell_facepos, grid->cell_facepos + nc + 1);
    PORSOL_REQUIRE(facepos[0] == 0, PORSOL_ERR_BAD_ARG, "grid: cell_facepos[0] must be 0");
    for (int c = 0; c < nc; ++c)
        PORSOL_REQUIRE(facepos[c + 1] > facepos[c], PORSOL_ERR_BAD_ARG, "grid: cell without faces");
    nhf = facepos[nc];
    nb.assign(grid->hf_neighbour, grid->hf_neighbour + nhf);
    bid.assign(grid->hf_bid, grid->hf_bid + nhf);
    area.assign(grid->hf_area, grid->hf_area + nhf);
    fcent.assign(grid->hf_centroid, grid->hf_centroid + 3 * size_t(nhf));
    fnormal.assign(grid->hf_normal, grid->hf_normal + 3 * size_t(nhf));
    cvol.assign(grid->cell_volume, grid->cell_volume + nc);
    ccent.assign(grid->cell_centroid, grid->cell_centroid + 3 * size_t(nc));
    for (int hf = 0; hf < nhf; ++hf)
        PORSOL_REQUIRE(nb[hf] < nc && nb[hf] >= -1, PORSOL_ERR_BAD_ARG, "grid: neighbour index out of range");
}

int Structure::partner_cell(int hf) const
{
    auto j = bdry_id_map.find(hf_partner_bid[hf]);
    PORSOL_REQUIRE(j != bdry_id_map.end(), PORSOL_ERR_BAD_ARG, "periodic partner boundary id not found");
    return j->second.first;
}

int Structure::partner_dof(int hf) const
{
    auto j = bdry_id_map.find(hf_partner_bid[hf]);
    PORSOL_REQUIRE(j != bdry_id_map.end(), PORSOL_ERR_BAD_ARG, "periodic partner boundary id not found");
    return cf[g.facepos[j->second.first] + j->second.second];
}

long long Structure::slot(int i, int j) const
{
    auto b = colind.begin() + rowptr[i], e = colind.begin() + rowptr[i + 1];
    auto p = std::lower_bound(b, e, j);
    PORSOL_REQUIRE(p != e && *p == j, PORSOL_ERR_BAD_ARG, "assembly writes outside the sparsity pattern");
    return csr2sell[p - colind.begin()];
}

void Structure::build(const porsol_grid* grid, const int* flow_type, const int* partner_bid)
{
    g.copy_from(grid);
    const int nc = g.nc, nhf = g.nhf;
    hf_partner_bid.assign(nhf, 0);
    if (partner_bid) hf_partner_bid.assign(partner_bid, partner_bid + nhf);
    init_periodic.assign(nhf, 0);
    if (flow_type)
        for (int hf = 0; hf < nhf; ++hf)
            init_periodic[hf] = (g.boundary(hf) && flow_type[hf] == PORSOL_BC_PERIODIC) ? 1 : 0;
    hf_cell.resize(nhf);
    for (int c = 0; c < nc; ++c)
        for (int hf = g.facepos[c]; hf < g.facepos[c + 1]; ++hf) hf_cell[hf] = c;

    // ---- enumerateGridDof, pass 1: internal faces discovered by the earlier cell
    std::vector<int> newrank(nhf, -1);  // rank among the cell's newly discovered faces
    std::vector<int> fpos(nc + 1, 0);
    max_ncf = 0;
    int nint = 0;
    for (int c = 0; c < nc; ++c) {
        int k = 0;
        for (int hf = g.facepos[c]; hf < g.facepos[c + 1]; ++hf) {
            if (!g.boundary(hf)) {
                const int c1 = g.nb[hf];
                PORSOL_REQUIRE(c1 != c, PORSOL_ERR_BAD_ARG, "grid: cell is its own neighbour");
                if (c1 > c) newrank[hf] = k++;   // cell[c1] == -1 <=> c1 not yet visited
            }
        }
        fpos[c + 1] = fpos[c] + k;
        nint += k;
        max_ncf = std::max(max_ncf, g.nf(c));
    }
    num_internal = nint;
    // ---- pass 2: half-face -> dof
    cf.assign(nhf, -1);
    int total = nint;
    for (int c = 0; c < nc; ++c) {
        for (int hf = g.facepos[c]; hf < g.facepos[c + 1]; ++hf) {
            if (g.boundary(hf)) {
                cf[hf] = total++;
                continue;
            }
            int t = c, seek = g.nb[hf];
            if (seek < t) std::swap(t, seek);
            int found = -1;
            for (int h2 = g.facepos[t]; h2 < g.facepos[t + 1]; ++h2)
                if (g.nb[h2] == seek) {
                    found = h2;
                    break;
                }
            PORSOL_REQUIRE(found >= 0 && newrank[found] >= 0, PORSOL_ERR_BAD_ARG,
                           "grid: neighbour relation is not symmetric");
            cf[hf] = fpos[t] + newrank[found];
        }
    }
    N = total;

    // ---- enumerateBCDof: periodic partners
    bdry_id_map.clear();
    boundary_hf.clear();
    for (int hf = 0; hf < nhf; ++hf) {
        if (!g.boundary(hf)) continue;
        boundary_hf.push_back(hf);
        if (init_periodic[hf])
            bdry_id_map.insert(std::make_pair(g.bid[hf], std::make_pair(hf_cell[hf], hf - g.facepos[hf_cell[hf]])));
    }
    ppartner.clear();
    partner_hf.assign(nhf, -1);
    if (!bdry_id_map.empty()) {
        ppartner.assign(N, -1);
        for (int hf : boundary_hf) {
            if (!init_periodic[hf]) continue;
            const int dof1 = cf[hf], dof2 = partner_dof(hf);
            ppartner[dof1] = dof2;
            ppartner[dof2] = dof1;
            auto j = bdry_id_map.find(hf_partner_bid[hf]);
            partner_hf[hf] = g.facepos[j->second.first] + j->second.second;
        }
    }

    // ---- sparsity: cell cliques (setGridConnections :1241-1257), periodic couplings
    // (setBCConnections :1261-1319) and the diagonal (setrowsize(f, 1) :1128-1130)
    std::vector<int> cnt(N + 1, 0);
    auto visit = [&](auto&& emit) {
        for (int i = 0; i < N; ++i) emit(i, i);
        for (int c = 0; c < nc; ++c)
            for (int a = g.facepos[c]; a < g.facepos[c + 1]; ++a)
                for (int b = g.facepos[c]; b < g.facepos[c + 1]; ++b) emit(cf[a], cf[b]);
        if (!bdry_id_map.empty()) {
            for (int hf : boundary_hf) {
                if (!init_periodic[hf]) continue;
                const int dof1 = cf[hf], c2 = partner_cell(hf), dof2 = partner_dof(hf);
                if (dof1 >= dof2) continue;
                for (int k = g.facepos[c2]; k < g.facepos[c2 + 1]; ++k) {
                    int ii = cf[k];
                    const int pp = ppartner[ii];
                    if (pp != -1 && pp != dof1 && pp < ii) ii = pp;
                    emit(dof1, ii);
                    emit(ii, dof1);
                    emit(dof2, ii);
                    emit(ii, dof2);
                }
            }
        }
    };
    visit([&](int i, int) { cnt[i + 1]++; });
    std::vector<long long> start(N + 1, 0);
    for (int i = 0; i < N; ++i) start[i + 1] = start[i] + cnt[i + 1];
    std::vector<int> cand(start[N]);
    std::vector<long long> fill(start.begin(), start.end() - 1);
    visit([&](int i, int j) { cand[fill[i]++] = j; });
    rowptr.assign(N + 1, 0);
    for (int i = 0; i < N; ++i) {
        auto b = cand.begin() + start[i], e = cand.begin() + start[i + 1];
        std::sort(b, e);
        rowptr[i + 1] = rowptr[i] + int(std::unique(b, e) - b);
    }
    colind.resize(rowptr[N]);
    for (int i = 0; i < N; ++i) {
        auto b = cand.begin() + start[i];
        std::copy(b, b + (rowptr[i + 1] - rowptr[i]), colind.begin() + rowptr[i]);
    }
    build_sell(N, rowptr, colind, pat, &csr2sell);

    // ---- postProcessFluxes pairs (:754-807): twin half-faces of every internal face and
    // the half-faces of periodic partners, ordered by visit order (half-face index)
    pairs.clear();
    std::vector<int> first_hf(N, -1);
    for (int hf = 0; hf < nhf; ++hf) {
        if (g.boundary(hf)) continue;
        const int f = cf[hf];
        if (first_hf[f] < 0) first_hf[f] = hf;
        else {
            pairs.push_back(first_hf[f]);
            pairs.push_back(hf);
        }
    }
    if (!ppartner.empty()) {
        for (int hf : boundary_hf) {
            const int ph = partner_hf[hf];
            if (ph > hf) {
                pairs.push_back(hf);
                pairs.push_back(ph);
            }
        }
    }
}

void build_sell(int n, const std::vector<int>& rowptr, const std::vector<int>& col, SellPattern& P,
                std::vector<long long>* csr2sell)
{
    P.n = n;
    P.nslices = (n + SELL_C - 1) / SELL_C;
    P.h_slice_ptr.assign(P.nslices + 1, 0);
    P.h_rowlen.assign(n, 0);
    long long off = 0;
    for (int s = 0; s < P.nslices; ++s) {
        int w = 0;
        for (int r = s * SELL_C; r < std::min(n, (s + 1) * SELL_C); ++r) {
            P.h_rowlen[r] = rowptr[r + 1] - rowptr[r];
            w = std::max(w, P.h_rowlen[r]);
        }
        PORSOL_REQUIRE(off + (long long)w * SELL_C < (1LL << 31), PORSOL_ERR_BAD_ARG,
                       "matrix too large for 32-bit SELL offsets");
        P.h_slice_ptr[s] = int(off);
        off += (long long)w * SELL_C;
    }
    P.h_slice_ptr[P.nslices] = int(off);
    P.nent = off;
    P.h_col.assign(off, 0);
    if (csr2sell) csr2sell->assign(rowptr[n], 0);
    for (int s = 0; s < P.nslices; ++s) {
        const int w = (P.h_slice_ptr[s + 1] - P.h_slice_ptr[s]) / SELL_C;
        for (int lane = 0; lane < SELL_C; ++lane) {
            const int r = s * SELL_C + lane;
            for (int t = 0; t < w; ++t) {
                const long long k = P.h_slice_ptr[s] + (long long)t * SELL_C + lane;
                if (r < n && t < P.h_rowlen[r]) {
                    P.h_col[k] = col[rowptr[r] + t];
                    if (csr2sell) (*csr2sell)[rowptr[r] + t] = k;
                } else {
                    P.h_col[k] = r < n ? r : 0;   // padding: self column, zero value
                }
            }
        }
    }
}

void SellPattern::upload(cudaStream_t s)
{
    slice_ptr.upload(h_slice_ptr, s);
    col.upload(h_col, s);
    rowlen.upload(h_rowlen, s);
    std::vector<int> d(n, -1);
    for (int r = 0; r < n; ++r) {
        const int sl = r / SELL_C, lane = r % SELL_C;
        for (int t = 0; t < h_rowlen[r]; ++t) {
            const long long k = h_slice_ptr[sl] + (long long)t * SELL_C + lane;
            if (h_col[k] == r) d[r] = int(k);
        }
        PORSOL_REQUIRE(d[r] >= 0, PORSOL_ERR_BAD_ARG, "matrix row without diagonal");
    }
    diag.upload(d, s);
    PORSOL_CUDA(cudaStreamSynchronize(s));   // host vectors may be freed by the caller
}

// ---------------------------------------------------------------------------
// Assembly recipe: enumerate every write of addCellContrib (:1817-1901) in the reference
// order.  Matrix writes become (slot <- +/- packed local entry); right-hand-side writes are
// folded per local row into one per-half-face value computed by the cell kernel
// (rrow: all rhs_[ii] updates made while processing local row r, except the periodic
// +/-b terms, which go through pb).
void Recipe::build(const Structure& S, const int* flow_type, int npk)
{
    const HostGrid& g = S.g;
    const int nc = g.nc, nhf = g.nhf;
    kind.assign(nhf, HK_INTERNAL);
    do_reg = true;
    for (int hf : S.boundary_hf) {
        const int t = flow_type[hf];
        if (t == PORSOL_BC_DIRICHLET) {
            kind[hf] = HK_DIRICHLET;
            do_reg = false;
        } else if (t == PORSOL_BC_PERIODIC) {
            PORSOL_REQUIRE(S.init_periodic[hf], PORSOL_ERR_BAD_ARG,
                           "periodic condition on a face that was not periodic at init");
            kind[hf] = (S.partner_dof(hf) < S.cf[hf]) ? HK_PERIODIC_LO : HK_PERIODIC_HI;
        } else if (t == PORSOL_BC_NEUMANN) {
            kind[hf] = HK_NEUMANN;
        } else {
            throw Error(PORSOL_ERR_BAD_ARG, "unknown flow boundary condition type");
        }
    }
    const long long nent = S.pat.nent;
    const int N = S.N;
    auto enc = [&](int c, int r, int s, bool neg) -> int {
        const long long idx = (long long)packed_index(r, s) * nc + c;
        PORSOL_REQUIRE(idx < (1LL << 31) - 1, PORSOL_ERR_BAD_ARG, "grid too large for 32-bit recipe");
        return neg ? ~int(idx) : int(idx);
    };
    // kind codes of rhs pieces: 0 = +rrow[hf], 1 = +pb[hf], 2 = -pb[hf]
    auto visit = [&](auto&& emat, auto&& erhs) {
        for (int c = 0; c < nc; ++c) {
            const int f0 = g.facepos[c], nf = g.nf(c);
            for (int r = 0; r < nf; ++r) {
                int ii = S.cf[f0 + r];
                const int t = kind[f0 + r];
                if (t == HK_DIRICHLET) {
                    emat(S.slot(ii, ii), enc(c, r, r, false), true);
                    erhs(ii, (f0 + r) * 4 + 0, true);
                    continue;
                }
                if (t == HK_PERIODIC_HI || t == HK_PERIODIC_LO) {
                    const int pp = S.partner_dof(f0 + r);
                    emat(S.slot(ii, ii), enc(c, r, r, false), false);
                    emat(S.slot(ii, pp), enc(c, r, r, true), false);
                    erhs(ii, (f0 + r) * 4 + 1, false);
                    emat(S.slot(pp, ii), enc(c, r, r, true), false);
                    emat(S.slot(pp, pp), enc(c, r, r, false), false);
                    erhs(pp, (f0 + r) * 4 + 2, false);
                    ii = std::min(ii, pp);
                }
                for (int cc = 0; cc < nf; ++cc) {
                    int jj = S.cf[f0 + cc];
                    const int tc = kind[f0 + cc];
                    if (tc == HK_DIRICHLET) continue;
                    if (tc == HK_PERIODIC_LO) jj = S.partner_dof(f0 + cc);
                    emat(S.slot(ii, jj), enc(c, r, cc, false), false);
                }
                erhs(ii, (f0 + r) * 4 + 0, false);
            }
        }
    };
    (void)npk;
    // pass 1: counts (an assignment resets the count of its target)
    std::vector<int> scount(nent, 0), rcount(N, 0);
    visit([&](long long k, int, bool assign) { scount[k] = assign ? 1 : scount[k] + 1; },
          [&](int i, int, bool assign) { rcount[i] = assign ? 1 : rcount[i] + 1; });
    h_slot_ptr.assign(nent + 1, 0);
    for (long long k = 0; k < nent; ++k) h_slot_ptr[k + 1] = h_slot_ptr[k] + scount[k];
    h_rhs_ptr.assign(N + 1, 0);
    for (int i = 0; i < N; ++i) h_rhs_ptr[i + 1] = h_rhs_ptr[i] + rcount[i];
    h_slot_ent.assign(h_slot_ptr[nent], 0);
    h_rhs_ent.assign(h_rhs_ptr[N], 0);
    std::fill(scount.begin(), scount.end(), 0);
    std::fill(rcount.begin(), rcount.end(), 0);
    visit([&](long long k, int e, bool assign) {
              if (assign) scount[k] = 0;
              h_slot_ent[h_slot_ptr[k] + scount[k]++] = e;
          },
          [&](int i, int e, bool assign) {
              if (assign) rcount[i] = 0;
              h_rhs_ent[h_rhs_ptr[i] + rcount[i]++] = e;
          });
    valid = true;
}

}  // namespace porsol
