// structure.cpp -- face-DOF enumeration, periodic pairing, sparsity and assembly recipe.
//
// Restates IncompFlowSolverHybrid::enumerateGridDof / enumerateBCDof
// (IncompFlowSolverHybrid.hpp:956-1110), allocateConnections / setConnections
// (:1115-1319) and the write pattern of addCellContrib (:1817-1901).  The numbering is
// the reference's: internal faces in order of first discovery by the cell iteration,
// then boundary faces in cell order.  The reference's std::find over the discovering
// cell's new faces is replaced by a scan of that cell's half-faces (same result: the
// first half-face of the earlier cell that points at the later one).
//
// The build runs on the host's cores: every pass is a loop over cells, half-faces, rows or
// slices split into contiguous chunks, with prefix sums between passes where the reference's
// sequential counters number things in visit order.  Row sparsity is collected in any order and
// then sorted; the assembly recipe's per-slot entries are placed by atomic counters and then
// ordered by cell (a stable sort: one cell's writes arrive in emission order), which is the
// serial visit order.  The result
// is identical to a serial build.
#include "structure.h"

#include <algorithm>
#include <atomic>
#include <exception>
#include <mutex>
#include <numeric>
#include <thread>

namespace porsol {

namespace {

int host_threads()
{
    static const int n = [] {
        const unsigned h = std::thread::hardware_concurrency();
        return int(std::max(1u, std::min(h == 0 ? 1u : h, 32u)));
    }();
    return n;
}

// fn(begin, end, chunk) over [0, n) in contiguous chunks (chunk order = index order); serial
// below `grain` items per extra thread.  An exception in any chunk is rethrown on the calling
// thread after all chunks have finished (the first one caught).
template <class F>
int parallel_chunks(long long n, F&& fn, long long grain = 1 << 16)
{
    int T = int(std::min<long long>(host_threads(), std::max<long long>(1, n / grain)));
    if (T <= 1) {
        fn(0LL, n, 0);
        return 1;
    }
    std::vector<std::thread> th;
    th.reserve(T - 1);
    std::exception_ptr err;
    std::mutex err_mutex;
    auto run = [&](long long b, long long e, int t) {
        try {
            fn(b, e, t);
        } catch (...) {
            std::lock_guard<std::mutex> lk(err_mutex);
            if (!err) err = std::current_exception();
        }
    };
    auto range = [&](int t, long long& b, long long& e) {
        b = n * t / T;
        e = n * (t + 1) / T;
    };
    for (int t = 1; t < T; ++t) {
        long long b, e;
        range(t, b, e);
        th.emplace_back([&run, b, e, t] { run(b, e, t); });
    }
    long long b, e;
    range(0, b, e);
    run(b, e, 0);
    for (auto& x : th) x.join();
    if (err) std::rethrow_exception(err);
    return T;
}

template <class F>
void parallel_for(long long n, F&& fn, long long grain = 1 << 16)
{
    parallel_chunks(
        n, [&](long long b, long long e, int) {
            for (long long i = b; i < e; ++i) fn(i);
        },
        grain);
}

inline int atomic_inc(int* p) { return __atomic_fetch_add(p, 1, __ATOMIC_RELAXED); }

template <class V, class T>
void parallel_fill(V& v, size_t n, T value)
{
    v.resize(n);
    parallel_for((long long)n, [&](long long i) { v[i] = value; });
}

// out[0] = 0, out[i + 1] = out[i] + cnt(i) for i < n (out holds n + 1 values)
template <class Out, class F>
void parallel_exclusive_scan(long long n, F&& cnt, Out* out)
{
    std::vector<Out> part(host_threads() + 1, Out(0));
    const int T = parallel_chunks(n, [&](long long b, long long e, int t) {
        Out s = 0;
        for (long long i = b; i < e; ++i) s += Out(cnt(i));
        part[t + 1] = s;
    });
    for (int t = 0; t < T; ++t) part[t + 1] += part[t];
    parallel_chunks(n, [&](long long b, long long e, int t) {
        Out s = part[t];
        for (long long i = b; i < e; ++i) {
            out[i] = s;
            s += Out(cnt(i));
        }
    });
    out[n] = part[T];
}

}  // namespace

void HostGrid::copy_from(const porsol_grid* grid, bool geometry)
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
    std::atomic<bool> bad{false};
    parallel_for(nhf, [&](long long hf) {
        if (nb[hf] >= nc || nb[hf] < -1) bad = true;
    });
    PORSOL_REQUIRE(!bad, PORSOL_ERR_BAD_ARG, "grid: neighbour index out of range");
    if (geometry) {
        area.assign(grid->hf_area, grid->hf_area + nhf);
        fcent.assign(grid->hf_centroid, grid->hf_centroid + 3 * size_t(nhf));
        fnormal.assign(grid->hf_normal, grid->hf_normal + 3 * size_t(nhf));
        cvol.assign(grid->cell_volume, grid->cell_volume + nc);
        ccent.assign(grid->cell_centroid, grid->cell_centroid + 3 * size_t(nc));
    } else {
        area.clear();
        fcent.clear();
        fnormal.clear();
        cvol.clear();
        ccent.clear();
    }
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
    g.copy_from(grid, false);
    const int nc = g.nc, nhf = g.nhf;
    hf_partner_bid.assign(nhf, 0);
    if (partner_bid) hf_partner_bid.assign(partner_bid, partner_bid + nhf);
    init_periodic.assign(nhf, 0);
    if (flow_type)
        parallel_for(nhf, [&](long long hf) {
            init_periodic[hf] = (g.boundary(int(hf)) && flow_type[hf] == PORSOL_BC_PERIODIC) ? 1 : 0;
        });
    hf_cell.resize(nhf);
    parallel_for(nc, [&](long long c) {
        for (int hf = g.facepos[c]; hf < g.facepos[c + 1]; ++hf) hf_cell[hf] = int(c);
    });

    // ---- enumerateGridDof, pass 1: internal faces discovered by the earlier cell
    std::vector<int> newrank(nhf, -1);  // rank among the cell's newly discovered faces
    std::vector<int> fpos(nc + 1, 0);
    std::atomic<bool> self_nb{false};
    std::vector<int> chunk_max(host_threads(), 0);
    parallel_chunks(nc, [&](long long b, long long e, int t) {
        int mx = 0;
        for (long long c = b; c < e; ++c) {
            int k = 0;
            for (int hf = g.facepos[c]; hf < g.facepos[c + 1]; ++hf) {
                if (!g.boundary(hf)) {
                    const int c1 = g.nb[hf];
                    if (c1 == c) self_nb = true;
                    if (c1 > c) newrank[hf] = k++;   // cell[c1] == -1 <=> c1 not yet visited
                }
            }
            fpos[c + 1] = k;
            mx = std::max(mx, g.nf(int(c)));
        }
        chunk_max[t] = mx;
    });
    PORSOL_REQUIRE(!self_nb, PORSOL_ERR_BAD_ARG, "grid: cell is its own neighbour");
    max_ncf = *std::max_element(chunk_max.begin(), chunk_max.end());
    for (int c = 0; c < nc; ++c) fpos[c + 1] += fpos[c];
    const int nint = fpos[nc];
    num_internal = nint;
    // ---- pass 2: half-face -> dof; boundary faces numbered after the internal ones in
    // half-face order (chunk offsets from a count pass)
    cf.assign(nhf, -1);
    const int T = host_threads();
    std::vector<long long> bcount(T + 1, 0);
    std::atomic<bool> asym{false};
    const int used = parallel_chunks(nc, [&](long long b, long long e, int t) {
        long long k = 0;
        for (int hf = g.facepos[b]; hf < g.facepos[e]; ++hf) k += g.boundary(hf) ? 1 : 0;
        bcount[t + 1] = k;
    });
    for (int t = 0; t < used; ++t) bcount[t + 1] += bcount[t];
    parallel_chunks(nc, [&](long long b, long long e, int t) {
        long long next = nint + bcount[t];
        for (long long c = b; c < e; ++c) {
            for (int hf = g.facepos[c]; hf < g.facepos[c + 1]; ++hf) {
                if (g.boundary(hf)) {
                    cf[hf] = int(next++);
                    continue;
                }
                int tc = int(c), seek = g.nb[hf];
                if (seek < tc) std::swap(tc, seek);
                int found = -1;
                for (int h2 = g.facepos[tc]; h2 < g.facepos[tc + 1]; ++h2)
                    if (g.nb[h2] == seek) {
                        found = h2;
                        break;
                    }
                if (found < 0 || newrank[found] < 0) {
                    asym = true;
                    continue;
                }
                cf[hf] = fpos[tc] + newrank[found];
            }
        }
    });
    PORSOL_REQUIRE(!asym, PORSOL_ERR_BAD_ARG, "grid: neighbour relation is not symmetric");
    N = int(nint + bcount[used]);

    // ---- enumerateBCDof: periodic partners
    bdry_id_map.clear();
    boundary_hf.clear();
    boundary_hf.reserve(size_t(bcount[used]));
    for (int hf = 0; hf < nhf; ++hf) {
        if (!g.boundary(hf)) continue;
        boundary_hf.push_back(hf);
        if (init_periodic[hf])
            bdry_id_map.insert(std::make_pair(g.bid[hf], std::make_pair(hf_cell[hf], hf - g.facepos[hf_cell[hf]])));
    }
    ppartner.clear();
    partner_hf.assign(nhf, -1);
    std::vector<int> per_hf;   // periodic boundary half-faces in order
    if (!bdry_id_map.empty()) {
        ppartner.assign(N, -1);
        for (int hf : boundary_hf) {
            if (!init_periodic[hf]) continue;
            per_hf.push_back(hf);
            const int dof1 = cf[hf], dof2 = partner_dof(hf);
            ppartner[dof1] = dof2;
            ppartner[dof2] = dof1;
            auto j = bdry_id_map.find(hf_partner_bid[hf]);
            partner_hf[hf] = g.facepos[j->second.first] + j->second.second;
        }
    }

    // ---- sparsity: cell cliques (setGridConnections :1241-1257), periodic couplings
    // (setBCConnections :1261-1319) and the diagonal (setrowsize(f, 1) :1128-1130).  Candidates
    // are collected per row in any order (atomic positions), then sorted and made unique.
    HVec<int> cnt;
    parallel_fill(cnt, size_t(N) + 1, 0);
    auto periodic_visit = [&](auto&& emit) {
        for (int hf : per_hf) {
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
    };
    parallel_for(N, [&](long long i) { cnt[i + 1] = 1; });   // the diagonal
    parallel_for(nc, [&](long long c) {
        const int nf = g.nf(int(c));
        for (int a = g.facepos[c]; a < g.facepos[c + 1]; ++a) {
            int* p = &cnt[cf[a] + 1];
            __atomic_fetch_add(p, nf, __ATOMIC_RELAXED);
        }
    });
    periodic_visit([&](int i, int) { cnt[i + 1]++; });
    HVec<long long> start(size_t(N) + 1);
    parallel_exclusive_scan(N, [&](long long i) { return cnt[i + 1]; }, start.data());
    HVec<int> cand(size_t(start[N]));
    HVec<int> fill(N);
    parallel_for(N, [&](long long i) {
        cand[start[i]] = int(i);
        fill[i] = 1;
    });
    parallel_for(nc, [&](long long c) {
        for (int a = g.facepos[c]; a < g.facepos[c + 1]; ++a) {
            const int i = cf[a];
            const int nf = g.nf(int(c));
            const int p0 = __atomic_fetch_add(&fill[i], nf, __ATOMIC_RELAXED);
            int q = 0;
            for (int b = g.facepos[c]; b < g.facepos[c + 1]; ++b) cand[start[i] + p0 + q++] = cf[b];
        }
    });
    periodic_visit([&](int i, int j) { cand[start[i] + fill[i]++] = j; });
    HVec<int> ulen(N);
    parallel_for(N, [&](long long i) {
        auto b = cand.begin() + start[i], e = cand.begin() + start[i + 1];
        std::sort(b, e);
        ulen[i] = int(std::unique(b, e) - b);
    });
    rowptr.resize(size_t(N) + 1);
    parallel_exclusive_scan(N, [&](long long i) { return ulen[i]; }, rowptr.data());
    colind.resize(rowptr[N]);
    parallel_for(N, [&](long long i) {
        auto b = cand.begin() + start[i];
        std::copy(b, b + ulen[i], colind.begin() + rowptr[i]);
    });
    HVec<int>().swap(cand);
    build_sell(N, rowptr, colind, pat, &csr2sell);

    // ---- postProcessFluxes pairs (:754-807): twin half-faces of every internal face and
    // the half-faces of periodic partners, ordered by visit order (half-face index)
    pairs.clear();
    {
        std::vector<int> first_hf(N, nhf);
        parallel_for(nhf, [&](long long hf) {
            if (g.boundary(int(hf))) return;
            int* p = &first_hf[cf[hf]];
            int cur = __atomic_load_n(p, __ATOMIC_RELAXED);
            while (int(hf) < cur && !__atomic_compare_exchange_n(p, &cur, int(hf), true, __ATOMIC_RELAXED,
                                                                 __ATOMIC_RELAXED)) {
            }
        });
        // the second half-face of each internal face closes a pair, in half-face order
        std::vector<long long> pc(T + 1, 0);
        const int u2 = parallel_chunks(nhf, [&](long long b, long long e, int t) {
            long long k = 0;
            for (long long hf = b; hf < e; ++hf)
                if (!g.boundary(int(hf)) && first_hf[cf[hf]] != hf) ++k;
            pc[t + 1] = k;
        });
        for (int t = 0; t < u2; ++t) pc[t + 1] += pc[t];
        pairs.resize(size_t(2 * pc[u2]));
        parallel_chunks(nhf, [&](long long b, long long e, int t) {
            long long k = pc[t];
            for (long long hf = b; hf < e; ++hf)
                if (!g.boundary(int(hf)) && first_hf[cf[hf]] != hf) {
                    pairs[2 * k] = first_hf[cf[hf]];
                    pairs[2 * k + 1] = int(hf);
                    ++k;
                }
        });
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

void build_sell(int n, const HVec<int>& rowptr, const HVec<int>& col, SellPattern& P, HVec<int>* csr2sell)
{
    P.n = n;
    P.nslices = (n + SELL_C - 1) / SELL_C;
    P.h_slice_ptr.resize(size_t(P.nslices) + 1);
    P.h_rowlen.resize(n);
    std::vector<int> width(P.nslices, 0);
    parallel_for(P.nslices, [&](long long s) {
        int w = 0;
        for (int r = int(s) * SELL_C; r < std::min(n, int(s + 1) * SELL_C); ++r) {
            P.h_rowlen[r] = rowptr[r + 1] - rowptr[r];
            w = std::max(w, P.h_rowlen[r]);
        }
        width[s] = w;
    });
    long long off = 0;
    for (int s = 0; s < P.nslices; ++s) {
        PORSOL_REQUIRE(off + (long long)width[s] * SELL_C < (1LL << 31), PORSOL_ERR_BAD_ARG,
                       "matrix too large for 32-bit SELL offsets");
        P.h_slice_ptr[s] = int(off);
        off += (long long)width[s] * SELL_C;
    }
    P.h_slice_ptr[P.nslices] = int(off);
    P.nent = off;
    P.h_col.resize(off);                          // every slot is written below
    if (csr2sell) csr2sell->resize(rowptr[n]);    // every CSR entry has its slot
    parallel_for(P.nslices, [&](long long s) {
        const int w = (P.h_slice_ptr[s + 1] - P.h_slice_ptr[s]) / SELL_C;
        for (int lane = 0; lane < SELL_C; ++lane) {
            const int r = int(s) * SELL_C + lane;
            for (int t = 0; t < w; ++t) {
                const long long k = P.h_slice_ptr[s] + (long long)t * SELL_C + lane;
                if (r < n && t < P.h_rowlen[r]) {
                    P.h_col[k] = col[rowptr[r] + t];
                    if (csr2sell) (*csr2sell)[rowptr[r] + t] = int(k);
                } else {
                    P.h_col[k] = r < n ? r : 0;   // padding: self column, zero value
                }
            }
        }
    });
}

void SellPattern::upload(cudaStream_t s)
{
    slice_ptr.upload(h_slice_ptr, s);
    col.upload(h_col, s);
    rowlen.upload(h_rowlen, s);
    std::vector<int> d(n, -1);
    parallel_for(n, [&](long long r) {
        const int sl = int(r) / SELL_C, lane = int(r) % SELL_C;
        for (int t = 0; t < h_rowlen[r]; ++t) {
            const long long k = h_slice_ptr[sl] + (long long)t * SELL_C + lane;
            if (h_col[k] == r) d[r] = int(k);
        }
    });
    for (int r = 0; r < n; ++r) PORSOL_REQUIRE(d[r] >= 0, PORSOL_ERR_BAD_ARG, "matrix row without diagonal");
    diag.upload(d, s);
    PORSOL_CUDA(cudaStreamSynchronize(s));   // host vectors may be freed by the caller
}

// ---------------------------------------------------------------------------
// Assembly recipe: enumerate every write of addCellContrib (:1817-1901) in the reference
// order.  Matrix writes become (slot <- +/- packed local entry); right-hand-side writes are
// folded per local row into one per-half-face value computed by the cell kernel
// (rrow: all rhs_[ii] updates made while processing local row r, except the periodic
// +/-b terms, which go through pb).  The writes of addCellContrib that assign instead of
// adding (Dirichlet rows) touch only the diagonal slot and the right-hand side of a face that
// belongs to one cell, which nothing else writes; so every target's entry list is the
// sequence of its writes, and the cells can be visited in parallel.
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
    // partner dof of every periodic half-face (the hash lookups once, before the parallel visit)
    std::vector<int> pdof(nhf, -1);
    for (int hf : S.boundary_hf)
        if (kind[hf] == HK_PERIODIC_HI || kind[hf] == HK_PERIODIC_LO) pdof[hf] = S.partner_dof(hf);
    const long long nent = S.pat.nent;
    const int N = S.N;
    PORSOL_REQUIRE((long long)npk * nc < (1LL << 31) - 1, PORSOL_ERR_BAD_ARG, "grid too large for 32-bit recipe");
    auto enc = [&](int c, int r, int s, bool neg) -> int {
        const long long idx = (long long)packed_index(r, s) * nc + c;
        return neg ? ~int(idx) : int(idx);
    };
    // the writes of cell c in the serial order; emat(slot, entry, seq), erhs(row, entry, seq)
    // (kind codes of rhs pieces: 0 = +rrow[hf], 1 = +pb[hf], 2 = -pb[hf])
    auto visit_cell = [&](int c, auto&& emat, auto&& erhs) {
        int seq = 0;
        const int f0 = g.facepos[c], nf = g.nf(c);
        for (int r = 0; r < nf; ++r) {
            int ii = S.cf[f0 + r];
            const int t = kind[f0 + r];
            if (t == HK_DIRICHLET) {
                emat(S.slot(ii, ii), enc(c, r, r, false), seq++);
                erhs(ii, (f0 + r) * 4 + 0, seq++);
                continue;
            }
            if (t == HK_PERIODIC_HI || t == HK_PERIODIC_LO) {
                const int pp = pdof[f0 + r];
                emat(S.slot(ii, ii), enc(c, r, r, false), seq++);
                emat(S.slot(ii, pp), enc(c, r, r, true), seq++);
                erhs(ii, (f0 + r) * 4 + 1, seq++);
                emat(S.slot(pp, ii), enc(c, r, r, true), seq++);
                emat(S.slot(pp, pp), enc(c, r, r, false), seq++);
                erhs(pp, (f0 + r) * 4 + 2, seq++);
                ii = std::min(ii, pp);
            }
            for (int cc = 0; cc < nf; ++cc) {
                int jj = S.cf[f0 + cc];
                const int tc = kind[f0 + cc];
                if (tc == HK_DIRICHLET) continue;
                if (tc == HK_PERIODIC_LO) jj = pdof[f0 + cc];
                emat(S.slot(ii, jj), enc(c, r, cc, false), seq++);
            }
            erhs(ii, (f0 + r) * 4 + 0, seq++);
        }
    };
    // pass 1: counts
    HVec<int> scount, rcount;
    parallel_fill(scount, size_t(nent), 0);
    parallel_fill(rcount, size_t(N), 0);
    parallel_for(nc, [&](long long c) {
        visit_cell(int(c), [&](long long k, int, int) { atomic_inc(&scount[k]); },
                   [&](int i, int, int) { atomic_inc(&rcount[i]); });
    }, 1 << 12);
    h_slot_ptr.resize(size_t(nent) + 1);
    parallel_exclusive_scan(nent, [&](long long k) { return scount[k]; }, h_slot_ptr.data());
    h_rhs_ptr.resize(size_t(N) + 1);
    parallel_exclusive_scan(N, [&](long long i) { return rcount[i]; }, h_rhs_ptr.data());
    // pass 2: entries at atomic positions.  A cell's writes to one target come from one thread in
    // emission order, so their positions increase; a stable sort of every list by cell then gives
    // the serial visit order.
    h_slot_ent.resize(size_t(h_slot_ptr[nent]));
    h_rhs_ent.resize(size_t(h_rhs_ptr[N]));
    parallel_fill(scount, size_t(nent), 0);
    parallel_fill(rcount, size_t(N), 0);
    parallel_for(nc, [&](long long c) {
        visit_cell(
            int(c), [&](long long k, int e, int) { h_slot_ent[h_slot_ptr[k] + atomic_inc(&scount[k])] = e; },
            [&](int i, int e, int) { h_rhs_ent[h_rhs_ptr[i] + atomic_inc(&rcount[i])] = e; });
    }, 1 << 12);
    // stable insertion sort by cell (lists hold a few entries)
    auto order = [](HVec<int>& ent, long long b, long long e, auto&& cell) {
        for (long long i = b + 1; i < e; ++i) {
            const int ev = ent[i];
            const int kc = cell(ev);
            long long j = i - 1;
            while (j >= b && cell(ent[j]) > kc) {
                ent[j + 1] = ent[j];
                --j;
            }
            ent[j + 1] = ev;
        }
    };
    auto slot_cell = [nc](int e) { return (e < 0 ? ~e : e) % nc; };
    auto rhs_cell = [&S](int e) { return S.hf_cell[e >> 2]; };
    parallel_for(nent, [&](long long k) { order(h_slot_ent, h_slot_ptr[k], h_slot_ptr[k + 1], slot_cell); });
    parallel_for(N, [&](long long i) { order(h_rhs_ent, h_rhs_ptr[i], h_rhs_ptr[i + 1], rhs_cell); });
    valid = true;
}

}  // namespace porsol
