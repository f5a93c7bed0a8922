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
#include <cmath>
#include <cstdlib>
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

// Lattice indices of the cell centroids along one axis: the sorted distinct coordinates (values
// within 1e-9 of the axis extent merge) and each cell's position among them.
int lattice_axis(const double* cent, int nc, int a, std::vector<int>& idx)
{
    std::vector<double> v(nc);
    double lo = 1e300, hi = -1e300;
    for (int c = 0; c < nc; ++c) {
        v[c] = cent[3 * size_t(c) + a];
        lo = std::min(lo, v[c]);
        hi = std::max(hi, v[c]);
    }
    if (!(hi >= lo)) return -1;   // non-finite coordinates
    const double tol = 1e-9 * std::max(hi - lo, 1e-300);
    std::vector<double> u(v);
    std::sort(u.begin(), u.end());
    std::vector<double> w;
    for (double x : u)
        if (w.empty() || x - w.back() > tol) w.push_back(x);
    idx.resize(nc);
    for (int c = 0; c < nc; ++c) {
        auto it = std::lower_bound(w.begin(), w.end(), v[c] - tol);
        if (it == w.end() || std::fabs(*it - v[c]) > tol) return -1;
        idx[c] = int(it - w.begin());
    }
    return int(w.size());
}

// Reverse Cuthill-McKee order of the cell graph (cells adjacent through internal faces): per
// connected component a breadth-first search from a pseudo-peripheral cell, neighbours taken in
// order of increasing degree, the whole sequence reversed.
std::vector<int> rcm_order(const HostGrid& g)
{
    const int nc = g.nc;
    std::vector<int> deg(nc, 0);
    for (int c = 0; c < nc; ++c)
        for (int hf = g.facepos[c]; hf < g.facepos[c + 1]; ++hf) deg[c] += g.nb[hf] >= 0 ? 1 : 0;
    std::vector<int> stamp(nc, -1), level(nc, 0), queue;
    queue.reserve(nc);
    int run = 0;
    // breadth-first levels from r (stamp marks this run); returns the last level's cells
    auto bfs = [&](int r, std::vector<int>& last) {
        ++run;
        queue.clear();
        queue.push_back(r);
        stamp[r] = run;
        level[r] = 0;
        int maxl = 0;
        for (size_t h = 0; h < queue.size(); ++h) {
            const int u = queue[h];
            maxl = std::max(maxl, level[u]);
            for (int hf = g.facepos[u]; hf < g.facepos[u + 1]; ++hf) {
                const int v = g.nb[hf];
                if (v >= 0 && stamp[v] != run) {
                    stamp[v] = run;
                    level[v] = level[u] + 1;
                    queue.push_back(v);
                }
            }
        }
        last.clear();
        for (int u : queue)
            if (level[u] == maxl) last.push_back(u);
        return maxl;
    };
    std::vector<char> placed(nc, 0);
    std::vector<int> order;
    order.reserve(nc);
    std::vector<int> last, nbrs;
    for (int seed = 0; seed < nc; ++seed) {
        if (placed[seed]) continue;
        // pseudo-peripheral start: repeat "farthest cell of least degree" while the eccentricity grows
        int r = seed;
        int ecc = bfs(r, last);
        for (int it = 0; it < 8; ++it) {
            int best = last[0];
            for (int u : last)
                if (deg[u] < deg[best] || (deg[u] == deg[best] && u < best)) best = u;
            std::vector<int> last2;
            const int e2 = bfs(best, last2);
            if (e2 <= ecc) break;
            r = best;
            ecc = e2;
            last.swap(last2);
        }
        const size_t first = order.size();
        order.push_back(r);
        placed[r] = 1;
        for (size_t h = first; h < order.size(); ++h) {
            const int u = order[h];
            nbrs.clear();
            for (int hf = g.facepos[u]; hf < g.facepos[u + 1]; ++hf) {
                const int v = g.nb[hf];
                if (v >= 0 && !placed[v]) {
                    placed[v] = 1;
                    nbrs.push_back(v);
                }
            }
            std::sort(nbrs.begin(), nbrs.end(),
                      [&](int a, int b) { return deg[a] != deg[b] ? deg[a] < deg[b] : a < b; });
            order.insert(order.end(), nbrs.begin(), nbrs.end());
        }
    }
    std::reverse(order.begin(), order.end());
    return order;
}

// Visiting order of the cells for the internal face numbering.  Cells whose centroids form a
// Cartesian lattice (nx x ny x nz distinct coordinates, one cell per node) are taken in lattice
// order with the axis of fewest cells fastest and the axis of most cells slowest, which gives the
// smallest bandwidth of the orders along the axes (n_fast * n_mid cells); other grids in reverse
// Cuthill-McKee order.
std::vector<int> cell_order(const porsol_grid* grid, const HostGrid& g)
{
    const int nc = g.nc;
    std::vector<int> idx[3];
    int n[3] = {-1, -1, -1};
    bool lattice = grid->cell_centroid != nullptr;
    for (int a = 0; a < 3 && lattice; ++a) {
        n[a] = lattice_axis(grid->cell_centroid, nc, a, idx[a]);
        lattice = n[a] > 0;
    }
    if (lattice && (long long)n[0] * n[1] * n[2] == nc) {
        int ax[3] = {0, 1, 2};   // slowest .. fastest
        std::stable_sort(ax, ax + 3, [&](int a, int b) { return n[a] > n[b]; });
        std::vector<int> order(nc, -1);
        bool ok = true;
        for (int c = 0; c < nc && ok; ++c) {
            const long long key =
                (long long)idx[ax[2]][c] + (long long)n[ax[2]] * (idx[ax[1]][c] + (long long)n[ax[1]] * idx[ax[0]][c]);
            if (order[key] >= 0) ok = false;
            else order[key] = c;
        }
        if (ok) return order;
    }
    return rcm_order(g);
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

    // ---- internal numbering (not with periodic faces: their couplings span the grid in any order)
    dof_perm.clear();
    dof_iperm.clear();
    cf_int.clear();
    ref_pattern_built = false;
    auto csr_bandwidth = [&](const int* perm) {
        std::vector<int> part(host_threads(), 0);
        parallel_chunks(N, [&](long long b, long long e, int t) {
            int m = 0;
            for (long long i = b; i < e; ++i) {
                const int pi = perm ? perm[i] : int(i);
                for (long long k = rowptr[i]; k < rowptr[i + 1]; ++k)
                    m = std::max(m, std::abs((perm ? perm[colind[k]] : colind[k]) - pi));
            }
            part[t] = std::max(part[t], m);
        });
        return *std::max_element(part.begin(), part.end());
    };
    bandwidth_ref = csr_bandwidth(nullptr);
    bandwidth = bandwidth_ref;
    if (per_hf.empty() && nc > 1) {
        const std::vector<int> order = cell_order(grid, g);
        std::vector<int> perm(N, -1);
        int next = 0;
        for (int c : order)
            for (int hf = g.facepos[c]; hf < g.facepos[c + 1]; ++hf)
                if (perm[cf[hf]] < 0) perm[cf[hf]] = next++;
        if (next == N) {
            const int bw = csr_bandwidth(perm.data());
            if (bw < bandwidth_ref) {
                bandwidth = bw;
                dof_perm.swap(perm);
            }
        }
    }
    if (dof_perm.empty()) {
        build_sell(N, rowptr, colind, pat, &csr2sell);
    } else {
        dof_iperm.assign(N, 0);
        for (int i = 0; i < N; ++i) dof_iperm[dof_perm[i]] = i;
        cf_int.resize(nhf);
        parallel_for(nhf, [&](long long hf) { cf_int[hf] = dof_perm[cf[hf]]; });
        // the system's rows in the internal order, columns renumbered and sorted; src = CSR entry
        HVec<int> rp(size_t(N) + 1), ci(colind.size()), src(colind.size());
        parallel_exclusive_scan(N, [&](long long r) { return rowptr[dof_iperm[r] + 1] - rowptr[dof_iperm[r]]; },
                                rp.data());
        parallel_for(N, [&](long long r) {
            const int i = dof_iperm[r];
            const long long b = rowptr[i], len = rowptr[i + 1] - b, o = rp[r];
            for (long long q = 0; q < len; ++q) {
                ci[o + q] = dof_perm[colind[b + q]];
                src[o + q] = int(b + q);
            }
            for (long long q = 1; q < len; ++q) {   // insertion sort by column (rows are short)
                const int kc = ci[o + q], ks = src[o + q];
                long long p = q - 1;
                while (p >= 0 && ci[o + p] > kc) {
                    ci[o + p + 1] = ci[o + p];
                    src[o + p + 1] = src[o + p];
                    --p;
                }
                ci[o + p + 1] = kc;
                src[o + p + 1] = ks;
            }
        });
        HVec<int> c2s;
        build_sell(N, rp, ci, pat, &c2s);
        csr2sell.resize(colind.size());
        parallel_for((long long)colind.size(), [&](long long k) { csr2sell[src[k]] = c2s[k]; });
    }

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

void Structure::build_ref_pattern()
{
    if (ref_pattern_built || !renumbered()) return;
    HVec<int> c2s;
    build_sell(N, rowptr, colind, pat_ref, &c2s);
    ref_slot_src.resize(size_t(pat_ref.nent));
    parallel_for(pat_ref.nent, [&](long long k) { ref_slot_src[k] = -1; });
    parallel_for((long long)c2s.size(), [&](long long k) { ref_slot_src[c2s[k]] = int(csr2sell[k]); });
    ref_pattern_built = true;
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
    // 16-bit column offsets when they fit (rows past n in the last slice: offset 0)
    std::atomic<bool> fits{true};
    std::vector<short> off(static_cast<size_t>(nent));
    parallel_for(nslices, [&](long long sl) {
        const int w = (h_slice_ptr[sl + 1] - h_slice_ptr[sl]) / SELL_C;
        for (int lane = 0; lane < SELL_C; ++lane) {
            const int r = int(sl) * SELL_C + lane;
            for (int t = 0; t < w; ++t) {
                const long long k = h_slice_ptr[sl] + (long long)t * SELL_C + lane;
                const int o = r < n ? h_col[k] - r : 0;
                if (o < -32768 || o > 32767) fits = false;
                off[k] = short(r < n ? o : 0);
            }
        }
    });
    if (fits) off16.upload(off, s);
    else off16.release();
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
    // right-hand-side rows in the internal numbering (matrix slots already are: S.slot)
    parallel_for(nc, [&](long long c) {
        visit_cell(int(c), [&](long long k, int, int) { atomic_inc(&scount[k]); },
                   [&](int i, int, int) { atomic_inc(&rcount[S.dof(i)]); });
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
            [&](int i, int e, int) {
                const int r = S.dof(i);
                h_rhs_ent[h_rhs_ptr[r] + atomic_inc(&rcount[r])] = e;
            });
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
