// structure_test.cpp -- the host-side structure and recipe build (structure.cpp) on the CPU alone:
// reads a flattened grid topology and flow-BC types, builds the face numbering, the sparsity of S,
// the SELL layout and the assembly recipe, checks the recipe's invariants and writes the
// numbering and sparsity for comparison with the oracle.
//
// Input (binary, native endian): int64 nc, nhf; int32 facepos[nc+1], neighbour[nhf], bid[nhf],
// flow_type[nhf], partner_bid[nhf]; optionally float64 cell_centroid[3 nc] (else all zero).
// Output: int32 N, num_internal, then cf[nhf], rowptr[N+1], colind[rowptr[N]], ppartner[N]
// (all -1 without periodic faces), then the internal numbering: renumbered (0/1), bandwidth,
// bandwidth in the reference numbering, dof_perm[N] (identity when not renumbered).
//
// Checks of the internal numbering: dof_perm is a permutation; every coupling (i, j) of the
// reference CSR sits in the internal SELL layout at row dof_perm[i], column dof_perm[j]; rows
// keep sorted columns; cf_int = dof_perm[cf]; the recipe's right-hand-side rows are internal.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "structure.h"

using namespace porsol;

static void fail(const char* msg)
{
    std::fprintf(stderr, "structure_test: %s\n", msg);
    std::exit(1);
}

int main(int argc, char** argv)
{
    if (argc != 3) fail("usage: structure_test in.bin out.bin");
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) fail("cannot open input");
    long long hdr[2];
    if (std::fread(hdr, 8, 2, f) != 2) fail("short header");
    const int nc = int(hdr[0]), nhf = int(hdr[1]);
    std::vector<int> fp(nc + 1), nb(nhf), bid(nhf), bct(nhf), pb(nhf);
    if (std::fread(fp.data(), 4, nc + 1, f) != size_t(nc + 1) || std::fread(nb.data(), 4, nhf, f) != size_t(nhf) ||
        std::fread(bid.data(), 4, nhf, f) != size_t(nhf) || std::fread(bct.data(), 4, nhf, f) != size_t(nhf) ||
        std::fread(pb.data(), 4, nhf, f) != size_t(nhf))
        fail("short input");
    // geometry is not read by the build, except cell centroids for the internal cell order
    std::vector<double> d1(nhf, 1.0), d3(3 * size_t(nhf), 0.0), v(nc, 1.0), c3(3 * size_t(nc), 0.0);
    if (std::fread(c3.data(), 8, 3 * size_t(nc), f) != 3 * size_t(nc)) std::fill(c3.begin(), c3.end(), 0.0);
    std::fclose(f);
    porsol_grid g{nc, fp.data(), nb.data(), bid.data(), d1.data(), d3.data(), d3.data(), v.data(), c3.data()};
    Structure S;
    S.build(&g, bct.data(), pb.data());
    Recipe R;
    R.build(S, bct.data(), S.max_ncf <= 6 ? 21 : 78);
    // recipe invariants: every stored entry of S receives at least one contribution unless it is
    // slice padding; the entries of a slot come cell by cell in increasing cell order
    const long long nent = S.pat.nent;
    std::vector<char> real(nent, 0);
    for (size_t k = 0; k < S.csr2sell.size(); ++k) real[S.csr2sell[k]] = 1;
    for (long long k = 0; k < nent; ++k) {
        const int b = R.h_slot_ptr[k], e = R.h_slot_ptr[k + 1];
        if (e > b && !real[k]) fail("recipe writes a padding slot");
        int last = -1;
        for (int q = b; q < e; ++q) {
            const int x = R.h_slot_ent[q];
            const int cell = (x < 0 ? ~x : x) % nc;
            if (cell < last) fail("slot entries out of cell order");
            last = cell;
        }
    }
    for (int i = 0; i < S.N; ++i) {
        int last = -1;
        for (int q = R.h_rhs_ptr[i]; q < R.h_rhs_ptr[i + 1]; ++q) {
            const int cell = S.hf_cell[R.h_rhs_ent[q] >> 2];
            if (cell < last) fail("rhs entries out of cell order");
            last = cell;
        }
    }
    // internal numbering
    std::vector<int> perm(S.N);
    for (int i = 0; i < S.N; ++i) perm[i] = S.dof(i);
    {
        std::vector<char> seen(S.N, 0);
        for (int i = 0; i < S.N; ++i) {
            if (perm[i] < 0 || perm[i] >= S.N || seen[perm[i]]) fail("dof_perm is not a permutation");
            seen[perm[i]] = 1;
        }
        int bw = 0;
        for (int i = 0; i < S.N; ++i)
            for (int k = S.rowptr[i]; k < S.rowptr[i + 1]; ++k) {
                const long long slot = S.csr2sell[k];
                const int r = perm[i], sl = r / SELL_C, lane = r % SELL_C;
                const long long off = slot - S.pat.h_slice_ptr[sl];
                if (off < 0 || off % SELL_C != lane || off / SELL_C >= S.pat.h_rowlen[r])
                    fail("coupling not in its internal row");
                if (S.pat.h_col[slot] != perm[S.colind[k]]) fail("internal column differs");
                bw = std::max(bw, std::abs(perm[S.colind[k]] - r));
            }
        if (bw != S.bandwidth) fail("bandwidth differs");
        for (int r = 0; r < S.N; ++r) {
            const int sl = r / SELL_C, lane = r % SELL_C;
            for (int t = 1; t < S.pat.h_rowlen[r]; ++t)
                if (S.pat.h_col[S.pat.h_slice_ptr[sl] + (long long)t * SELL_C + lane] <=
                    S.pat.h_col[S.pat.h_slice_ptr[sl] + (long long)(t - 1) * SELL_C + lane])
                    fail("internal row columns not sorted");
        }
        if (S.renumbered())
            for (int hf = 0; hf < nhf; ++hf)
                if (S.cf_int[hf] != perm[S.cf[hf]]) fail("cf_int differs");
        // every half-face's rhs piece lands in its face's internal row
        for (int r = 0; r < S.N; ++r)
            for (int q = R.h_rhs_ptr[r]; q < R.h_rhs_ptr[r + 1]; ++q) {
                const int hf = R.h_rhs_ent[q] >> 2, kind = R.h_rhs_ent[q] & 3;
                if (kind == 0 && perm[S.cf[hf]] != r && R.kind[hf] != HK_PERIODIC_LO) fail("rhs piece in another row");
            }
        if (S.renumbered() && S.bandwidth >= S.bandwidth_ref) fail("renumbered without a smaller bandwidth");
    }
    FILE* o = std::fopen(argv[2], "wb");
    if (!o) fail("cannot open output");
    const int head[2] = {S.N, S.num_internal};
    std::vector<int> pp(S.N, -1);
    if (!S.ppartner.empty()) pp.assign(S.ppartner.begin(), S.ppartner.end());
    std::fwrite(head, 4, 2, o);
    std::fwrite(S.cf.data(), 4, nhf, o);
    std::fwrite(S.rowptr.data(), 4, S.N + 1, o);
    std::fwrite(S.colind.data(), 4, S.colind.size(), o);
    std::fwrite(pp.data(), 4, S.N, o);
    const int tail[3] = {S.renumbered() ? 1 : 0, S.bandwidth, S.bandwidth_ref};
    std::fwrite(tail, 4, 3, o);
    std::fwrite(perm.data(), 4, S.N, o);
    std::fclose(o);
    std::printf("OK N=%d nnz=%zu slots=%lld entries=%d\n", S.N, S.colind.size(), nent, R.h_slot_ptr[nent]);
    return 0;
}
