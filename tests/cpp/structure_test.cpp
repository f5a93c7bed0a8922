// structure_test.cpp -- the host-side structure and recipe build (structure.cpp) on the CPU alone:
// reads a flattened grid topology and flow-BC types, builds the face numbering, the sparsity of S,
// the SELL layout and the assembly recipe, checks the recipe's invariants and writes the
// numbering and sparsity for comparison with the oracle.
//
// Input (binary, native endian): int64 nc, nhf; int32 facepos[nc+1], neighbour[nhf], bid[nhf],
// flow_type[nhf], partner_bid[nhf].  Output: int32 N, num_internal, then cf[nhf],
// rowptr[N+1], colind[rowptr[N]], ppartner[N] (all -1 without periodic faces).
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
    std::fclose(f);
    // geometry is not read by the build; the grid needs non-null arrays
    std::vector<double> d1(nhf, 1.0), d3(3 * size_t(nhf), 0.0), v(nc, 1.0), c3(3 * size_t(nc), 0.0);
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
    std::fclose(o);
    std::printf("OK N=%d nnz=%zu slots=%lld entries=%d\n", S.N, S.colind.size(), nent, R.h_slot_ptr[nent]);
    return 0;
}
