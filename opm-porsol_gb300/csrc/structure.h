// structure.h -- host-side topology of the hybrid system: face DOFs, periodic partners,
// sparsity of S, SELL layout and the assembly recipe.  Built once per grid/BC topology.
#pragma once

#include "porsol_internal.h"

namespace porsol {

// Per-half-face boundary kind used by the assembly kernels (FaceType of
// IncompFlowSolverHybrid.hpp:378 plus the periodic orientation needed by addCellContrib).
enum HfKind : int {
    HK_INTERNAL = 0,
    HK_DIRICHLET = 1,
    HK_NEUMANN = 2,
    HK_PERIODIC_HI = 3,  // periodic face whose partner dof is larger: column kept
    HK_PERIODIC_LO = 4,  // periodic face whose partner dof is smaller: column moved to partner
};

struct HostGrid {
    int nc = 0, nhf = 0;
    std::vector<int> facepos, nb, bid;
    std::vector<double> area, fcent, fnormal, cvol, ccent;
    // geometry = false keeps only the topology (facepos, nb, bid); area .. ccent stay empty
    void copy_from(const porsol_grid* g, bool geometry = true);
    int nf(int c) const { return facepos[c + 1] - facepos[c]; }
    bool boundary(int hf) const { return nb[hf] < 0; }
};

struct Structure {
    HostGrid g;
    int N = 0, num_internal = 0, max_ncf = 0;
    std::vector<int> cf;                    // half-face -> dof (cellFaces_)
    std::vector<int> hf_cell;               // half-face -> cell
    std::vector<int> hf_partner_bid;        // getPeriodicPartner(boundaryId) per half-face
    std::unordered_map<int, std::pair<int, int>> bdry_id_map;   // bid -> (cell, local face)
    std::vector<int> init_periodic;         // 1 where the face was periodic at init
    std::vector<int> ppartner;              // dof -> partner dof (-1); empty if no periodic face
    std::vector<int> partner_hf;            // half-face -> partner half-face for periodic faces (-1)
    HVec<int> rowptr, colind;               // CSR of S, sorted columns
    HVec<int> csr2sell;                     // SELL slot of each CSR entry (SELL offsets are 32-bit)
    SellPattern pat;
    std::vector<int> pairs;                 // post-process pairs (hf_first, hf_second) flattened
    std::vector<int> boundary_hf;           // all boundary half-faces in order

    // Internal numbering of the face unknowns.  Everything above (cf, rowptr/colind, ppartner,
    // the recipe's semantics) is in the reference's numbering; the device system (pat, the
    // assembly targets, every N-vector) uses the internal one, dof_perm[reference dof] = internal
    // dof (empty: the two coincide).  The internal numbering visits the cells in an order of small
    // bandwidth and numbers each cell's faces when the cell is first reached, so the couplings of a
    // row lie close to it (|i - j| <= bandwidth) and rows next to each other gather neighbouring
    // entries.
    std::vector<int> dof_perm, dof_iperm;   // reference -> internal, internal -> reference
    std::vector<int> cf_int;                // half-face -> internal dof
    int bandwidth = 0;                      // max |i - j| over the couplings, internal numbering
    int bandwidth_ref = 0;                  // the same in the reference numbering
    // The system in the reference numbering, for the ILU0 path (its factorisation depends on the
    // ordering): SELL pattern and, per slot of it, the internal slot (-1 for padding); built on
    // first use.
    SellPattern pat_ref;
    HVec<int> ref_slot_src;
    bool ref_pattern_built = false;

    void build(const porsol_grid* grid, const int* flow_type, const int* partner_bid);
    int partner_dof(int hf) const;
    int partner_cell(int hf) const;
    long long slot(int i, int j) const;     // SELL slot of (i, j) (reference dofs); throws if absent
    int dof(int i) const { return dof_perm.empty() ? i : dof_perm[i]; }   // reference -> internal
    bool renumbered() const { return !dof_perm.empty(); }
    void build_ref_pattern();               // pat_ref and ref_slot_src (renumbered systems only)
};

// The assembly recipe: which local Schur entries are summed into which SELL slot and
// which per-half-face right-hand-side pieces into which row.  Depends on the BC types
// (not their values); rebuilt whenever they change.
struct Recipe {
    bool valid = false;
    bool do_reg = true;
    std::vector<int> kind;               // HfKind per half-face
    HVec<int> h_slot_ptr, h_slot_ent, h_rhs_ptr, h_rhs_ent;
    DBuf<int> kind_d, slot_ptr, slot_ent, rhs_ptr, rhs_ent;
    void build(const Structure& S, const int* flow_type, int max_nf_packed);
};

// Packed index of symmetric entry (r, s) in an upper-triangle packing.
inline int packed_index(int r, int s)
{
    if (r > s) std::swap(r, s);
    return s * (s + 1) / 2 + r;
}

}  // namespace porsol
