// capi.cu -- the pressure-solver handle and the extern "C" entry points of porsol_gpu.h.
//
// Order of work in porsol_solve (IncompFlowSolverHybrid::solve, IncompFlowSolverHybrid.hpp:658-703):
//   1. assembleDynamic: k_assemble_cells (per-cell Schur complements and rhs pieces), then
//      the recipe gathers write the global matrix (SELL) and right-hand side;
//   2. pure-Neumann regularisation S[0][0] *= 2 (:1398-1400, :1493-1495);
//   3. linear solve: ILU0-CG (type 0) or AMG-CG (types 1-3), FP64, or mixed (FP32 AMG and CG recurrences, FP64 solution and residual replacements);
//   4. computePressureAndFluxes: k_recover.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <sstream>

#include "solver.h"

using namespace porsol;

// ---------------------------------------------------------------- profiler
namespace porsol {

std::atomic<long long> g_launches{0};

namespace {
thread_local int t_chain_paused = 0;
int chain_env()
{
    static const int mode = [] {
        const char* e = std::getenv("PORSOL_PDL");
        return e && e[0] >= '0' && e[0] <= '2' ? e[0] - '0' : 2;
    }();
    return mode;
}
}  // namespace

bool chain_enabled(long long blocks)
{
    const int m = chain_env();
    return t_chain_paused == 0 && (m == 1 || (m == 2 && blocks < 304));
}

ChainPause::ChainPause(bool on) : on_(on)
{
    if (on_) ++t_chain_paused;
}

ChainPause::~ChainPause()
{
    if (on_) --t_chain_paused;
}

cudaEvent_t Profiler::get()
{
    if (!pool.empty()) {
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    PORSOL_CUDA(cudaEventCreate(&e));
    return e;
}

void Profiler::begin(cudaStream_t s, int, double, cudaEvent_t* out_a)
{
    *out_a = get();
    PORSOL_CUDA(cudaEventRecord(*out_a, s));
}

void Profiler::end(cudaStream_t s, int k, double b, cudaEvent_t a)
{
    cudaEvent_t e = get();
    PORSOL_CUDA(cudaEventRecord(e, s));
    pending.push_back({a, e, k, b});
    if (pending.size() > 4096) collect();
}

void Profiler::collect()
{
    for (auto& p : pending) {
        PORSOL_CUDA(cudaEventSynchronize(p.b));
        float ms_ = 0.f;
        PORSOL_CUDA(cudaEventElapsedTime(&ms_, p.a, p.b));
        launches[p.k] += 1;
        ms[p.k] += ms_;
        bytes[p.k] += p.bytes;
        pool.push_back(p.a);
        pool.push_back(p.b);
    }
    pending.clear();
}

void Profiler::reset()
{
    collect();
    for (int k = 0; k < PK_COUNT; ++k) {
        launches[k] = 0;
        ms[k] = 0;
        bytes[k] = 0;
    }
}

Profiler::~Profiler()
{
    for (auto& p : pending) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    for (auto& e : pool) cudaEventDestroy(e);
}

}  // namespace porsol

// ---------------------------------------------------------------- solver
void porsol_solver::require_structure() const
{
    PORSOL_REQUIRE(structure_valid, PORSOL_ERR_STATE, "initSystemStructure must be called first");
}

void porsol_solver::check_status(const char* where)
{
    int st = 0;
    PORSOL_CUDA(cudaMemcpyAsync(&st, status.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
    PORSOL_CUDA(cudaStreamSynchronize(stream));
    if (st) {
        PORSOL_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), stream));
        std::ostringstream os;
        os << where << ": ";
        if (st & ST_NONFINITE) os << "non-finite value or non-positive pivot/mobility";
        else if (st & ST_BAD_INDEX) os << "index check failed (too many faces per cell?)";
        else os << "device status " << st;
        throw Error((st & ST_NONFINITE) ? PORSOL_ERR_NONFINITE : PORSOL_ERR_BAD_ARG, os.str());
    }
}

// True when grid topology, initial FlowBC periodicity and partner ids equal those the current
// structure was built from: the face numbering, sparsity and assembly recipe are then reused.
bool porsol_solver::same_topology(const porsol_grid* grid, const int* flow_type, const int* partner_bid) const
{
    if (!structure_valid || !grid || grid->num_cells != S.g.nc || !grid->cell_facepos) return false;
    const HostGrid& g = S.g;
    if (!std::equal(g.facepos.begin(), g.facepos.end(), grid->cell_facepos)) return false;
    const int nhf = g.nhf;
    if (!grid->hf_neighbour || !grid->hf_bid) return false;
    if (!std::equal(g.nb.begin(), g.nb.end(), grid->hf_neighbour)) return false;
    if (!std::equal(g.bid.begin(), g.bid.end(), grid->hf_bid)) return false;
    for (int hf = 0; hf < nhf; ++hf) {
        const int per = (flow_type && g.nb[hf] < 0 && flow_type[hf] == PORSOL_BC_PERIODIC) ? 1 : 0;
        if (per != S.init_periodic[hf]) return false;
        if ((partner_bid ? partner_bid[hf] : 0) != S.hf_partner_bid[hf]) return false;
    }
    return true;
}

// Geometry goes to the device straight from the caller's arrays (the host keeps topology only).
void porsol_solver::upload_geometry(const porsol_grid* grid)
{
    const size_t nc = size_t(grid->num_cells), nhf = size_t(grid->cell_facepos[nc]);
    cudaStream_t s = stream;
    area.upload(grid->hf_area, nhf, s);
    fcent.upload(grid->hf_centroid, 3 * nhf, s);
    fnormal.upload(grid->hf_normal, 3 * nhf, s);
    cvol.upload(grid->cell_volume, nc, s);
    ccent.upload(grid->cell_centroid, 3 * nc, s);
    PORSOL_CUDA(cudaStreamSynchronize(s));   // pageable sources: the copies complete before return
}

void porsol_solver::init_structure(const porsol_grid* grid, const int* flow_type, const int* partner_bid)
{
    NvtxRange range("porsol initSystemStructure");
    // the reference's init skips an empty grid (IncompFlowSolverHybrid.hpp:483-486); a solver
    // without cells has nothing to do, so the C ABI reports it instead of building empty arrays
    PORSOL_REQUIRE(grid && grid->num_cells > 0, PORSOL_ERR_BAD_ARG, "grid: no cells");
    amg64.set_profiler(&prof);
    amg32.set_profiler(&prof);
    if (same_topology(grid, flow_type, partner_bid)) {
        // geometry may differ: upload it; everything derived from topology is kept
        PORSOL_REQUIRE(grid->hf_area && grid->hf_centroid && grid->hf_normal && grid->cell_volume &&
                           grid->cell_centroid,
                       PORSOL_ERR_BAD_ARG, "grid: null array");
        upload_geometry(grid);
        ip_valid = solved = false;
        amg_ready = false;
        return;
    }
    structure_valid = ip_valid = solved = false;
    R.valid = false;
    amg_ready = false;
    ilu_levels = false;
    S = Structure();
    S.build(grid, flow_type, partner_bid);
    PORSOL_REQUIRE(S.max_ncf <= 12, PORSOL_ERR_BAD_ARG, "cells with more than 12 faces are not supported");
    maxnf = S.max_ncf <= 6 ? 6 : 12;
    npk = maxnf * (maxnf + 1) / 2;
    const HostGrid& g = S.g;
    cudaStream_t s = stream;
    facepos.upload(g.facepos, s);
    cf.upload(S.renumbered() ? S.cf_int : S.cf, s);   // the device system's (internal) numbering
    pairs.upload(S.pairs, s);
    if (S.renumbered()) dof_perm_d.upload(S.dof_perm, s);
    upload_geometry(grid);
    S.pat.upload(s);
    status.alloc(1);
    status.zero(s);
    redbits.alloc(4);
    const size_t nc = g.nc, nhf = g.nhf, N = S.N;
    W.alloc(npk * nc);
    W.zero(s);
    gflux.alloc(nhf);
    sloc.alloc(npk * nc);
    F.alloc(nhf);
    L.alloc(nc);
    this->g.alloc(nc);
    rrow.alloc(nhf);
    pb.alloc(nhf);
    totmob.alloc(nc);
    mobdens.alloc(nc);
    rhs.alloc(N);
    x.alloc(N);
    val.alloc(S.pat.nent);
    pressure.alloc(nc);
    outflux.alloc(nhf);
    pressure.zero(s);
    outflux.zero(s);
    x.zero(s);
    PORSOL_CUDA(cudaStreamSynchronize(s));
    structure_valid = true;
}

void porsol_solver::compute_inner_products(const double* perm_h, const double* grav)
{
    NvtxRange range("porsol computeInnerProducts");
    require_structure();
    PORSOL_REQUIRE(perm_h, PORSOL_ERR_BAD_ARG, "permeability array is null");
    const double g0[3] = {grav ? grav[0] : 0.0, grav ? grav[1] : 0.0, grav ? grav[2] : 0.0};
    gravity_zero = (g0[0] == 0.0 && g0[1] == 0.0 && g0[2] == 0.0);
    for (int d = 0; d < 3; ++d) grav_[d] = g0[d];
    perm.upload(perm_h, 9 * size_t(S.g.nc), stream);
    launch_static_ip(maxnf, stream, S.g.nc, facepos.p, area.p, fcent.p, fnormal.p, cvol.p, ccent.p, perm.p, g0, W.p,
                     gflux.p, status.p);
    check_status("computeInnerProducts");
    ip_valid = true;
}

void porsol_solver::ensure_recipe(const int* bct_host, const int* bct_dev)
{
    // Boundary FlowBC types of this solve; the recipe depends on them only.
    const std::vector<int>& bh = S.boundary_hf;
    std::vector<int> types(bh.size());
    if (bct_host) {
        for (size_t q = 0; q < bh.size(); ++q) types[q] = bct_host[bh[q]];
    } else {
        // Compare on the device first; the full array crosses to the host only on a change.
        if (R.valid) {
            PORSOL_CUDA(cudaMemsetAsync(redbits.p + 3, 0, sizeof(int), stream));
            launch_compare_types(stream, int(bh.size()), boundary_hf_d.p, bct_dev, recipe_types_d.p,
                                 (int*)(redbits.p + 3));
            int changed = 0;
            PORSOL_CUDA(cudaMemcpyAsync(&changed, redbits.p + 3, sizeof(int), cudaMemcpyDeviceToHost, stream));
            PORSOL_CUDA(cudaStreamSynchronize(stream));
            if (!changed) return;
        }
        std::vector<int> all(S.g.nhf);
        PORSOL_CUDA(cudaMemcpyAsync(all.data(), bct_dev, sizeof(int) * all.size(), cudaMemcpyDeviceToHost, stream));
        PORSOL_CUDA(cudaStreamSynchronize(stream));
        for (size_t q = 0; q < bh.size(); ++q) types[q] = all[bh[q]];
    }
    if (R.valid && types == recipe_types) return;
    std::vector<int> full(S.g.nhf, -1);
    for (size_t q = 0; q < bh.size(); ++q) full[bh[q]] = types[q];
    R.build(S, full.data(), npk);
    R.kind_d.upload(R.kind, stream);
    R.slot_ptr.upload(R.h_slot_ptr, stream);
    R.slot_ent.upload(R.h_slot_ent, stream);
    R.rhs_ptr.upload(R.h_rhs_ptr, stream);
    R.rhs_ent.upload(R.h_rhs_ent, stream);
    recipe_types_d.upload(types, stream);
    boundary_hf_d.upload(bh, stream);
    PORSOL_CUDA(cudaStreamSynchronize(stream));
    recipe_types = types;
    amg_ready = false;   // a different matrix structure of values
}

namespace {
double now_ms()
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
}  // namespace

// Algorithmic bytes of the linear solve just finished (values + columns of each stored entry read
// once per matrix pass, each vector read or written once per kernel; s_v / s_x the value and
// vector widths):
//   FP64 AMG-CG:  per iteration SpMV + p.q  Z(8+c) + 16N, update x, r  48N, z.r  16N,
//                 direction 24N, V-cycle; start: residual Z (8+c) + 24N, V-cycle, z.r, direction
//   mixed:        per iteration FP32 SpMV + p.q  Z(4+c) + 8N, update (x FP64)  32N, z.r  8N,
//                 direction 12N, FP32 V-cycle; per FP64 residual replacement Z (8+c) + 24N and the
//                 rescale 20N; start: FP64 residual, rescale, V-cycle, z.r, direction
//   ILU0-CG:      per iteration 2 Z (8+4) + 8 (N+1) + 19 N 8 (SpMV, both triangular sweeps, two
//                 dots, three vector updates)
// with c = 2 bytes of column index where the system's 16-bit offsets are in use, else 4.
void porsol_solver::count_krylov_bytes(const porsol_solve_opts& o, int iterations, int replacements)
{
    const double Z = double(S.pat.nent), N = double(S.N), it = iterations;
    const double c = S.pat.has_off16() ? 2.0 : 4.0;
    vcycle_level_bytes.clear();
    if (o.linsolver_type == 0) {
        bytes_krylov = (it + 1) * (2.0 * Z * 12.0 + 8.0 * (N + 1) + 19.0 * N * 8.0);
        return;
    }
    if (o.precision == PORSOL_FP64) {
        const double vc = amg64.apply_bytes(&vcycle_level_bytes);
        bytes_krylov = it * (Z * (8.0 + c) + 16.0 * N + 48.0 * N + 16.0 * N + 24.0 * N + vc) +
                       (Z * (8.0 + c) + 24.0 * N + vc + 16.0 * N + 16.0 * N);
    } else {
        const double vc = amg32.apply_bytes(&vcycle_level_bytes);
        bytes_krylov = it * (Z * (4.0 + c) + 8.0 * N + 32.0 * N + 8.0 * N + 12.0 * N + vc) +
                       replacements * (Z * (8.0 + c) + 24.0 * N + 20.0 * N) +
                       (Z * (8.0 + c) + 24.0 * N + 12.0 * N + vc + 8.0 * N + 8.0 * N);
    }
}

void porsol_solver::linear_solve(const porsol_solve_opts& o, porsol_solve_stats& st)
{
    NvtxRange range("porsol linear solve (setup + CG)");
    const double t_begin = now_ms();
    const int n = S.N;
    const int maxit = o.linsolver_maxit > 0 ? o.linsolver_maxit : n;
    const SellPattern& P = S.pat;
    st.amg_levels = 0;
    st.outer_iterations = 1;
    auto fail = [&](int iters, double red) {
        std::ostringstream os;
        os << "Linear solver failed to converge in " << iters << " iterations.\n"
           << "Residual reduction achieved is " << red << '\n';
        throw Error(PORSOL_ERR_NOT_CONVERGED, os.str());
    };
    if (batch.nblk > 0) {
        batched_solve(o, st, maxit);
        return;
    }
    if (o.linsolver_type == 0 && S.renumbered()) {
        ilu_solve_reference_order(o, st, maxit);
        return;
    }
    if (o.linsolver_type == 0) {
        // solveLinearSystem (:1387-1420): ILU0(S, 1.0), CG, zero initial guess
        if (!ilu_levels) {
            ilu.build_levels(P, stream);
            ilu_levels = true;
        }
        ilu.factor(stream, P, val.p);
        st.ms_precond_setup = now_ms() - t_begin;
        x.zero(stream);
        CgResult r = cg64.solve(stream, P, val.p, ilu, rhs.p, x.p, o.residual_tolerance, maxit, &prof, PK_SPMV64);
        st.iterations = r.iterations;
        st.reduction = r.reduction;
        count_krylov_bytes(o, r.iterations, 0);
        if (r.breakdown) throw Error(PORSOL_ERR_NONFINITE, "CG breakdown (non-positive curvature)");
        if (!r.converged) fail(r.iterations, r.reduction);
        return;
    }
    // solveLinearSystemAMG (:1481-1541): hierarchy rebuilt unless same_matrix, initial
    // guess with Dirichlet rows pre-solved, CG.
    AmgOpts ao;
    ao.smooth_steps = std::max(1, o.smooth_steps);
    ao.prolong = o.prolongate_factor;
    // linsolver_type 2 (solveLinearSystemKAMG, :1609-1666): the Krylov-accelerated cycle (dune's KAMG
    // is not available; this is the K-cycle on the first coarse level, the bandwidth-bound one: two
    // flexible-CG steps there per cycle, the deeper levels visited twice); types 1 and 3 the V-cycle
    ao.kcycle_levels = o.linsolver_type == 2 ? 1 : 0;
    dirichlet_guess(stream, P, val.p, rhs.p, x.p);
    if (o.precision == PORSOL_FP64) {
        if (!((o.same_matrix || reuse_amg) && amg_ready && amg_precision == PORSOL_FP64 &&
              amg_kcycle == ao.kcycle_levels)) {
            amg64.set_row_blocks(nullptr);
            amg64.setup(stream, P, val.p, ao);
            amg_ready = true;
            amg_precision = PORSOL_FP64;
            amg_kcycle = ao.kcycle_levels;
        }
        PORSOL_CUDA(cudaStreamSynchronize(stream));
        st.ms_precond_setup = now_ms() - t_begin;
        st.amg_levels = amg64.levels();
        CgResult r = cg64.solve(stream, P, val.p, amg64, rhs.p, x.p, o.residual_tolerance, maxit, &prof, PK_SPMV64);
        st.iterations = r.iterations;
        st.reduction = r.reduction;
        count_krylov_bytes(o, r.iterations, 0);
        if (r.breakdown) throw Error(PORSOL_ERR_NONFINITE, "CG breakdown (non-positive curvature)");
        if (!r.converged) fail(r.iterations, r.reduction);
        return;
    }
    // Mixed precision: FP32 matrix copy, FP32 AMG hierarchy and one FP32 CG recurrence with the
    // solution in FP64 and reliable updates (the iterated residual replaced by the FP64 residual
    // b - A x whenever it has dropped by inner_tolerance); see ReliableCg.
    if (!((o.same_matrix || reuse_amg) && amg_ready && amg_precision == PORSOL_MIXED &&
          amg_kcycle == ao.kcycle_levels)) {
        // the throughput path coarsens its small coarse levels by three pairing rounds instead of
        // two (on the 1M-cell system: 9 levels instead of 10, same CG iteration count, 2 % faster);
        // the FP64 drop-in keeps the two-round hierarchy
        AmgOpts ao32 = ao;
        ao32.round3_below = 30000;
        amg32.set_row_blocks(nullptr);
        amg32.setup(stream, P, val32.p, ao32);
        amg_ready = true;
        amg_precision = PORSOL_MIXED;
        amg_kcycle = ao.kcycle_levels;
    }
    PORSOL_CUDA(cudaStreamSynchronize(stream));
    st.ms_precond_setup = now_ms() - t_begin;
    st.amg_levels = amg32.levels();
    const double inner_tol = o.inner_tolerance > 0 ? o.inner_tolerance : 3e-3;
    CgResult r = rcg.solve(stream, P, val.p, val32.p, amg32, rhs.p, x.p, o.residual_tolerance, maxit, inner_tol, &prof);
    if (const int ast = amg32.solve_status(stream)) {
        amg_ready = false;   // the next solve sets the hierarchy (and its status) up again
        throw Error((ast & ST_TIMEOUT) ? PORSOL_ERR_TIMEOUT : PORSOL_ERR_BAD_ARG,
                    "AMG smoother: bulk copy of the matrix slices failed (wait gave up or staging area too small)");
    }
    st.iterations = r.iterations;
    st.outer_iterations = rcg.replacements();
    st.reduction = r.reduction;
    count_krylov_bytes(o, r.iterations, rcg.replacements());
    if (r.breakdown) throw Error(PORSOL_ERR_NONFINITE, "CG breakdown (non-positive curvature or non-finite residual)");
    if (!r.converged) fail(r.iterations, r.reduction);
}

// ILU0-CG (solveLinearSystem, :1387-1420) of a structure whose device numbering differs from the
// reference's: ILU(0) depends on the order of the unknowns, so the factorisation and the CG run on
// the system gathered into the reference numbering (same factors, iterates and iteration counts as
// the reference), and the solution is scattered back.
void porsol_solver::ilu_solve_reference_order(const porsol_solve_opts& o, porsol_solve_stats& st, int maxit)
{
    const double t_begin = now_ms();
    const int n = S.N;
    if (!S.ref_pattern_built) {
        S.build_ref_pattern();
        S.pat_ref.upload(stream);
        ref_slot_src_d.upload(S.ref_slot_src, stream);
        ilu_levels = false;
    }
    const SellPattern& P = S.pat_ref;
    val_ref.alloc(size_t(P.nent));
    rhs_ref.alloc(n);
    x_ref.alloc(n);
    launch_gather_values(stream, P.nent, ref_slot_src_d.p, val.p, val_ref.p);
    launch_permute(stream, n, dof_perm_d.p, rhs.p, rhs_ref.p, true);
    if (!ilu_levels) {
        ilu.build_levels(P, stream);
        ilu_levels = true;
    }
    ilu.factor(stream, P, val_ref.p);
    st.ms_precond_setup = now_ms() - t_begin;
    x_ref.zero(stream);
    CgResult r = cg64.solve(stream, P, val_ref.p, ilu, rhs_ref.p, x_ref.p, o.residual_tolerance, maxit, &prof,
                            PK_SPMV64);
    launch_permute(stream, n, dof_perm_d.p, x_ref.p, x.p, false);
    st.iterations = r.iterations;
    st.reduction = r.reduction;
    count_krylov_bytes(o, r.iterations, 0);
    if (r.breakdown) throw Error(PORSOL_ERR_NONFINITE, "CG breakdown (non-positive curvature)");
    if (!r.converged) {
        std::ostringstream os;
        os << "Linear solver failed to converge in " << r.iterations << " iterations.\n"
           << "Residual reduction achieved is " << r.reduction << '\n';
        throw Error(PORSOL_ERR_NOT_CONVERGED, os.str());
    }
}

// Block-diagonal systems (batched upscaling): one CG per block (BatchedPcg), each block with
// the stopping test ||r_g|| < tol ||r_g^0|| that its own solve would use.  FP64: ILU0 or AMG
// preconditioner; mixed: FP64 per-block residuals around FP32 batched CG + FP32 AMG.
void porsol_solver::batched_solve(const porsol_solve_opts& o, porsol_solve_stats& st, int maxit)
{
    const double t_begin = now_ms();
    const int n = S.N, nb = batch.nblk;
    const SellPattern& P = S.pat;
    st.amg_levels = 0;
    st.outer_iterations = 1;
    auto fail = [&](int iters, double red) {
        std::ostringstream os;
        os << "Linear solver failed to converge in " << iters << " iterations.\n"
           << "Residual reduction achieved is " << red << '\n';
        throw Error(PORSOL_ERR_NOT_CONVERGED, os.str());
    };
    std::vector<double> h(nb);
    auto upload = [&](DBuf<double>& d, const std::vector<double>& v) { d.upload(v, stream); };
    AmgOpts ao;
    ao.smooth_steps = std::max(1, o.smooth_steps);
    ao.prolong = o.prolongate_factor;
    ao.autotune = true;   // the sub-grid union's level shapes are unlike a single grid's
    // FP32 smoother values: with the FP16 copy the full-tensor, rotated sub-grids needed 491 CG
    // iterations for 512 sub-grids x 3 solves against 282 (and 239 in FP64)
    ao.half_smoother = false;
    const bool mixed = o.precision == PORSOL_MIXED && o.linsolver_type != 0;
    if (!mixed) {
        Precond<double>* M = nullptr;
        if (o.linsolver_type == 0) {
            if (!ilu_levels) {
                ilu.build_levels(P, stream);
                ilu_levels = true;
            }
            ilu.factor(stream, P, val.p);
            x.zero(stream);
            M = &ilu;
        } else {
            dirichlet_guess(stream, P, val.p, rhs.p, x.p);
            if (!((o.same_matrix || reuse_amg) && amg_ready && amg_precision == PORSOL_FP64)) {
                amg64.set_row_blocks(batch.blk.p);
                amg64.setup(stream, P, val.p, ao);
                amg_ready = true;
                amg_precision = PORSOL_FP64;
                amg_kcycle = 0;
            }
            st.amg_levels = amg64.levels();
            M = &amg64;
        }
        PORSOL_CUDA(cudaStreamSynchronize(stream));
        st.ms_precond_setup = now_ms() - t_begin;
        std::fill(h.begin(), h.end(), o.residual_tolerance);
        upload(btol, h);
        CgResult r = bcg64.solve(stream, P, val.p, *M, batch, rhs.p, x.p, btol.p, maxit);
        st.iterations = r.iterations;
        st.reduction = r.reduction;
        if (r.breakdown) throw Error(PORSOL_ERR_NONFINITE, "CG breakdown (non-positive curvature)");
        if (!r.converged) fail(r.iterations, r.reduction);
        return;
    }
    dirichlet_guess(stream, P, val.p, rhs.p, x.p);
    if (!((o.same_matrix || reuse_amg) && amg_ready && amg_precision == PORSOL_MIXED)) {
        amg32.set_row_blocks(batch.blk.p);
        amg32.setup(stream, P, val32.p, ao);
        amg_ready = true;
        amg_precision = PORSOL_MIXED;
        amg_kcycle = 0;
    }
    PORSOL_CUDA(cudaStreamSynchronize(stream));
    st.ms_precond_setup = now_ms() - t_begin;
    st.amg_levels = amg32.levels();
    // FP64 batched CG around the FP32 AMG hierarchy, per-block scaled into FP32 range
    ir_r.alloc(n);
    bnorm.alloc(nb);
    residual<double, double>(stream, P, val.p, x.p, rhs.p, ir_r.p);
    batch_norms<double>(stream, batch, ir_r.p, bnorm.p);
    std::vector<double> r0(nb), sc(nb);
    bnorm.download(r0.data(), nb, stream);
    PORSOL_CUDA(cudaStreamSynchronize(stream));
    for (int g = 0; g < nb; ++g) {
        const bool ok = r0[g] > 1e-300 && std::isfinite(r0[g]);
        sc[g] = ok ? 1.0 / r0[g] : 0.0;
        r0[g] = ok ? r0[g] : 0.0;
    }
    upload(bscale, sc);
    upload(bnorm, r0);
    cast_pre.bind(&amg32, &batch, bscale.p, bnorm.p);
    std::fill(h.begin(), h.end(), o.residual_tolerance);
    upload(btol, h);
    CgResult r = bcg64.solve(stream, P, val.p, cast_pre, batch, rhs.p, x.p, btol.p, maxit);
    // the FP32 hierarchy's finest level may run the bulk-staged smoother step: its status bits say
    // whether every staged copy arrived (as after the single-system mixed solve)
    if (const int ast = amg32.solve_status(stream)) {
        amg_ready = false;   // the next solve sets the hierarchy (and its status) up again
        throw Error((ast & ST_TIMEOUT) ? PORSOL_ERR_TIMEOUT : PORSOL_ERR_BAD_ARG,
                    "AMG smoother: bulk copy of the matrix slices failed (wait gave up or staging area too small)");
    }
    st.iterations = r.iterations;
    st.outer_iterations = 1;
    st.reduction = r.reduction;
    if (r.breakdown) throw Error(PORSOL_ERR_NONFINITE, "CG breakdown (non-positive curvature)");
    if (!r.converged) fail(r.iterations, r.reduction);
}

void porsol_solver::solve(const porsol_fluid* fluid, const double* sat, const double* mobd, const int* bct,
                          const double* bcv, const double* src, const porsol_solve_opts* opts_in,
                          porsol_solve_stats* stats, bool dev)
{
    NvtxRange range("porsol solve");
    require_structure();
    PORSOL_REQUIRE(ip_valid, PORSOL_ERR_STATE, "computeInnerProducts must be called before solve");
    PORSOL_REQUIRE(fluid && sat && bct && bcv && src, PORSOL_ERR_BAD_ARG, "solve: null argument");
    porsol_solve_opts o;
    porsol_solve_opts_default(&o);
    if (opts_in) o = *opts_in;
    if (o.linsolver_type < 0 || o.linsolver_type > 3) {
        throw Error(PORSOL_ERR_UNKNOWN_SOLVER, "Unknown linsolver_type");
    }
    PORSOL_REQUIRE(o.precision == PORSOL_FP64 || o.precision == PORSOL_MIXED, PORSOL_ERR_BAD_ARG,
                   "unknown precision mode");
    PORSOL_REQUIRE(fluid->model == PORSOL_FLUID_CELLWISE || fluid->model == PORSOL_FLUID_COREY2 ||
                       fluid->model == PORSOL_FLUID_TENSOR,
                   PORSOL_ERR_BAD_ARG, "unknown fluid model");
    const bool tensor = fluid->model == PORSOL_FLUID_TENSOR;
    if (o.precision == PORSOL_MIXED && o.linsolver_type == 0)
        o.precision = PORSOL_FP64;   // ILU0 path is FP64 only
    last_opts = o;
    const int nc = S.g.nc, nhf = S.g.nhf;
    cudaStream_t s = stream;
    ensure_recipe(dev ? nullptr : bct, dev ? bct : nullptr);
    const double *d_sat, *d_md = nullptr, *d_bcv, *d_src;
    if (dev) {
        d_sat = sat;
        d_md = mobd;
        d_bcv = bcv;
        d_src = src;
    } else {
        const size_t per = tensor ? 9 : 1;
        in_sat.upload(sat, per * nc, s);
        d_sat = in_sat.p;
        if (mobd) {
            in_mobdens.upload(mobd, per * nc, s);
            d_md = in_mobdens.p;
        }
        in_bcval.upload(bcv, nhf, s);
        d_bcv = in_bcval.p;
        in_src.upload(src, nc, s);
        d_src = in_src.p;
    }
    last_src = d_src;
    const bool mixed = o.precision == PORSOL_MIXED && o.linsolver_type != 0;
    if (mixed) val32.alloc(S.pat.nent);
    const double t_asm = now_ms();
    // Tensor mobilities: this solve's inner products (and gravity fluxes) are rebuilt into Wdyn
    // (gflux_dyn); the assembly then runs with unit scalar mobility on them.
    const double* W_use = W.p;
    const double* gflux_use = gflux.p;
    bool gzero = gravity_zero;
    if (tensor) {
        Wdyn.alloc(size_t(npk) * nc);
        gflux_dyn.alloc(nhf);
        if (ones.n != size_t(nc)) {
            std::vector<double> h1(nc, 1.0);
            ones.upload(h1, s);
        }
        gzero = gravity_zero || d_md == nullptr;
        TensorIpArgs ta;
        ta.nc = nc;
        ta.facepos = facepos.p;
        ta.area = area.p;
        ta.fcent = fcent.p;
        ta.fnormal = fnormal.p;
        ta.cvol = cvol.p;
        ta.ccent = ccent.p;
        ta.perm = perm.p;
        ta.lam = d_sat;
        ta.rlam = d_md;
        ta.gravity = gzero ? 0 : 1;
        ta.g0 = grav_[0];
        ta.g1 = grav_[1];
        ta.g2 = grav_[2];
        ta.W = Wdyn.p;
        ta.gflux = gflux_dyn.p;
        ta.status = status.p;
        launch_dynamic_ip_tensor(maxnf, s, ta);
        int st_dev = 0;
        PORSOL_CUDA(cudaMemcpyAsync(&st_dev, status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        PORSOL_CUDA(cudaStreamSynchronize(s));
        if (st_dev & ST_BAD_INDEX) {
            PORSOL_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), s));
            throw Error(PORSOL_ERR_BAD_ARG, "tensor mobility: lambda_t K must be symmetric (at most 12 faces per cell)");
        }
        check_status("tensor inner products");
        W_use = Wdyn.p;
        gflux_use = gflux_dyn.p;
        d_sat = ones.p;
        d_md = gzero ? nullptr : ones.p;
    }
    W_last = W_use;
    tensor_last = tensor;
    {
        // per cell: packed W read, local Schur entries written, mobilities/sources/F/L/g/rhs pieces
        // ~64 B; per SELL slot: recipe pointer + entry + gathered local entry + value written (+ the
        // FP32 copy); per row: right-hand-side recipe and pieces
        bytes_asm = double(nc) * (npk * 16.0 + 64.0) + double(S.pat.nent) * (4.0 + 4.0 + 8.0 + 8.0 + (mixed ? 4.0 : 0.0)) +
                    double(S.N) * (4.0 + 2.0 * (4.0 + 8.0) + 8.0);
        bytes_krylov = bytes_rec = bytes_post = 0.0;
        ProfScope ps(prof, s, PK_ASSEMBLE, double(nc) * (npk * 16.0 + 64) + double(S.pat.nent) * 16.0);
        AssembleArgs a;
        a.nc = nc;
        a.facepos = facepos.p;
        a.W = W_use;
        a.gflux = gflux_use;
        a.gravity_zero = gzero;
        a.fluid = tensor ? FluidParams{PORSOL_FLUID_CELLWISE, 1.0, 1.0, 0.0, 0.0}
                         : FluidParams{fluid->model, fluid->viscosity1, fluid->viscosity2, fluid->density1,
                                       fluid->density2};
        a.sat = d_sat;
        a.mobdens = d_md;
        a.kind = R.kind_d.p;
        a.bcval = d_bcv;
        a.src = d_src;
        a.sloc = sloc.p;
        a.F = F.p;
        a.L = L.p;
        a.g = this->g.p;
        a.rrow = rrow.p;
        a.pb = pb.p;
        a.totmob = totmob.p;
        a.mobdens_out = mobdens.p;
        a.status = status.p;
        launch_assemble_cells(maxnf, s, a);
        launch_gather_slots(s, S.pat.nent, R.slot_ptr.p, R.slot_ent.p, sloc.p, val.p, mixed ? val32.p : nullptr);
        launch_gather_rhs(s, S.N, R.rhs_ptr.p, R.rhs_ent.p, rrow.p, pb.p, rhs.p);
    }
    check_status("assembleDynamic");
    // Regularisation of pure Neumann/periodic problems: the ILU0 path always applies it
    // (:1398-1400); the AMG paths only when the hierarchy is rebuilt (:1491-1495).
    reg_applied = false;
    if (!reg_rows.empty()) {
        // batched sub-grids: each sub-grid's first DOF is pinned to 0, the face pressures its
        // own pure-periodic solve with S[0][0] *= 2 would give, without the tiny eigenvalue
        launch_pin_rows(s, int(reg_rows.size()), reg_rows_d.p, S.pat.slice_ptr.p, S.pat.col.p, S.pat.rowlen.p, val.p,
                        mixed ? val32.p : nullptr, rhs.p);
    } else if (R.do_reg && (o.linsolver_type == 0 || !o.same_matrix)) {
        launch_scale_entry(s, val.p, S.pat.diag.p, S.dof(0), 2.0, mixed ? val32.p : nullptr);
        reg_applied = true;
    }
    porsol_solve_stats st{};
    st.ms_assemble = now_ms() - t_asm;
    gflux_last = gflux_use;
    gzero_last = gzero;
    if (assemble_only) {   // batched upscaling solves the assembled systems itself
        if (stats) *stats = st;
        return;
    }
    const double t_lin = now_ms();
    linear_solve(o, st);
    st.ms_krylov = now_ms() - t_lin - st.ms_precond_setup;
    recover_solution(st);
    solved = true;
    if (stats) *stats = st;
}

// Pressure and flux recovery (computePressureAndFluxes) from the face pressures in x, and the FP64
// mass-balance check, with the inner products, gravity fluxes and sources of the last assembly.
void porsol_solver::recover_solution(porsol_solve_stats& st)
{
    const int nc = S.g.nc;
    cudaStream_t s = stream;
    const double* W_use = W_last;
    const double* gflux_use = gflux_last;
    const bool gzero = gzero_last;
    const double* d_src = last_src;
    const double t_rec = now_ms();
    {
        // per cell: W, the face pressures gathered through cf, F, L, g, mobility in; pressure and
        // half-face fluxes out (the profiler's figure for this kernel)
        bytes_rec = double(nc) * (npk * 8.0 + 6 * 8 * 4 + 32) + double(S.N) * 8.0;
        ProfScope ps(prof, s, PK_RECOVER, double(nc) * (npk * 8.0 + 6 * 8 * 4 + 32) + double(S.N) * 8.0);
        RecoverArgs ra;
        ra.nc = nc;
        ra.facepos = facepos.p;
        ra.cf = cf.p;
        ra.x = x.p;
        ra.W = W_use;
        ra.gflux = gflux_use;
        ra.gravity_zero = gzero;
        ra.F = F.p;
        ra.L = L.p;
        ra.g = this->g.p;
        ra.totmob = totmob.p;
        ra.mobdens = mobdens.p;
        ra.pressure = pressure.p;
        ra.outflux = outflux.p;
        launch_recover(maxnf, s, ra);
    }
    // FP64 mass-balance check
    PORSOL_CUDA(cudaMemsetAsync(redbits.p, 0, 3 * sizeof(unsigned long long), s));
    launch_mass_balance(s, nc, facepos.p, outflux.p, d_src, redbits.p);
    unsigned long long mb[3];
    PORSOL_CUDA(cudaMemcpyAsync(mb, redbits.p, sizeof(mb), cudaMemcpyDeviceToHost, s));
    PORSOL_CUDA(cudaStreamSynchronize(s));
    double v[3];
    std::memcpy(v, mb, sizeof(v));
    st.mass_balance = v[0] / std::max(std::max(v[1], v[2]), 1e-300);
    st.ms_recover = now_ms() - t_rec;
}

double porsol_solver::post_process()
{
    NvtxRange range("porsol postProcessFluxes");
    PORSOL_REQUIRE(solved, PORSOL_ERR_STATE, "postProcessFluxes before solve");
    PORSOL_CUDA(cudaMemsetAsync(redbits.p + 3, 0, sizeof(unsigned long long), stream));
    launch_post_process(stream, int(S.pairs.size() / 2), pairs.p, outflux.p, redbits.p + 3);
    bytes_post = double(S.pairs.size() / 2) * (2 * 4.0 + 2 * 8.0 + 2 * 8.0);   // pair indices, fluxes in and out
    unsigned long long b = 0;
    PORSOL_CUDA(cudaMemcpyAsync(&b, redbits.p + 3, sizeof(b), cudaMemcpyDeviceToHost, stream));
    PORSOL_CUDA(cudaStreamSynchronize(stream));
    double d;
    std::memcpy(&d, &b, sizeof(d));
    return d;
}

// Batched periodic upscaling: one block-diagonal system over the disjoint union of the
// sub-grids, solved for the three unit pressure drops with one AMG hierarchy.
void porsol_solver::upscale(const porsol_grid* grid, int ngrids, const int* cellpos, const int* partner,
                            const int* side, const double* perm_h, const porsol_solve_opts* opts_in, double* keff,
                            porsol_solve_stats* stats)
{
    NvtxRange range("porsol upscale periodic");
    PORSOL_REQUIRE(grid && cellpos && partner && side && perm_h && keff && ngrids > 0, PORSOL_ERR_BAD_ARG,
                   "upscale: null argument");
    const int nc = grid->num_cells;
    PORSOL_REQUIRE(cellpos[0] == 0 && cellpos[ngrids] == nc, PORSOL_ERR_BAD_ARG, "upscale: grid_cellpos");
    for (int g = 0; g < ngrids; ++g)
        PORSOL_REQUIRE(cellpos[g + 1] > cellpos[g], PORSOL_ERR_BAD_ARG, "upscale: empty sub-grid");
    const int nhf = grid->cell_facepos[nc];
    std::vector<int> bct(nhf, PORSOL_BC_NEUMANN);
    for (int hf = 0; hf < nhf; ++hf)
        if (grid->hf_neighbour[hf] < 0) {
            PORSOL_REQUIRE(side[hf] >= 1 && side[hf] <= 6, PORSOL_ERR_BAD_ARG, "upscale: boundary side not in 1..6");
            bct[hf] = PORSOL_BC_PERIODIC;
        }
    init_structure(grid, bct.data(), partner);
    // every boundary face is periodic, so the face numbering is the reference's (the sub-grids'
    // unknown ranges below rely on it)
    PORSOL_REQUIRE(!S.renumbered(), PORSOL_ERR_STATE, "upscale: unexpected internal face numbering");
    const double zero3[3] = {0.0, 0.0, 0.0};
    compute_inner_products(perm_h, zero3);
    // per sub-grid: side areas A_i (high sides), extents L_d, first DOF
    std::vector<double> A(3 * size_t(ngrids), 0.0), L(3 * size_t(ngrids), 0.0);
    std::vector<int> dof0(ngrids);
    const HostGrid& hg = S.g;   // topology; the geometry is read from the caller's grid
    for (int g = 0; g < ngrids; ++g) {
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        int d0 = S.N;
        for (int c = cellpos[g]; c < cellpos[g + 1]; ++c)
            for (int hf = hg.facepos[c]; hf < hg.facepos[c + 1]; ++hf) {
                d0 = std::min(d0, S.cf[hf]);
                const int sd = side[hf];
                if (!hg.boundary(hf)) continue;
                const int ax = (sd - 1) / 2;
                const double x = grid->hf_centroid[3 * size_t(hf) + ax];
                if (sd % 2 == 1) lo[ax] = std::min(lo[ax], x);
                else {
                    hi[ax] = std::max(hi[ax], x);
                    A[3 * size_t(g) + ax] += grid->hf_area[hf];
                }
            }
        for (int ax = 0; ax < 3; ++ax) {
            PORSOL_REQUIRE(hi[ax] > lo[ax] && A[3 * size_t(g) + ax] > 0.0, PORSOL_ERR_BAD_ARG,
                           "upscale: a sub-grid lacks boundary faces on some side");
            L[3 * size_t(g) + ax] = hi[ax] - lo[ax];
        }
        dof0[g] = d0;
    }
    reg_rows = dof0;
    reg_rows_d.upload(reg_rows, stream);
    // Unknowns of each sub-grid: its internal faces and its boundary faces are each numbered
    // contiguously (faces are numbered in cell order, internal before boundary).
    {
        std::vector<int> rg(4 * size_t(ngrids));
        for (int g = 0; g < ngrids; ++g) {
            int lo[2] = {S.N, S.N}, hi[2] = {-1, -1};
            long long cnt[2] = {0, 0};
            for (int c = cellpos[g]; c < cellpos[g + 1]; ++c)
                for (int hf = hg.facepos[c]; hf < hg.facepos[c + 1]; ++hf) {
                    const int b = hg.boundary(hf) ? 1 : 0;
                    lo[b] = std::min(lo[b], S.cf[hf]);
                    hi[b] = std::max(hi[b], S.cf[hf]);
                    cnt[b] += b ? 2 : 1;   // internal faces are seen from both cells
                }
            for (int b = 0; b < 2; ++b) {
                if (hi[b] < 0) lo[b] = hi[b] = 0;
                else
                    PORSOL_REQUIRE(cnt[b] == 2LL * (hi[b] - lo[b] + 1), PORSOL_ERR_BAD_ARG,
                                   "upscale: face unknowns of a sub-grid are not contiguous");
                rg[4 * size_t(g) + 2 * b] = lo[b];
                rg[4 * size_t(g) + 2 * b + 1] = hi[b] < 0 ? 0 : hi[b] + 1;
            }
        }
        batch.build(rg, S.N, stream);
    }
    DBuf<int> cellpos_d, side_d;
    cellpos_d.upload(cellpos, ngrids + 1, stream);
    side_d.upload(side, nhf, stream);
    DBuf<double> q_d;
    q_d.alloc(3 * size_t(ngrids));
    // the solves' inputs on the device: unit mobility, zero sources, the boundary types once, and
    // each direction's pressure jumps written from the side tags (no host arrays per direction)
    std::vector<double> q(3 * size_t(ngrids));
    up_ones.alloc(nc);
    up_zeros.alloc(nc);
    up_bcv.alloc(nhf);
    launch_fill(stream, nc, 1.0, up_ones.p);
    up_zeros.zero(stream);
    in_bctype.upload(bct, stream);
    auto jumps = [&](int d) { launch_jump_values(stream, nhf, side_d.p, d, up_bcv.p); };
    porsol_fluid fl{PORSOL_FLUID_CELLWISE, 1.0, 1.0, 0.0, 0.0};
    porsol_solve_opts o;
    porsol_solve_opts_default(&o);
    if (opts_in) o = *opts_in;
    o.same_matrix = 0;
    porsol_solve_stats acc{};
    up_last = UpscaleSchedule{};
    auto finish = [&] {
        assemble_only = false;
        reuse_amg = false;
        reg_rows.clear();
        batch.nblk = 0;
    };
    if (upscale_schedule == PORSOL_UPSCALE_PERSISTENT) {
        // the three systems differ only in their right-hand sides: assemble each (matrix and
        // pinned rows), keep its right-hand side, solve all sub-grids and directions in one
        // launch, then recover each direction's fluxes
        try {
            const int N = S.N;
            up_b3.alloc(3 * size_t(N));
            up_x3.alloc(3 * size_t(N));
            o.precision = PORSOL_MIXED;   // the assembly also writes the FP32 copy of the matrix
            o.linsolver_type = 1;
            for (int d = 0; d < 3; ++d) {
                jumps(d);
                porsol_solve_stats st{};
                assemble_only = true;
                solve(&fl, up_ones.p, up_zeros.p, in_bctype.p, up_bcv.p, up_zeros.p, &o, &st, true);
                assemble_only = false;
                launch_put3(stream, N, rhs.p, up_b3.p, d);
                acc.ms_assemble += st.ms_assemble;
            }
            const double t0 = now_ms();
            // 0: the unknowns of the largest sub-grid (each sub-grid is its own system)
            int largest = 1;
            for (size_t g = 0; g + 3 < batch.h.size(); g += 4)
                largest = std::max(largest, (batch.h[g + 1] - batch.h[g]) + (batch.h[g + 3] - batch.h[g + 2]));
            const int maxit = o.linsolver_maxit > 0 ? o.linsolver_maxit : largest;
            const UpscaleResult r = pup.solve(stream, S.pat, val.p, val32.p, batch.h, batch.ranges.p, up_b3.p,
                                              up_x3.p, o.residual_tolerance,
                                              o.inner_tolerance > 0 ? o.inner_tolerance : 3e-3, maxit, upscale_fixed);
            up_last = pup.last_schedule();
            acc.ms_krylov = now_ms() - t0;
            bytes_krylov = pup.bytes();
            vcycle_level_bytes.clear();
            if (r.breakdown) throw Error(PORSOL_ERR_NONFINITE, "CG breakdown (non-positive curvature)");
            if (!r.converged) {
                std::ostringstream os;
                os << "Linear solver failed to converge in " << maxit << " iterations.\n"
                   << "Residual reduction achieved is " << r.reduction << '\n';
                throw Error(PORSOL_ERR_NOT_CONVERGED, os.str());
            }
            acc.iterations = 3 * r.iterations;
            acc.outer_iterations = 1;
            acc.reduction = r.reduction;
            acc.amg_levels = 0;
            for (int d = 0; d < 3; ++d) {
                launch_get3(stream, N, up_x3.p, x.p, d, up_last.layout);
                porsol_solve_stats st{};
                recover_solution(st);
                acc.mass_balance = std::max(acc.mass_balance, st.mass_balance);
                acc.ms_recover += st.ms_recover;
                launch_side_fluxes(stream, ngrids, cellpos_d.p, facepos.p, side_d.p, outflux.p, q_d.p);
                q_d.download(q.data(), q.size(), stream);
                PORSOL_CUDA(cudaStreamSynchronize(stream));
                for (int g = 0; g < ngrids; ++g)
                    for (int i = 0; i < 3; ++i)
                        keff[9 * size_t(g) + 3 * i + d] =
                            L[3 * size_t(g) + d] * q[3 * size_t(g) + i] / A[3 * size_t(g) + i];
            }
            solved = true;
        } catch (...) {
            finish();
            throw;
        }
        finish();
        if (stats) *stats = acc;
        return;
    }
    try {
        for (int d = 0; d < 3; ++d) {
            jumps(d);
            reuse_amg = d > 0;
            porsol_solve_stats st{};
            solve(&fl, up_ones.p, up_zeros.p, in_bctype.p, up_bcv.p, up_zeros.p, &o, &st, true);
            launch_side_fluxes(stream, ngrids, cellpos_d.p, facepos.p, side_d.p, outflux.p, q_d.p);
            q_d.download(q.data(), q.size(), stream);
            PORSOL_CUDA(cudaStreamSynchronize(stream));
            for (int g = 0; g < ngrids; ++g)
                for (int i = 0; i < 3; ++i)
                    keff[9 * size_t(g) + 3 * i + d] = L[3 * size_t(g) + d] * q[3 * size_t(g) + i] / A[3 * size_t(g) + i];
            acc.iterations += st.iterations;
            acc.outer_iterations += st.outer_iterations;
            acc.reduction = std::max(acc.reduction, st.reduction);
            acc.amg_levels = st.amg_levels;
            acc.mass_balance = std::max(acc.mass_balance, st.mass_balance);
            acc.ms_assemble += st.ms_assemble;
            acc.ms_precond_setup += st.ms_precond_setup;
            acc.ms_krylov += st.ms_krylov;
            acc.ms_recover += st.ms_recover;
        }
    } catch (...) {
        reuse_amg = false;
        reg_rows.clear();
        batch.nblk = 0;
        throw;
    }
    reuse_amg = false;
    reg_rows.clear();
    batch.nblk = 0;
    if (stats) *stats = acc;
}

// ---------------------------------------------------------------- adjoint
namespace {
const double* upload_or_null(DBuf<double>& b, const double* h, size_t n, cudaStream_t s)
{
    if (!h) return nullptr;
    b.upload(h, n, s);
    return b.p;
}
}  // namespace

double porsol_solver::objective(const porsol_objective* obj)
{
    PORSOL_REQUIRE(solved, PORSOL_ERR_STATE, "objective: no solution (call solve first)");
    PORSOL_REQUIRE(obj, PORSOL_ERR_BAD_ARG, "objective: null argument");
    PORSOL_REQUIRE(gravity_zero, PORSOL_ERR_BAD_ARG, "adjoint: only zero gravity is supported");
    PORSOL_REQUIRE(!R.do_reg && reg_rows.empty(), PORSOL_ERR_BAD_ARG,
                   "adjoint: the problem needs at least one Dirichlet face");
    for (int k : R.kind)
        PORSOL_REQUIRE(k != HK_PERIODIC_HI && k != HK_PERIODIC_LO, PORSOL_ERR_BAD_ARG,
                       "adjoint: periodic faces are not supported");
    const int nc = S.g.nc, nhf = S.g.nhf;
    cudaStream_t s = stream;
    AdjointArgs a{};
    a.nc = nc;
    a.facepos = facepos.p;
    a.cf = cf.p;
    a.kind = R.kind_d.p;
    a.sloc = sloc.p;
    a.W = W_last;
    a.F = F.p;
    a.L = L.p;
    a.g = this->g.p;
    a.totmob = totmob.p;
    a.pressure = pressure.p;
    a.x = x.p;
    a.wp = upload_or_null(adj_wp, obj->cell_weight, nc, s);
    a.pstar = upload_or_null(adj_pstar, obj->cell_target, nc, s);
    a.wv = upload_or_null(adj_wv, obj->hf_weight, nhf, s);
    adj_y.alloc(nhf);
    adj_jc.alloc(nc);
    a.y = adj_y.p;
    a.jc = adj_jc.p;
    a.status = status.p;
    launch_adjoint_source(maxnf, s, a);
    adj_sum.alloc(sum_scratch_size());
    launch_sum(s, nc, adj_jc.p, adj_sum.p);
    double J = 0.0;
    PORSOL_CUDA(cudaMemcpyAsync(&J, adj_sum.p + sum_result_index(nc), sizeof(double), cudaMemcpyDeviceToHost, s));
    check_status("objective");
    return J;
}

void porsol_solver::adjoint_gradient(const porsol_objective* obj, int mode, const porsol_solve_opts* opts_in,
                                     double* value, double* grad, porsol_solve_stats* stats)
{
    NvtxRange range("porsol adjoint gradient");
    PORSOL_REQUIRE(mode == PORSOL_GRAD_LOGK || mode == PORSOL_GRAD_LOGK_AXES, PORSOL_ERR_BAD_ARG,
                   "adjoint: unknown gradient mode");
    PORSOL_REQUIRE(grad, PORSOL_ERR_BAD_ARG, "adjoint: null gradient array");
    PORSOL_REQUIRE(!(tensor_last && mode == PORSOL_GRAD_LOGK_AXES), PORSOL_ERR_BAD_ARG,
                   "adjoint: axis gradients are not available with tensor mobilities");
    const double J = objective(obj);   // also leaves dJ/dpi in adj_y
    const int nc = S.g.nc, N = S.N;
    cudaStream_t s = stream;
    adj_rhs.alloc(N);
    adj_x.alloc(N);
    launch_adjoint_rhs(s, N, R.rhs_ptr.p, R.rhs_ent.p, R.kind_d.p, adj_y.p, adj_rhs.p);
    // The adjoint system is the assembled (symmetric) matrix of the forward solve: swap the
    // adjoint vectors in as right-hand side and solution, keep the hierarchy.
    porsol_solve_opts o = opts_in ? *opts_in : last_opts;
    if (o.precision == PORSOL_MIXED && o.linsolver_type == 0) o.precision = PORSOL_FP64;
    o.same_matrix = 1;
    porsol_solve_stats st{};
    std::swap(rhs, adj_rhs);
    std::swap(x, adj_x);
    const double t0 = now_ms();
    try {
        linear_solve(o, st);
    } catch (...) {
        std::swap(rhs, adj_rhs);
        std::swap(x, adj_x);
        throw;
    }
    std::swap(rhs, adj_rhs);
    std::swap(x, adj_x);
    st.ms_krylov = now_ms() - t0 - st.ms_precond_setup;
    const double t1 = now_ms();
    AdjointArgs a{};
    a.nc = nc;
    a.mode = mode;
    a.facepos = facepos.p;
    a.cf = cf.p;
    a.kind = R.kind_d.p;
    a.W = W_last;
    a.F = F.p;
    a.L = L.p;
    a.g = this->g.p;
    a.totmob = totmob.p;
    a.pressure = pressure.p;
    a.x = x.p;
    a.mu = adj_x.p;
    a.wp = obj->cell_weight ? adj_wp.p : nullptr;
    a.pstar = obj->cell_target ? adj_pstar.p : nullptr;
    a.wv = obj->hf_weight ? adj_wv.p : nullptr;
    a.area = area.p;
    a.fcent = fcent.p;
    a.fnormal = fnormal.p;
    a.cvol = cvol.p;
    a.ccent = ccent.p;
    a.perm = perm.p;
    const size_t ng = (mode == PORSOL_GRAD_LOGK ? 1 : 3) * size_t(nc);
    adj_grad.alloc(ng);
    a.grad = adj_grad.p;
    a.status = status.p;
    launch_adjoint_grad(maxnf, s, a);
    adj_grad.download(grad, ng, s);
    {
        int st_dev = 0;
        PORSOL_CUDA(cudaMemcpyAsync(&st_dev, status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        PORSOL_CUDA(cudaStreamSynchronize(s));
        if (st_dev & ST_BAD_INDEX) {
            PORSOL_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), s));
            throw Error(PORSOL_ERR_BAD_ARG, "adjoint: axis gradients need diagonal permeability tensors");
        }
    }
    check_status("adjoint gradient");
    st.ms_recover = now_ms() - t1;
    if (value) *value = J;
    if (stats) *stats = st;
}

// ---------------------------------------------------------------- C ABI
namespace {

template <class F>
int guarded(porsol_solver* h, F&& f)
{
    if (!h) return PORSOL_ERR_BAD_ARG;
    try {
        PORSOL_CUDA(cudaSetDevice(h->device));
        f();
        h->err.clear();
        return PORSOL_OK;
    } catch (const Error& e) {
        h->err = e.what();
        return e.code;
    } catch (const std::exception& e) {
        h->err = e.what();
        return PORSOL_ERR_BAD_ARG;
    } catch (...) {
        h->err = "unknown error";
        return PORSOL_ERR_BAD_ARG;
    }
}

}  // namespace

extern "C" {

void porsol_solve_opts_default(porsol_solve_opts* o)
{
    if (!o) return;
    o->residual_tolerance = 1e-8;
    o->linsolver_verbosity = 1;
    o->linsolver_type = 1;
    o->same_matrix = 0;
    o->linsolver_maxit = 0;
    o->prolongate_factor = 1.6;
    o->smooth_steps = 1;
    o->precision = PORSOL_FP64;
    o->inner_tolerance = 3e-3;
    o->max_outer = 30;
}

int porsol_create(porsol_solver** out)
{
    if (!out) return PORSOL_ERR_BAD_ARG;
    *out = nullptr;
    auto* h = new (std::nothrow) porsol_solver();
    if (!h) return PORSOL_ERR_BAD_ARG;
    if (cudaGetDevice(&h->device) != cudaSuccess || cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return PORSOL_ERR_CUDA;
    }
    *out = h;
    return PORSOL_OK;
}

void porsol_destroy(porsol_solver* h)
{
    if (!h) return;
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    cudaStream_t s = h->stream;
    delete h;
    cudaStreamDestroy(s);
}

const char* porsol_last_error(const porsol_solver* h) { return h ? h->err.c_str() : "null handle"; }

int porsol_clear(porsol_solver* h)
{
    return guarded(h, [&] {
        h->structure_valid = h->ip_valid = h->solved = false;
        h->R.valid = false;
        h->amg_ready = false;
    });
}

int porsol_init_system_structure(porsol_solver* h, const porsol_grid* grid, const int* flow_type,
                                 const int* partner_bid)
{
    return guarded(h, [&] { h->init_structure(grid, flow_type, partner_bid); });
}

int porsol_compute_inner_products(porsol_solver* h, const double* perm, const double* grav)
{
    return guarded(h, [&] { h->compute_inner_products(perm, grav); });
}

int porsol_assemble_static(porsol_solver* h, const double* perm, const double* grav)
{
    return porsol_compute_inner_products(h, perm, grav);
}

int porsol_init(porsol_solver* h, const porsol_grid* grid, const double* perm, const double* grav,
                const int* flow_type, const int* partner_bid)
{
    return guarded(h, [&] {
        if (grid && grid->num_cells == 0) {
            h->structure_valid = h->ip_valid = false;
            return;
        }
        h->init_structure(grid, flow_type, partner_bid);
        h->compute_inner_products(perm, grav);
    });
}

int porsol_solve(porsol_solver* h, const porsol_fluid* fluid, const double* sat, const double* mobdens,
                 const int* bct, const double* bcv, const double* src, const porsol_solve_opts* opts,
                 porsol_solve_stats* stats)
{
    return guarded(h, [&] { h->solve(fluid, sat, mobdens, bct, bcv, src, opts, stats, false); });
}

int porsol_solve_device(porsol_solver* h, const porsol_fluid* fluid, const double* sat, const double* mobdens,
                        const int* bct, const double* bcv, const double* src, const porsol_solve_opts* opts,
                        porsol_solve_stats* stats)
{
    return guarded(h, [&] { h->solve(fluid, sat, mobdens, bct, bcv, src, opts, stats, true); });
}

int porsol_upscale_periodic(porsol_solver* h, const porsol_grid* grid, int num_grids, const int* grid_cellpos,
                            const int* hf_partner_bid, const int* hf_side, const double* perm,
                            const porsol_solve_opts* opts, double* k_eff, porsol_solve_stats* stats)
{
    return guarded(h, [&] {
        h->upscale(grid, num_grids, grid_cellpos, hf_partner_bid, hf_side, perm, opts, k_eff, stats);
    });
}

int porsol_upscale_set_schedule(porsol_solver* h, int schedule, int cta_threads, int warp_max_unknowns,
                                int vector_layout, int cluster_ctas, int cluster_min_unknowns)
{
    return guarded(h, [&] {
        PORSOL_REQUIRE(schedule == PORSOL_UPSCALE_AMG || schedule == PORSOL_UPSCALE_PERSISTENT, PORSOL_ERR_BAD_ARG,
                       "upscale schedule: unknown schedule");
        PORSOL_REQUIRE(cta_threads == 0 || cta_threads == 256 || cta_threads == 512 || cta_threads == 1024,
                       PORSOL_ERR_BAD_ARG, "upscale schedule: CTA threads must be 0, 256, 512 or 1024");
        PORSOL_REQUIRE(warp_max_unknowns >= 0, PORSOL_ERR_BAD_ARG, "upscale schedule: negative warp limit");
        PORSOL_REQUIRE(vector_layout == 0 || vector_layout == 1, PORSOL_ERR_BAD_ARG,
                       "upscale schedule: vector layout must be 0 or 1");
        PORSOL_REQUIRE(cluster_ctas == 1 || cluster_ctas == 2 || cluster_ctas == 4, PORSOL_ERR_BAD_ARG,
                       "upscale schedule: cluster size must be 1, 2 or 4");
        PORSOL_REQUIRE(cluster_min_unknowns >= 0, PORSOL_ERR_BAD_ARG, "upscale schedule: negative cluster limit");
        h->upscale_schedule = schedule;
        h->upscale_fixed = porsol::UpscaleSchedule{};
        h->upscale_fixed.cta_threads = cta_threads;
        h->upscale_fixed.warp_max_unknowns = cta_threads ? warp_max_unknowns : 0;
        h->upscale_fixed.layout = vector_layout;
        h->upscale_fixed.cluster = cta_threads ? cluster_ctas : 1;
        h->upscale_fixed.cluster_min_unknowns = cta_threads && cluster_ctas > 1 ? cluster_min_unknowns : 0;
    });
}

int porsol_upscale_last_schedule(porsol_solver* h, int* cta_threads, int* warp_max_unknowns, int* vector_layout,
                                 int* cluster_ctas, int* cluster_min_unknowns, int* tuned)
{
    return guarded(h, [&] {
        PORSOL_REQUIRE(cta_threads && warp_max_unknowns && vector_layout && cluster_ctas && cluster_min_unknowns &&
                           tuned,
                       PORSOL_ERR_BAD_ARG, "upscale schedule: null argument");
        const porsol::UpscaleSchedule& sc = h->up_last;
        *cta_threads = sc.cta_threads;
        *warp_max_unknowns = sc.warp_max_unknowns;
        *vector_layout = sc.cta_threads ? sc.layout : 0;
        *cluster_ctas = sc.cta_threads ? sc.cluster : 0;
        *cluster_min_unknowns = sc.cta_threads ? sc.cluster_min_unknowns : 0;
        *tuned = sc.tuned ? 1 : 0;
    });
}

int porsol_cell_fields(porsol_solver* h, const porsol_fluid* fluid, const double* sat, double* velocity,
                       double* water_velocity, double* oil_velocity, double* fractional_flow, double* cap_pressure)
{
    return guarded(h, [&] {
        PORSOL_REQUIRE(h->solved, PORSOL_ERR_STATE, "cell fields: no solution (call solve first)");
        const bool satf = water_velocity || oil_velocity || fractional_flow || cap_pressure;
        PORSOL_REQUIRE(!satf || (sat && fluid && fluid->model == PORSOL_FLUID_COREY2), PORSOL_ERR_BAD_ARG,
                       "cell fields: saturation fields need sat and a Corey-2 fluid");
        const int nc = h->S.g.nc;
        cudaStream_t s = h->stream;
        DBuf<double> d_sat, out;
        const size_t o_v = 0, o_w = 3 * size_t(nc), o_o = 6 * size_t(nc), o_f = 9 * size_t(nc), o_p = 10 * size_t(nc);
        out.alloc(11 * size_t(nc));
        CellFieldArgs a{};
        a.nc = nc;
        a.facepos = h->facepos.p;
        a.fcent = h->fcent.p;
        a.ccent = h->ccent.p;
        a.cvol = h->cvol.p;
        a.outflux = h->outflux.p;
        if (satf) {
            d_sat.upload(sat, nc, s);
            a.sat = d_sat.p;
            a.mu1 = fluid->viscosity1;
            a.mu2 = fluid->viscosity2;
        }
        a.vel = velocity ? out.p + o_v : nullptr;
        a.vw = water_velocity ? out.p + o_w : nullptr;
        a.vo = oil_velocity ? out.p + o_o : nullptr;
        a.fw = fractional_flow ? out.p + o_f : nullptr;
        a.pc = cap_pressure ? out.p + o_p : nullptr;
        launch_cell_fields(s, a);
        auto get = [&](double* dst, size_t off, size_t n) {
            if (dst) PORSOL_CUDA(cudaMemcpyAsync(dst, out.p + off, n * sizeof(double), cudaMemcpyDeviceToHost, s));
        };
        get(velocity, o_v, 3 * size_t(nc));
        get(water_velocity, o_w, 3 * size_t(nc));
        get(oil_velocity, o_o, 3 * size_t(nc));
        get(fractional_flow, o_f, nc);
        get(cap_pressure, o_p, nc);
        PORSOL_CUDA(cudaStreamSynchronize(s));
    });
}

int porsol_write_field(const double* field, int n, const char* filename)
{
    if (!filename || n < 0 || (n > 0 && !field)) return PORSOL_ERR_BAD_ARG;
    FILE* f = std::fopen(filename, "w");
    if (!f) return PORSOL_ERR_BAD_ARG;
    // the reference streams with the default ostream format (6 significant digits, %g)
    std::fprintf(f, "%d\n", n);
    for (int i = 0; i < n; ++i) std::fprintf(f, "%g\n", field[i]);
    return std::fclose(f) == 0 ? PORSOL_OK : PORSOL_ERR_BAD_ARG;
}

int porsol_objective_value(porsol_solver* h, const porsol_objective* obj, double* value)
{
    return guarded(h, [&] {
        PORSOL_REQUIRE(value, PORSOL_ERR_BAD_ARG, "objective: null value");
        *value = h->objective(obj);
    });
}

int porsol_adjoint_gradient(porsol_solver* h, const porsol_objective* obj, int mode, const porsol_solve_opts* opts,
                            double* value, double* grad, porsol_solve_stats* stats)
{
    return guarded(h, [&] { h->adjoint_gradient(obj, mode, opts, value, grad, stats); });
}

int porsol_post_process_fluxes(porsol_solver* h, double* max_modification)
{
    return guarded(h, [&] {
        const double m = h->post_process();
        if (max_modification) *max_modification = m;
    });
}

int porsol_get_solution(porsol_solver* h, double* p, double* v, double* pi)
{
    return guarded(h, [&] {
        PORSOL_REQUIRE(h->solved, PORSOL_ERR_STATE, "getSolution before solve");
        if (p) h->pressure.download(p, h->S.g.nc, h->stream);
        if (v) h->outflux.download(v, h->S.g.nhf, h->stream);
        if (pi) {
            if (h->S.renumbered()) {
                h->pi_ref.alloc(h->S.N);
                launch_permute(h->stream, h->S.N, h->dof_perm_d.p, h->x.p, h->pi_ref.p, true);
                h->pi_ref.download(pi, h->S.N, h->stream);
            } else {
                h->x.download(pi, h->S.N, h->stream);
            }
        }
        PORSOL_CUDA(cudaStreamSynchronize(h->stream));
    });
}

int porsol_get_solution_device(porsol_solver* h, const double** p, const double** v, const double** pi)
{
    return guarded(h, [&] {
        PORSOL_REQUIRE(h->solved, PORSOL_ERR_STATE, "getSolution before solve");
        PORSOL_CUDA(cudaStreamSynchronize(h->stream));
        if (p) *p = h->pressure.p;
        if (v) *v = h->outflux.p;
        if (pi) {
            if (h->S.renumbered()) {   // face pressures in the reference numbering
                h->pi_ref.alloc(h->S.N);
                launch_permute(h->stream, h->S.N, h->dof_perm_d.p, h->x.p, h->pi_ref.p, true);
                PORSOL_CUDA(cudaStreamSynchronize(h->stream));
                *pi = h->pi_ref.p;
            } else {
                *pi = h->x.p;
            }
        }
    });
}

int porsol_num_dofs(porsol_solver* h, int* num_dofs, int* nnz, int* max_ncf, int* num_internal)
{
    return guarded(h, [&] {
        h->require_structure();
        if (num_dofs) *num_dofs = h->S.N;
        if (nnz) *nnz = int(h->S.colind.size());
        if (max_ncf) *max_ncf = h->S.max_ncf;
        if (num_internal) *num_internal = h->S.num_internal;
    });
}

int porsol_get_structure(porsol_solver* h, int* cellfaces, int* rowptr, int* colind, int* ppartner)
{
    return guarded(h, [&] {
        h->require_structure();
        const Structure& S = h->S;
        if (cellfaces) std::copy(S.cf.begin(), S.cf.end(), cellfaces);
        if (rowptr) std::copy(S.rowptr.begin(), S.rowptr.end(), rowptr);
        if (colind) std::copy(S.colind.begin(), S.colind.end(), colind);
        if (ppartner) {
            if (S.ppartner.empty()) std::fill(ppartner, ppartner + S.N, -1);
            else std::copy(S.ppartner.begin(), S.ppartner.end(), ppartner);
        }
    });
}

int porsol_get_inner_products(porsol_solver* h, double* binv, double* gflux)
{
    return guarded(h, [&] {
        PORSOL_REQUIRE(h->ip_valid, PORSOL_ERR_STATE, "computeInnerProducts first");
        const int nc = h->S.g.nc;
        if (binv) {
            std::vector<double> W(size_t(h->npk) * nc);
            h->W.download(W.data(), W.size(), h->stream);
            PORSOL_CUDA(cudaStreamSynchronize(h->stream));
            size_t o = 0;
            for (int c = 0; c < nc; ++c) {
                const int nf = h->S.g.nf(c);
                for (int j = 0; j < nf; ++j)
                    for (int i = 0; i < nf; ++i) binv[o++] = W[size_t(packed_index(i, j)) * nc + c];
            }
        }
        if (gflux) h->gflux.download(gflux, h->S.g.nhf, h->stream);
        PORSOL_CUDA(cudaStreamSynchronize(h->stream));
    });
}

int porsol_get_system(porsol_solver* h, double* values, double* rhs)
{
    return guarded(h, [&] {
        PORSOL_REQUIRE(h->solved, PORSOL_ERR_STATE, "get_system before solve");
        const Structure& S = h->S;
        if (values) {
            std::vector<double> v(S.pat.nent);
            h->val.download(v.data(), v.size(), h->stream);
            PORSOL_CUDA(cudaStreamSynchronize(h->stream));
            for (size_t k = 0; k < S.csr2sell.size(); ++k) values[k] = v[S.csr2sell[k]];
            if (h->reg_applied && S.N > 0) {
                // report the assembled value before the pure-Neumann regularisation
                const long long k0 = S.slot(0, 0);
                for (size_t k = 0; k < S.csr2sell.size(); ++k)
                    if (S.csr2sell[k] == k0) values[k] = v[k0] / 2.0;
            }
        }
        if (rhs) {
            if (S.renumbered()) {
                std::vector<double> r(S.N);
                h->rhs.download(r.data(), S.N, h->stream);
                PORSOL_CUDA(cudaStreamSynchronize(h->stream));
                for (int i = 0; i < S.N; ++i) rhs[i] = r[S.dof_perm[i]];
            } else {
                h->rhs.download(rhs, S.N, h->stream);
            }
        }
        PORSOL_CUDA(cudaStreamSynchronize(h->stream));
    });
}

int porsol_solve_bytes(porsol_solver* h, double* out4, int max_levels, double* vcycle_level_bytes)
{
    return guarded(h, [&] {
        PORSOL_REQUIRE(h->solved, PORSOL_ERR_STATE, "solve_bytes before solve");
        if (out4) {
            out4[0] = h->bytes_asm;
            out4[1] = h->bytes_krylov;
            out4[2] = h->bytes_rec;
            out4[3] = h->bytes_post;
        }
        for (int l = 0; vcycle_level_bytes && l < max_levels && l < int(h->vcycle_level_bytes.size()); ++l)
            vcycle_level_bytes[l] = h->vcycle_level_bytes[size_t(l)];
    });
}

int porsol_amg_info(porsol_solver* h, int max_levels, int* levels, int* rows, long long* entries)
{
    return guarded(h, [&] {
        const bool f32 = h->amg_precision == PORSOL_MIXED;
        const std::vector<int>& sz = f32 ? h->amg32.level_sizes() : h->amg64.level_sizes();
        const std::vector<long long>& nz = f32 ? h->amg32.level_nnz() : h->amg64.level_nnz();
        if (levels) *levels = int(sz.size());
        for (int l = 0; l < int(sz.size()) && l < max_levels; ++l) {
            if (rows) rows[l] = sz[l];
            if (entries) entries[l] = nz[l];
        }
    });
}

int porsol_profile_enable(porsol_solver* h, int enable)
{
    return guarded(h, [&] { h->prof.on = enable != 0; });
}

int porsol_profile_get(porsol_solver* h, int kernel, int* launches, double* ms, double* bytes)
{
    return guarded(h, [&] {
        PORSOL_REQUIRE(kernel >= 0 && kernel < PK_COUNT, PORSOL_ERR_BAD_ARG, "unknown profiled kernel");
        h->prof.collect();
        if (launches) *launches = h->prof.launches[kernel];
        if (ms) *ms = h->prof.ms[kernel];
        if (bytes) *bytes = h->prof.bytes[kernel];
    });
}

int porsol_profile_reset(porsol_solver* h)
{
    return guarded(h, [&] { h->prof.reset(); });
}

void* porsol_stream(porsol_solver* h) { return h ? (void*)h->stream : nullptr; }

long long porsol_launch_count(void) { return porsol::g_launches.load(); }

int porsol_selftest_bulk_wait(int expire, float* r, float* d, float* x)
{
    if (!r || !d || !x) return PORSOL_ERR_BAD_ARG;
    try {
        const int st = porsol::bulk_step_selftest(expire != 0, r, d, x);
        if (st & porsol::ST_TIMEOUT) return PORSOL_ERR_TIMEOUT;
        return st ? PORSOL_ERR_BAD_ARG : PORSOL_OK;
    } catch (const porsol::Error& e) {
        return e.code;
    } catch (...) {
        return PORSOL_ERR_CUDA;
    }
}

}  // extern "C"
