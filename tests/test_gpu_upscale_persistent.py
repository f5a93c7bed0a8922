"""Batched periodic upscaling in one persistent launch (PORSOL_UPSCALE_PERSISTENT): every sub-grid's
three unit pressure-jump solves (the pattern of setupUpscalingConditions,
common/setupBoundaryConditions.hpp:136-157) by a Jacobi-preconditioned CG per sub-grid, run by a cluster
of CTAs, one CTA or one warp, with FP32 recurrences and FP64 residual replacements deciding convergence.  Checked
against the oracle's per-sub-grid solves, the AMG schedule, analytic cases, and across the schedules
the autotuner chooses from."""
import numpy as np
import pytest

from upscaling import layered_perm, oracle_keff

pytestmark = pytest.mark.gpu


def _solve(pkg, union, K, tol, schedule=None, maxit=4000):
    s = pkg.PressureSolver()
    if schedule is not None:
        s.set_upscale_schedule(pkg.UPSCALE_PERSISTENT, *schedule)
    opts = pkg.default_solve_opts(residual_tolerance=tol, linsolver_maxit=maxit)
    keff, st = s.upscale_periodic(union, union.cellpos, union.partner, union.side, K.ravel(), opts)
    return s, keff, st


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_persistent_small_subgrids_match_oracle_autotuned(pkg, gpulib, orc, workloads):
    union, sizes, K = workloads.periodic_subgrids(num=5, nmin=3, nmax=6, seed=21)
    s, keff, st = _solve(pkg, union, K, 1e-12, schedule=(0, 0))
    sc = s.upscale_last_schedule()
    assert sc["tuned"] and sc["cta_threads"] in (512, 1024) and sc["warp_max_unknowns"] in (0, 4096)
    assert sc["vector_layout"] in (0, 1) and sc["cluster_ctas"] in (1, 2, 4)
    assert st.amg_levels == 0 and st.iterations > 0
    for g in range(len(sizes)):
        c0, c1 = union.cellpos[g], union.cellpos[g + 1]
        ref = oracle_keff(orc, union.grids[g], K[c0:c1])
        assert _rel(keff[g], ref) < 1e-9, g
        assert np.abs(keff[g] - keff[g].T).max() < 1e-8 * np.abs(keff[g]).max()
        assert np.linalg.eigvalsh(0.5 * (keff[g] + keff[g].T)).min() > 0
    s.close()


def test_persistent_sides_8_to_32_against_oracle(pkg, gpulib, orc, workloads):
    """Sides spanning the 512-sub-grid workload's U{8..32}: the 8^3 sub-grid (1728 unknowns) goes to
    a single warp, the others to 512-thread CTAs; both vector layouts."""
    union, sizes, K = workloads.periodic_subgrids(seed=23, sides=[8, 13, 19, 26, 32])
    for layout in (0, 1):
        s, keff, st = _solve(pkg, union, K, 1e-12, schedule=(512, 4096, layout))
        sc = s.upscale_last_schedule()
        assert (sc["cta_threads"], sc["warp_max_unknowns"], sc["vector_layout"], sc["cluster_ctas"], sc["tuned"]) == \
            (512, 4096, layout, 1, False)
        for gi in range(len(sizes)):
            c0, c1 = union.cellpos[gi], union.cellpos[gi + 1]
            ref = oracle_keff(orc, union.grids[gi], K[c0:c1])
            assert _rel(keff[gi], ref) < 1e-9, (layout, int(sizes[gi]), _rel(keff[gi], ref))
        s.close()


def test_persistent_schedules_agree_with_amg_schedule(pkg, gpulib, workloads):
    """Warp and CTA schedules of every size, the autotuned one and the AMG schedule give the same
    tensors to the solve tolerance; a repeated call with the same schedule is bitwise equal."""
    union, sizes, K = workloads.periodic_subgrids(num=24, nmin=8, nmax=20, seed=5)
    s0, ref, _ = _solve(pkg, union, K, 1e-12)   # AMG schedule, FP64
    s0.close()
    for sched in ((256, 0, 1), (1024, 16384, 0), (512, 4096, 1), (1024, 0, 0), (1024, 0, 1, 2, 20000),
                  (512, 4096, 0, 4, 20000), (0, 0, 1)):
        s, k1, st1 = _solve(pkg, union, K, 1e-12, schedule=sched)
        keff2, st2 = s.upscale_periodic(union, union.cellpos, union.partner, union.side, K.ravel(),
                                        pkg.default_solve_opts(residual_tolerance=1e-12, linsolver_maxit=4000))
        assert np.array_equal(k1, keff2), sched
        assert st1.iterations == st2.iterations
        for g in range(len(sizes)):
            assert _rel(k1[g], ref[g]) < 1e-9, (sched, g, _rel(k1[g], ref[g]))
        s.close()


def test_persistent_analytic_cases(pkg, gpulib, cart):
    """Homogeneous full tensor reproduced; layered medium gives the arithmetic mean along and the
    harmonic mean across the layers."""
    rng = np.random.default_rng(4)
    A = rng.normal(size=(3, 3))
    Kh = (A @ A.T + np.eye(3)) * 1e-13
    g1 = cart.CartesianGrid(4, 5, 3, unique_bids=True)
    kz = np.array([1.0, 4.0, 0.5, 2.0, 3.0]) * 1e-13
    g2, K2 = layered_perm(cart, 4, kz)
    union = cart.UnionGrid([g1, g2])
    K = np.concatenate([np.tile(Kh.ravel(), (g1.num_cells, 1)), K2])
    s, keff, st = _solve(pkg, union, K, 1e-13, schedule=(256, 0, 1))
    assert np.abs(keff[0] - Kh).max() < 1e-8 * np.abs(Kh).max()
    assert abs(keff[1][0, 0] - kz.mean()) < 1e-8 * kz.mean()
    assert abs(keff[1][2, 2] - 1.0 / np.mean(1.0 / kz)) < 1e-8 * kz.mean()
    s.close()


def test_persistent_errors(pkg, gpulib, workloads):
    """Too few iterations: the reference's non-convergence error; the handle stays usable. Unknown
    schedules and CTA sizes are rejected."""
    union, sizes, K = workloads.periodic_subgrids(num=3, nmin=6, nmax=8, seed=2)
    s = pkg.PressureSolver()
    s.set_upscale_schedule(pkg.UPSCALE_PERSISTENT, 256, 0, 0)
    with pytest.raises(pkg.PorsolError) as e:
        s.upscale_periodic(union, union.cellpos, union.partner, union.side, K.ravel(),
                           pkg.default_solve_opts(residual_tolerance=1e-12, linsolver_maxit=3))
    assert "failed to converge" in str(e.value)
    keff, st = s.upscale_periodic(union, union.cellpos, union.partner, union.side, K.ravel(),
                                  pkg.default_solve_opts(residual_tolerance=1e-12, linsolver_maxit=4000))
    assert np.isfinite(keff).all()
    for bad in ((7, 0, 0, 1), (1, 300, 0, 1), (1, 256, -1, 1), (1, 256, 0, 2), (1, 256, 0, 1, 3), (1, 256, 0, 1, 2, -1)):
        with pytest.raises(pkg.PorsolError):
            s.set_upscale_schedule(*bad)
    # back to the AMG schedule: the last-schedule query reports zeros
    s.set_upscale_schedule(pkg.UPSCALE_AMG)
    s.upscale_periodic(union, union.cellpos, union.partner, union.side, K.ravel(),
                       pkg.default_solve_opts(residual_tolerance=1e-10))
    assert s.upscale_last_schedule() == dict(cta_threads=0, warp_max_unknowns=0, vector_layout=0, cluster_ctas=0,
                                             cluster_min_unknowns=0, tuned=False)
    s.close()


def test_persistent_cluster_items_against_oracle(pkg, gpulib, orc, workloads):
    """The largest sub-grids solved by clusters of 2 and 4 CTAs (their reductions over distributed
    shared memory, their rows on several SMs), the rest by CTAs and warps, in one launch: the same
    tensors as the oracle's per-sub-grid solves, and bitwise the same on a repeated call."""
    union, sizes, K = workloads.periodic_subgrids(seed=29, sides=[6, 9, 14, 20, 24, 27])
    for cluster in (2, 4):
        s, keff, st = _solve(pkg, union, K, 1e-12, schedule=(512, 2000, 1, cluster, 30000))
        sc = s.upscale_last_schedule()
        assert sc["cluster_ctas"] == cluster and sc["cluster_min_unknowns"] == 30000
        for gi in range(len(sizes)):
            c0, c1 = union.cellpos[gi], union.cellpos[gi + 1]
            ref = oracle_keff(orc, union.grids[gi], K[c0:c1])
            assert _rel(keff[gi], ref) < 1e-9, (cluster, int(sizes[gi]), _rel(keff[gi], ref))
        keff2, _ = s.upscale_periodic(union, union.cellpos, union.partner, union.side, K.ravel(),
                                      pkg.default_solve_opts(residual_tolerance=1e-12, linsolver_maxit=4000))
        assert np.array_equal(keff, keff2), cluster
        s.close()
