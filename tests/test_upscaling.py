"""Batched periodic upscaling (512-sub-grid workload shape): the GPU batch against per-sub-grid FP64 oracle
solves, and analytic effective permeabilities."""
import numpy as np
import pytest

from upscaling import layered_perm, oracle_keff


def test_oracle_homogeneous_tensor_is_reproduced(orc, cart):
    """A spatially constant full tensor is its own effective permeability (CPU)."""
    g = cart.CartesianGrid(4, 3, 5, unique_bids=True)
    rng = np.random.default_rng(1)
    A = rng.normal(size=(3, 3))
    K = A @ A.T + np.eye(3)
    keff = oracle_keff(orc, g, np.tile(K.ravel(), g.num_cells))
    assert np.abs(keff - K).max() < 1e-9 * np.abs(K).max()


def test_oracle_layered_medium_means(orc, cart):
    """Layers across z: arithmetic mean along the layers, harmonic mean across them (CPU)."""
    kz = [1.0, 4.0, 0.5, 2.0]
    g, K = layered_perm(cart, 3, kz)
    keff = oracle_keff(orc, g, K)
    assert abs(keff[0, 0] - np.mean(kz)) < 1e-10 and abs(keff[1, 1] - np.mean(kz)) < 1e-10
    assert abs(keff[2, 2] - 1.0 / np.mean(1.0 / np.array(kz))) < 1e-10
    assert np.abs(keff - np.diag(np.diag(keff))).max() < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_batch_matches_per_subgrid_oracle(pkg, gpulib, orc, workloads, precision):
    union, sizes, K = workloads.periodic_subgrids(num=5, nmin=3, nmax=6, seed=21)
    s = pkg.PressureSolver()
    opts = pkg.default_solve_opts(residual_tolerance=1e-12, precision=precision)
    keff, st = s.upscale_periodic(union, union.cellpos, union.partner, union.side, K.ravel(), opts)
    for g in range(len(sizes)):
        c0, c1 = union.cellpos[g], union.cellpos[g + 1]
        ref = oracle_keff(orc, union.grids[g], K[c0:c1])
        err = np.abs(keff[g] - ref).max() / np.abs(ref).max()
        assert err < (1e-9 if precision == 0 else 1e-8), (g, err)
        # effective tensors are symmetric positive definite
        assert np.abs(keff[g] - keff[g].T).max() < 1e-8 * np.abs(keff[g]).max()
        assert np.linalg.eigvalsh(0.5 * (keff[g] + keff[g].T)).min() > 0


@pytest.mark.gpu
def test_batch_analytic_cases(pkg, gpulib, cart):
    """Homogeneous tensor and layered medium inside one batch."""
    rng = np.random.default_rng(4)
    A = rng.normal(size=(3, 3))
    Kh = (A @ A.T + np.eye(3)) * 1e-13
    g1 = cart.CartesianGrid(4, 5, 3, unique_bids=True)
    kz = np.array([1.0, 4.0, 0.5, 2.0, 3.0]) * 1e-13
    g2, K2 = layered_perm(cart, 4, kz)
    union = cart.UnionGrid([g1, g2])
    K = np.concatenate([np.tile(Kh.ravel(), (g1.num_cells, 1)), K2])
    s = pkg.PressureSolver()
    keff, st = s.upscale_periodic(union, union.cellpos, union.partner, union.side, K.ravel(),
                                  pkg.default_solve_opts(residual_tolerance=1e-13))
    assert np.abs(keff[0] - Kh).max() < 1e-8 * np.abs(Kh).max()
    assert abs(keff[1][0, 0] - kz.mean()) < 1e-8 * kz.mean()
    assert abs(keff[1][2, 2] - 1.0 / np.mean(1.0 / kz)) < 1e-8 * kz.mean()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_converged_blocks_are_skipped_without_changing_results(pkg, gpulib, workloads, precision):
    """The batched CG tells the AMG which sub-grids still iterate; the cycle then leaves the rows of
    converged sub-grids alone. The hierarchy is block diagonal, so the iterating sub-grids see the
    values of a full cycle: the tensors are bitwise those of a sweep over every row
    (PORSOL_BLOCK_SKIP=0). 64 sub-grids of sides 8..32 (0.7 M cells) converge at 26..96 iterations;
    in FP32 the converged sub-grids' partly recomputed rows overflow here, which the dense coarsest
    solve must keep away from the iterating ones."""
    import os
    union, sizes, K = workloads.periodic_subgrids(num=64)
    out = {}
    old = os.environ.get("PORSOL_BLOCK_SKIP")
    try:
        for flag in ("1", "0"):
            os.environ["PORSOL_BLOCK_SKIP"] = flag
            s = pkg.PressureSolver()
            opts = pkg.default_solve_opts(residual_tolerance=1e-11, precision=precision)
            out[flag] = s.upscale_periodic(union, union.cellpos, union.partner, union.side, K.ravel(), opts)
            s.close()
    finally:
        if old is None:
            os.environ.pop("PORSOL_BLOCK_SKIP", None)
        else:
            os.environ["PORSOL_BLOCK_SKIP"] = old
    (k1, st1), (k0, st0) = out["1"], out["0"]
    assert st1.iterations == st0.iterations
    assert np.array_equal(k1, k0)
