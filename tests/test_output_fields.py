"""Output fields (SimulatorUtilities.hpp): the numpy restatement on an analytic flux field,
the GPU kernel against it, and writeField's file format."""
import numpy as np
import pytest

from parity import gpu_solve


def test_restated_velocity_is_exact_for_uniform_flow(orc, cart):
    """For a uniform Darcy velocity u the face fluxes are u.n A and the cell estimate is u."""
    g = cart.CartesianGrid(5, 4, 3, dx=0.3, dy=0.5, dz=0.2)
    u = np.array([1.5, -0.25, 0.75])
    flux = (g.fnormal @ u) * g.area
    vel = orc.cell_fields(g, flux)["velocity"]
    assert np.abs(vel - u).max() < 1e-13


def test_write_field_format(pkg, tmp_path):
    """Count line then %g values, the default-ostream output of the reference."""
    if not __import__("os").path.exists(pkg.LIB_PATH):
        pytest.skip("library not built")
    f = tmp_path / "field.dat"
    pkg.write_field([1.0, 0.1234567891, -2.5e-7, 1e20], f)
    assert f.read_text() == "4\n1\n0.123457\n-2.5e-07\n1e+20\n"


@pytest.mark.gpu
def test_cell_fields_match_restatement(pkg, gpulib, orc, workloads):
    prob = workloads.anisotropic_corey(dims=(12, 10, 6))
    r = gpu_solve(pkg, prob, ltype=1, tol=1e-12, post=True)
    s = r["solver"]
    _, mu1, mu2, r1, r2 = prob.fluid
    fl = pkg.Fluid(pkg.FLUID_COREY2, mu1, mu2, r1, r2)
    got = s.cell_fields(fl, prob.sat)
    ref = orc.cell_fields(prob.grid, r["v"], prob.sat, mu1, mu2)
    for k in ref:
        scale = max(np.abs(ref[k]).max(), 1e-300)
        assert np.abs(got[k] - ref[k]).max() <= 1e-12 * scale, k
    assert set(s.cell_fields().keys()) == {"velocity"}
