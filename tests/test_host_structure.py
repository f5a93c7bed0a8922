"""The host-side structure build (face numbering, sparsity, SELL layout, assembly recipe) runs on
all host cores; on the CPU alone it must reproduce the oracle's serial numbering and sparsity
exactly (IncompFlowSolverHybrid.hpp:956-1319) and keep the recipe's serial write order, for grids
large enough that every pass is split across threads."""
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "opm-porsol_gb300", "csrc")


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("st") / "structure_test")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["g++", "-O2", "-std=c++17", "-pthread", "-I", os.path.join(ROOT, "include"), "-I", CSRC,
           "-I", os.path.join(cuda, "include"), os.path.join(HERE, "cpp", "structure_test.cpp"),
           os.path.join(CSRC, "structure.cpp"), "-o", out, "-L", os.path.join(cuda, "lib64"), "-lcudart",
           f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _run(exe, tmp_path, g, bct, pb, centroids=False, internal=None):
    a = g.arrays()
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(inp, "wb") as f:
        np.array([a["num_cells"], g.num_half_faces], np.int64).tofile(f)
        for x in (a["facepos"], a["neighbour"], a["bid"], bct, pb):
            np.ascontiguousarray(x, np.int32).tofile(f)
        if centroids:
            np.ascontiguousarray(g.ccentroid, np.float64).tofile(f)
    r = subprocess.run([exe, inp, outp], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr
    v = np.fromfile(outp, np.int32)
    N, nint = int(v[0]), int(v[1])
    o = 2
    cf = v[o:o + g.num_half_faces]; o += g.num_half_faces
    rp = v[o:o + N + 1]; o += N + 1
    ci = v[o:o + rp[-1]]; o += rp[-1]
    pp = v[o:o + N]; o += N
    if internal is not None:
        internal.update(renumbered=bool(v[o]), bandwidth=int(v[o + 1]), bandwidth_ref=int(v[o + 2]),
                        perm=v[o + 3:o + 3 + N].copy())
    return cf, rp, ci, pp


@pytest.mark.parametrize("periodic", [False, True])
def test_host_structure_matches_oracle(exe, tmp_path, orc, cart, workloads, periodic):
    g = cart.CartesianGrid(60, 50, 40, unique_bids=True)   # 120k cells, 720k half-faces
    bct, _ = workloads.x_dirichlet_bc(g)
    pb = np.zeros(g.num_half_faces, np.int32)
    if periodic:
        ybnd = (g.side == 3) | (g.side == 4)
        bct[ybnd] = workloads.BC_PERIODIC
        pb = np.where(ybnd, g.periodic_partner_bids(), 0).astype(np.int32)
    mine = _run(exe, tmp_path, g, bct, pb)
    o = orc.OraclePressure(g, bct, pb if periodic else None)
    ref = o.structure()
    for a, b, name in zip(mine, ref, ("cellfaces", "rowptr", "colind", "ppartner")):
        assert np.array_equal(a, b), name
    # the same build again: no dependence on thread timing
    again = _run(exe, tmp_path, g, bct, pb)
    for a, b in zip(mine, again):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("order", ["lattice", "rcm"])
def test_internal_numbering(exe, tmp_path, cart, workloads, order):
    """The device system's internal face numbering: a permutation of the reference numbering with a
    smaller bandwidth (structure_test checks that every coupling sits at its permuted row and
    column).  Cartesian cell centroids give the lattice order (axis of fewest cells fastest: about
    3 * ny * nz faces for 60 x 50 x 40); without centroids the reverse Cuthill-McKee order.  Grids
    with periodic faces keep the reference numbering."""
    g = cart.CartesianGrid(60, 50, 40, unique_bids=True)
    bct, _ = workloads.x_dirichlet_bc(g)
    pb = np.zeros(g.num_half_faces, np.int32)
    info = {}
    cf, rp, ci, pp = _run(exe, tmp_path, g, bct, pb, centroids=(order == "lattice"), internal=info)
    assert info["renumbered"] and info["bandwidth"] < info["bandwidth_ref"]
    assert np.array_equal(np.sort(info["perm"]), np.arange(len(info["perm"])))
    if order == "lattice":
        assert info["bandwidth"] <= 2 * 3 * 50 * 40, info
    assert info["bandwidth"] < 32768   # fits 16-bit column offsets
    ybnd = (g.side == 3) | (g.side == 4)
    bct2 = bct.copy()
    bct2[ybnd] = workloads.BC_PERIODIC
    pb2 = np.where(ybnd, g.periodic_partner_bids(), 0).astype(np.int32)
    info2 = {}
    _run(exe, tmp_path, g, bct2, pb2, centroids=True, internal=info2)
    assert not info2["renumbered"]
