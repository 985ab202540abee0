"""Mesh2D on the GPU against the oracle: pattern, neighbour lists and geometry bit for bit."""
import os

import numpy as np
import pytest

import gpupfem2_gb300 as g
from gpupfem2_gb300 import meshgen as mg
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = {"square64": lambda: mg.unit_square(64), "channel": lambda: mg.channel(),
         "cyl_small": lambda: mg.cylinder_channel(nxh=100, nyh=100, nr=6)}


@pytest.mark.parametrize("case", list(CASES))
def test_mesh_arrays_match_oracle_bitwise(cuda, case):
    xy, tri = CASES[case]()
    m = g.Mesh2D.from_arrays(xy, tri)
    area, invJ = O.mesh_geometry(xy, tri)
    assert np.array_equal(m.download("area"), area)
    assert np.array_equal(m.download("inv_jacobi"), invJ)
    off, idx = O.neighbors(xy.shape[0], tri)
    assert np.array_equal(m.download("neighbor_offsets"), off)
    assert np.array_equal(m.download("neighbor_indices"), idx)
    rp, col = O.csr_structure(xy.shape[0], tri)
    A = g.SparseMatrixCSR(m)
    grp, gcol, gval = A.download()
    assert np.array_equal(grp, rp) and np.array_equal(gcol, col)
    assert not gval.any()


def test_edge_boundary_ids(cuda):
    xy, tri = mg.cylinder_channel(nxh=100, nyh=100, nr=6)
    m = g.Mesh2D.from_arrays(xy, tri)
    m.set_channel_boundary_ids(2.2, 0.41, (0.2, 0.2, 0.05))
    ids = m.download("edge_ids")
    ref = O.edge_boundary_ids(xy, tri, 2.2, 0.41, (0.2, 0.2, 0.05))
    assert np.array_equal(ids, ref)
    # one body edge per O-grid ray: the box [0.1, 0.3]^2 has 20 + 20 + 20 + 20 perimeter nodes at h = 0.01
    assert (ids == 3).sum() == 80 and (ids == 1).sum() > 0


def test_load_dat_equals_arrays(cuda, tmp_path):
    xy, tri = mg.channel(32, 8)
    p = os.path.join(tmp_path, "c.dat")
    mg.write_dat(p, xy, tri)
    a = g.Mesh2D.load_dat(p)
    b = g.Mesh2D.from_arrays(xy, tri)
    for f in ("xy", "tri", "inv_jacobi", "neighbor_indices"):
        assert np.array_equal(a.download(f), b.download(f))


def test_bad_meshes_are_rejected(cuda, tmp_path):
    xy, tri = mg.unit_square(4)
    bad = tri.copy()
    bad[3, 1] = xy.shape[0] + 5
    with pytest.raises(g.Pf2Error) as e:
        g.Mesh2D.from_arrays(xy, bad)
    assert e.value.status == g.BAD_INPUT
    p = os.path.join(tmp_path, "t.dat")
    open(p, "w").write("4 2\n1 0 0 0\n2 1 0 0\n")
    with pytest.raises(g.Pf2Error) as e:
        g.Mesh2D.load_dat(p)
    assert e.value.status == g.IO_ERROR
    with pytest.raises(g.Pf2Error):
        g.Mesh2D.load_dat(os.path.join(tmp_path, "missing.dat"))
