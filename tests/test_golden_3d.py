"""The 3D path against fixtures produced by the reference's own host code
(tests/golden/reference_host.json, made by make_reference_fixtures.py): the DAT reader of
Mesh3D, the CSR pattern of SparseMatrixCSR(const Mesh3D&) and the 6-point quadrature
rule, bit for bit; the oracle's face-sharing neighbour lists against their definition."""
import hashlib
import json
import os

import numpy as np
import pytest

from gpupfem2_gb300 import meshgen as mg
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = json.load(open(os.path.join(HERE, "golden", "reference_host.json")))
GENERATED = {"box8x4x2": lambda: mg.box_tets(8, 4, 2), "box40x20x10": lambda: mg.box_tets()}
SHIPPED = {"BoxMesh.dat": "Poisson3D", "BoxMesh2.dat": "Poisson3D"}
SHIPPED_DIR = os.path.join(os.environ.get("PF2_REFERENCE_DIR", "/root/reference"), "cases")


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def oracle_arrays(xyz, tet):
    rp, col = O.csr_structure_3d(xyz.shape[0], tet)
    return {"xyz": xyz, "tet": tet.astype(np.int32), "rowptr": rp, "col": col}


def check(rec, arrays):
    for k, v in arrays.items():
        assert digest(v) == rec["sha256_" + k], k


@pytest.mark.parametrize("name", list(GENERATED))
def test_oracle_matches_reference_host_code_on_generated_meshes(name, tmp_path):
    xyz, tet = GENERATED[name]()
    # through the DAT format the reference reads
    p = os.path.join(tmp_path, name + ".dat")
    mg.write_dat3(p, xyz, tet)
    xyz2, tet2 = mg.read_dat3(p)
    assert np.array_equal(xyz2, xyz) and np.array_equal(tet2, tet)
    check(FIX["meshes3d"][name], oracle_arrays(xyz, tet))


@pytest.mark.parametrize("name", list(SHIPPED))
def test_oracle_matches_reference_host_code_on_shipped_meshes(name):
    path = os.path.join(SHIPPED_DIR, SHIPPED[name], name)
    if not os.path.exists(path):
        pytest.skip("the reference's meshes are only present where the reference tree is mounted")
    xyz, tet = mg.read_dat3(path)
    check(FIX["meshes3d"][name], oracle_arrays(xyz, tet))


def test_cell_quadrature_matches_reference():
    ref = np.array([float.fromhex(v) for v in FIX["quadrature3d"]["cell_index1_xyzw_weight"]]).reshape(-1, 5)
    c, w = O.cell_quadrature_3d()
    assert np.array_equal(c, ref[:, :4]) and np.array_equal(w, ref[:, 4])
    assert abs(w.sum() - 1.0) < 1e-12


def test_oracle_neighbours_share_faces():
    xyz, tet = mg.box_tets(6, 3, 2)
    off, idx = O.mesh3d_neighbors(tet)
    sets = [set(t) for t in tet.tolist()]
    for c in range(tet.shape[0]):
        lst = idx[off[c]:off[c + 1]].tolist()
        assert lst == sorted(lst) and c not in lst
        want = [d for d in range(tet.shape[0]) if d != c and len(sets[c] & sets[d]) == 3]
        assert lst == want
    # every interior face is shared by exactly two cells: 4 nc = 2 interior + boundary
    n_boundary_faces = 2 * (6 * 3 + 6 * 2 + 3 * 2) * 2
    assert idx.size == 4 * tet.shape[0] - n_boundary_faces


def test_oracle_poisson3d_matrix_properties():
    xyz, tet = mg.box_tets(6, 4, 3)
    vol, invJ = O.mesh3d_geometry(xyz, tet)
    assert abs(vol.sum() - 1.0) < 1e-12  # the [-1,1] x [0,1] x [-0.25,0.25] box
    rp, col = O.csr_structure_3d(xyz.shape[0], tet)
    val, rhs = O.assemble_poisson_3d(xyz, tet, vol, invJ, rp, col, rhs_kind=0, lam=0.5)
    rowsum = np.add.reduceat(val, rp[:-1])
    assert np.abs(rowsum).max() < 1e-13  # gradients of a partition of unity
    dense = np.zeros((rp.size - 1,) * 2)
    for i in range(rp.size - 1):
        dense[i, col[rp[i]:rp[i + 1]]] = val[rp[i]:rp[i + 1]]
    assert np.abs(dense - dense.T).max() < 1e-15
    # a linear field has zero energy only along constants: x^T A x for x = x-coordinate
    x = xyz[:, 0]
    assert abs(x @ dense @ x - 0.5 * vol.sum()) < 1e-12  # lambda |grad x|^2 |box|
