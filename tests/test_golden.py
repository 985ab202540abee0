"""The oracle (CPU) and the engine (GPU) against fixtures produced by the reference's own
host code (tests/golden/reference_host.json, made by make_reference_fixtures.py):
DAT parsing, vertex-sharing neighbour lists, CSR pattern, sub-cell centroids and
quadrature tables, bit for bit."""
import hashlib
import json
import os

import numpy as np
import pytest

from gpupfem2_gb300 import meshgen as mg
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = json.load(open(os.path.join(HERE, "golden", "reference_host.json")))
GENERATED = {
    "square64": lambda: mg.unit_square(64),
    "channel256x64": lambda: mg.channel(),
    "channel64x16": lambda: mg.channel(64, 16, 4.0, 1.0),
    "cylinder_nx100": lambda: mg.cylinder_channel(nxh=100, nyh=100, nr=6),
}
SHIPPED_DIR = os.path.join(os.environ.get("PF2_REFERENCE_DIR", "/root/reference"), "cases")
SHIPPED = {"TestProblem2.dat": "Poisson2D", "ChannelMesh.dat": "PoiseuilleFlow2D",
           "CylinderMesh.dat": "Cylinder2D", "CylinderMesh3.dat": "Cylinder2D"}


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def oracle_arrays(xy, tri):
    off, idx = O.neighbors(xy.shape[0], tri)
    rp, col = O.csr_structure(xy.shape[0], tri)
    return {"xy": xy, "tri": tri.astype(np.int32), "nboff": off, "nbidx": idx, "rowptr": rp, "col": col}


def check(rec, arrays):
    for k, v in arrays.items():
        assert digest(v) == rec["sha256_" + k], k


@pytest.mark.parametrize("name", list(GENERATED))
def test_oracle_matches_reference_host_code_on_generated_meshes(name):
    xy, tri = GENERATED[name]()
    check(FIX["meshes"][name], oracle_arrays(xy, tri))


@pytest.mark.parametrize("name", list(SHIPPED))
def test_oracle_matches_reference_host_code_on_shipped_meshes(name):
    path = os.path.join(SHIPPED_DIR, SHIPPED[name], name)
    if not os.path.exists(path):
        pytest.skip("the reference's meshes are only present where the reference tree is mounted")
    xy, tri = mg.read_dat(path)
    check(FIX["meshes"][name], oracle_arrays(xy, tri))


@pytest.mark.parametrize("level", [1, 2, 3, 4])
def test_subcell_centres_match_reference(level):
    ref = np.array([float.fromhex(v) for v in FIX["subcell_centers"][str(level)]]).reshape(-1, 3)
    assert np.array_equal(O.subcell_centers(level), ref)


def test_quadrature_tables_match_reference():
    c3, w = np.zeros(9), np.zeros(3)
    O.lib().or_face_quadrature.argtypes = [O.C.c_int, O.C.c_void_p, O.C.c_void_p]
    O.lib().or_face_quadrature(1, c3.ctypes.data_as(O.C.c_void_p), w.ctypes.data_as(O.C.c_void_p))
    ref = np.array([float.fromhex(v) for v in FIX["quadrature"]["face_index1_xyzw"]]).reshape(3, 4)
    assert np.array_equal(c3.reshape(3, 3), ref[:, :3]) and np.array_equal(w, ref[:, 3])


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(GENERATED))
def test_engine_matches_reference_host_code(cuda, name, tmp_path):
    import gpupfem2_gb300 as g
    xy, tri = GENERATED[name]()
    p = os.path.join(tmp_path, name + ".dat")
    mg.write_dat(p, xy, tri)
    m = g.Mesh2D.load_dat(p)
    A = g.SparseMatrixCSR(m)
    rp, col, _ = A.download()
    arrays = {"xy": m.download("xy"), "tri": m.download("tri"), "nboff": m.download("neighbor_offsets"),
              "nbidx": m.download("neighbor_indices"), "rowptr": rp, "col": col}
    check(FIX["meshes"][name], arrays)


def test_reference_vtu_fixtures_parse():
    """The committed output of the reference's VTU writers: well-formed VTK XML with the
    mesh of the 8 x 4 channel and four particles per cell."""
    import xml.etree.ElementTree as ET
    here = os.path.dirname(os.path.abspath(__file__))
    xy, tri = mg.channel(8, 4, 4.0, 1.0)
    for part, npts, ncells in (("mesh", xy.shape[0], tri.shape[0]), ("particles", 4 * tri.shape[0],
                                                                     4 * tri.shape[0])):
        root = ET.parse(os.path.join(here, "golden", "reference_channel8x4.%s.vtu" % part)).getroot()
        piece = root.find("UnstructuredGrid/Piece")
        assert int(piece.get("NumberOfPoints")) == npts and int(piece.get("NumberOfCells")) == ncells
    root = ET.parse(os.path.join(here, "golden", "reference_channel8x4.mesh.vtu")).getroot()
    conn = [a for a in root.iter("DataArray") if a.get("Name") == "connectivity"][0]
    assert np.array_equal(np.array(conn.text.split(), int).reshape(-1, 3), tri)
