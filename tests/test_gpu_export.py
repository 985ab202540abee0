"""VTU output (DataExport, src/data_export.cu): the written file parses as VTK XML and
holds the mesh, the fields and the particles."""
import xml.etree.ElementTree as ET

import numpy as np
import pytest
import torch

import gpupfem2_gb300 as g
from gpupfem2_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


def _arrays(path):
    root = ET.parse(path).getroot()
    piece = root.find("UnstructuredGrid/Piece")
    out = {a.get("Name", "points"): np.array(a.text.split(), float) for a in piece.iter("DataArray")}
    return piece, out


def test_mesh_fields_vtu(cuda, tmp_path):
    xy, tri = mg.channel(8, 4, 4.0, 1.0)
    m = g.Mesh2D.from_arrays(xy, tri)
    ux = torch.tensor(xy[:, 0] * 1.25, device="cuda")
    p = torch.tensor(xy[:, 1] - 0.5, device="cuda")
    path = tmp_path / "mesh.vtu"
    g.export_vtu(m, path, {"u": ux, "p": p})
    piece, a = _arrays(path)
    assert int(piece.get("NumberOfPoints")) == xy.shape[0] and int(piece.get("NumberOfCells")) == tri.shape[0]
    assert np.allclose(a["points"].reshape(-1, 3)[:, :2], xy, rtol=1e-7, atol=1e-7)
    assert np.array_equal(a["connectivity"].reshape(-1, 3).astype(int), tri)
    assert np.array_equal(a["offsets"].astype(int), 3 * np.arange(1, tri.shape[0] + 1))
    assert set(a["types"].astype(int)) == {5}
    assert np.allclose(a["u"], xy[:, 0] * 1.25, rtol=1e-7) and np.allclose(a["p"], xy[:, 1] - 0.5, atol=1e-7)


def test_particles_vtu(cuda, tmp_path):
    xy, tri = mg.channel(8, 4, 4.0, 1.0)
    m = g.Mesh2D.from_arrays(xy, tri)
    ph = g.ParticleHandler2D(m, 2)
    ph.seed()
    path = tmp_path / "particles.vtu"
    ph.export_vtu(path)
    piece, a = _arrays(path)
    P = ph.download()
    n = P["x"].size
    assert int(piece.get("NumberOfPoints")) == n == tri.shape[0] * 4
    pts = a["points"].reshape(-1, 3)
    assert np.allclose(pts[:, 0], P["x"], rtol=1e-7) and np.allclose(pts[:, 1], P["y"], rtol=1e-7)
    assert np.array_equal(a["connectivity"].astype(int), np.arange(n))
