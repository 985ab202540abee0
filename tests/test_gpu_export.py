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


def _vtu_tree(path):
    """(element tags with their attributes in document order, arrays by name)."""
    root = ET.parse(path).getroot()
    elems = [(e.tag, tuple(sorted(e.attrib.items()))) for e in root.iter()]
    arrays = {a.get("Name", "points"): np.array(a.text.split(), float) for a in root.iter("DataArray")}
    return elems, arrays


def _compare_with_reference(ours, ref):
    """Same elements and attributes in the same order; integer arrays equal; floating
    values within the reference's 6 significant digits (ostream default precision)."""
    e1, a1 = _vtu_tree(ours)
    e2, a2 = _vtu_tree(ref)
    assert e1 == e2
    assert a1.keys() == a2.keys()
    for k in a2:
        assert a1[k].shape == a2[k].shape, k
        if k in ("connectivity", "offsets", "types"):
            assert np.array_equal(a1[k], a2[k]), k
        else:
            assert np.allclose(a1[k], a2[k], rtol=1e-5, atol=1e-6), k


def test_vtu_files_match_the_reference_writer(cuda, tmp_path):
    """pf2_export_vtu and pf2_export_particles_vtu against the files the reference's own
    DataExport::exportToVTK / exportParticlesToVTK (src/data_export.cu:17-171) wrote for
    the same mesh, fields and particles (tests/golden/reference_channel8x4.*.vtu, made by
    oracle/refhost/dump_ref_vtu.cu, which states the fields and particles)."""
    import os
    golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    xy, tri = mg.channel(8, 4, 4.0, 1.0)
    m = g.Mesh2D.from_arrays(xy, tri)
    x, y = xy[:, 0], xy[:, 1]
    fields = {"pressure": 1.0 - 0.3 * x + 0.2 * y * y, "velX": 1.25 * x, "velY": x * y - 0.5}
    path = tmp_path / "mesh.vtu"
    g.export_vtu(m, path, {k: torch.tensor(v, device="cuda") for k, v in fields.items()})
    _compare_with_reference(path, os.path.join(golden, "reference_channel8x4.mesh.vtu"))
    nc = tri.shape[0]
    k = np.tile(np.arange(4), nc)
    c = np.repeat(np.arange(nc), 4)
    w = np.stack([(k + 1.0) / (k + 6.0), 2.0 / (k + 6.0), 3.0 / (k + 6.0)], axis=1)
    pos = (w[:, :, None] * xy[tri[c]]).sum(axis=1)
    # the engine keeps l2 = 1 - l0 - l1 (the file holds positions and velocities only)
    P = {"x": pos[:, 0], "y": pos[:, 1], "l0": w[:, 0], "l1": w[:, 1], "l2": 1.0 - w[:, 0] - w[:, 1],
         "u": 0.5 * pos[:, 0], "v": 0.25 * pos[:, 1] - 1.0, "cell": c.astype(np.int32)}
    ph = g.ParticleHandler2D(m, 2)
    ph.upload(P)
    ppath = tmp_path / "particles.vtu"
    ph.export_vtu(ppath)
    _compare_with_reference(ppath, os.path.join(golden, "reference_channel8x4.particles.vtu"))
