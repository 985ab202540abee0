"""Mesh3D, SparseMatrixCSR(const Mesh3D&), the Poisson3D integrator, PCG on the 3D
system and the 3D VTU writer through the C ABI, against the oracle, the reference's
host-code fixtures and the exact solution of a sin-sin-sin problem."""
import hashlib
import json
import os
import re

import numpy as np
import pytest
import torch

import gpupfem2_gb300 as g
from gpupfem2_gb300 import meshgen as mg
from oracle import oracle as O
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = json.load(open(os.path.join(HERE, "golden", "reference_host.json")))
# FP64 geometry and assembly in another summation order than the oracle: rounding only
GEO_TOL = 1e-13
ASM_TOL = 1e-12


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name,make", [("box8x4x2", lambda: mg.box_tets(8, 4, 2)),
                                       ("box40x20x10", lambda: mg.box_tets())])
def test_dat_csr_match_reference_host_code(cuda, tmp_path, name, make):
    xyz, tet = make()
    p = os.path.join(tmp_path, name + ".dat")
    mg.write_dat3(p, xyz, tet)
    m = g.Mesh3D.load_dat(p)
    rp, col, _ = g.SparseMatrixCSR(m).download()
    rec = FIX["meshes3d"][name]
    assert (m.nv, m.nc) == (rec["nv"], rec["nc"])
    assert digest(m.download("xyz")) == rec["sha256_xyz"]
    assert digest(m.download("tet")) == rec["sha256_tet"]
    assert digest(rp) == rec["sha256_rowptr"] and digest(col) == rec["sha256_col"]


def test_geometry_and_neighbours_match_oracle(cuda):
    xyz, tet = mg.box_tets(12, 6, 4)
    m = g.Mesh3D.from_arrays(xyz, tet)
    vol, invJ = O.mesh3d_geometry(xyz, tet)
    assert rel_err(m.download("volume"), vol) < GEO_TOL
    assert rel_err(m.download("inv_jacobi"), invJ) < GEO_TOL
    off, idx = O.mesh3d_neighbors(tet)
    assert np.array_equal(m.download("neighbor_offsets"), off)
    assert np.array_equal(m.download("neighbor_indices"), idx)
    # inverse Jacobians: invJ . J = I per cell
    J = np.stack([xyz[tet[:, k]] - xyz[tet[:, 3]] for k in range(3)], axis=1)
    assert np.abs(np.einsum("cij,cjk->cik", m.download("inv_jacobi"), J) - np.eye(3)).max() < 1e-10


def test_neighbour_lists_off_and_bad_input(cuda):
    xyz, tet = mg.box_tets(4, 2, 2)
    m = g.Mesh3D.from_arrays(xyz, tet, fill_neighbors=False)
    assert m.n_neighbor_entries == 0 and not m.download("neighbor_offsets").any()
    bad = tet.copy()
    bad[3, 1] = bad[3, 0]
    with pytest.raises(g.Pf2Error) as e:
        g.Mesh3D.from_arrays(xyz, bad)
    assert e.value.status == g.BAD_INPUT
    bad = tet.copy()
    bad[0, 2] = xyz.shape[0]
    with pytest.raises(g.Pf2Error):
        g.Mesh3D.from_arrays(xyz, bad)


def _poisson(xyz, tet, kind, lam, bcs):
    m = g.Mesh3D.from_arrays(xyz, tet)
    A = g.SparseMatrixCSR(m)
    rhs = torch.zeros(m.nv, dtype=torch.float64, device="cuda")
    bc = g.DirichletBCs(m.nv, bcs) if bcs else None
    vol, invJ = O.mesh3d_geometry(xyz, tet)
    rp, col = O.csr_structure_3d(xyz.shape[0], tet)
    val, orhs = O.assemble_poisson_3d(xyz, tet, vol, invJ, rp, col, kind, lam)
    return m, A, rhs, bc, (rp, col, val, orhs)


@pytest.mark.parametrize("kind,lam", [(g.RHS3D_GAUSSIAN, 0.5), (g.RHS3D_SINSINSIN, 1.0)])
def test_assembly_matches_oracle(cuda, kind, lam):
    xyz, tet = mg.box_tets(12, 6, 4)
    m, A, rhs, _, (rp, col, val, orhs) = _poisson(xyz, tet, kind, lam, None)
    g.assemble_poisson_3d(m, A, rhs, kind, lam)
    grp, gcol, gval = A.download()
    assert np.array_equal(grp, rp) and np.array_equal(gcol, col)
    assert rel_err(gval, val) < ASM_TOL
    assert rel_err(rhs.cpu().numpy(), orhs) < ASM_TOL
    # reassembly overwrites (clearValues + assemble)
    g.assemble_poisson_3d(m, A, rhs, kind, lam)
    assert np.array_equal(A.download()[2], gval)


def test_poisson3d_case_solves_like_the_oracle(cuda):
    """The Poisson3D driver (cases/Poisson3D/main.cu:86-176) on a generated box: the
    reference's boundary values, lambda 0.5, Jacobi-PCG to 1e-8 (absolute), 1000
    iterations at most."""
    xyz, tet = mg.box_tets(20, 10, 6)
    bcs = mg.box_boundary_nodes(xyz)
    m, A, rhs, bc, (rp, col, val, orhs) = _poisson(xyz, tet, g.RHS3D_GAUSSIAN, 0.5, bcs)
    g.assemble_poisson_3d(m, A, rhs, g.RHS3D_GAUSSIAN, 0.5, bc)
    bn = np.array([b for b, _ in bcs], np.int32)
    bv = np.array([v for _, v in bcs])
    oval, orhs2 = O.apply_bcs(rp, col, val, orhs, bn, bv)
    assert rel_err(A.download()[2], oval) < ASM_TOL and rel_err(rhs.cpu().numpy(), orhs2) < ASM_TOL
    x = torch.zeros(m.nv, dtype=torch.float64, device="cuda")
    info = g.LinearSolver(A, "cg", "jacobi", tol=1e-8, maxit=1000).solve(A, x, rhs)
    assert info.converged == 1
    ox, oinfo = O.pcg(rp, col, oval, orhs2, tol=1e-8, maxit=1000, precond="jacobi")
    assert abs(info.iterations - oinfo.iterations) <= 2
    assert rel_err(x.cpu().numpy(), ox) < 1e-6
    xs = x.cpu().numpy()
    assert np.allclose(xs[bn], bv)  # boundary rows stay identities
    assert xs.min() >= bv.min() - 1e-6 and xs.max() <= bv.max() + 1e-6  # the boundary values bound it here


@pytest.mark.parametrize("precond", ["jacobi", "ic"])
def test_sinsinsin_converges_to_the_exact_solution(cuda, precond):
    errs = []
    for n in (8, 16):
        xyz, tet = mg.box_tets(n, n, n, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), jitter=0.1)
        bcs = mg.cube_boundary_nodes(xyz)
        m, A, rhs, bc, _ = _poisson(xyz, tet, g.RHS3D_SINSINSIN, 1.0, bcs)
        g.assemble_poisson_3d(m, A, rhs, g.RHS3D_SINSINSIN, 1.0, bc)
        x = torch.zeros(m.nv, dtype=torch.float64, device="cuda")
        info = g.LinearSolver(A, "cg", precond, tol=1e-10, maxit=3000, criterion=g.CRITERION_REL).solve(A, x, rhs)
        assert info.converged == 1
        exact = np.sin(np.pi * xyz[:, 0]) * np.sin(np.pi * xyz[:, 1]) * np.sin(np.pi * xyz[:, 2])
        errs.append(np.abs(x.cpu().numpy() - exact).max())
    assert errs[0] < 0.1 and errs[1] < 0.35 * errs[0]  # second order in h


def test_vtu_3d_layout(cuda, tmp_path):
    xyz, tet = mg.box_tets(3, 2, 2, lo=(0.0, 0.0, 0.0), hi=(3.0, 2.0, 2.0), jitter=0.0)
    m = g.Mesh3D.from_arrays(xyz, tet)
    f = torch.tensor(xyz[:, 0] + 2 * xyz[:, 2], device="cuda")
    path = tmp_path / "box.vtu"
    g.export_vtu(m, path, {"solution": f})
    text = path.read_text()
    assert 'NumberOfPoints="%d" NumberOfCells="%d"' % (m.nv, m.nc) in text
    types = re.search(r'Name="types" Format="ascii">\s*([^<]*)<', text).group(1).split()
    assert types == ["10"] * m.nc
    conn = np.array(re.search(r'Name="connectivity" Format="ascii">\s*([^<]*)<', text).group(1).split(), int)
    assert np.array_equal(conn.reshape(-1, 4), tet)
    pts = np.array(re.search(r'NumberOfComponents="3" Format="ascii">\s*([^<]*)<', text).group(1).split(), float)
    assert np.array_equal(pts.reshape(-1, 3), xyz)  # integer coordinates: exact in %.9g
    sol = np.array(re.search(r'Name="solution" Format="ascii">\s*([^<]*)<', text).group(1).split(), float)
    assert np.abs(sol - f.cpu().numpy()).max() < 1e-7
