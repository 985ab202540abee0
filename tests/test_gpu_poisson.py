"""2D Poisson on the unit square (64 x 64 quads): assembly, Dirichlet rule and PCG
through the C ABI against the oracle and the exact solution sin(pi x) sin(pi y)."""
import numpy as np
import pytest
import torch

import gpupfem2_gb300 as g
from oracle import oracle as O
from tests.helpers import poisson_square, rel_err

pytestmark = pytest.mark.gpu

# FP64 assembly in closed form vs the oracle's quadrature loop: rounding only
ASM_TOL = 1e-12


def _setup(n=64, kind=g.RHS_SINSIN, lam=1.0):
    xy, tri, bcs = poisson_square(n)
    m = g.Mesh2D.from_arrays(xy, tri)
    A = g.SparseMatrixCSR(m)
    rhs = torch.zeros(m.nv, dtype=torch.float64, device="cuda")
    bc = g.DirichletBCs(m.nv, bcs)
    area, invJ = O.mesh_geometry(xy, tri)
    rp, col = O.csr_structure(xy.shape[0], tri)
    val, orhs = O.assemble_poisson(xy, tri, area, invJ, rp, col, kind, lam)
    bn = np.array([b for b, _ in bcs], np.int32)
    bv = np.array([v for _, v in bcs])
    return xy, m, A, rhs, bc, (rp, col, val, orhs, bn, bv)


@pytest.mark.parametrize("kind,lam", [(g.RHS_SINSIN, 1.0), (g.RHS_GAUSSIAN, 0.5)])
def test_assembly_matches_oracle(cuda, kind, lam):
    xy, m, A, rhs, bc, (rp, col, val, orhs, bn, bv) = _setup(kind=kind, lam=lam)
    g.assemble_poisson(m, A, rhs, kind, lam)
    _, _, gval = A.download()
    assert rel_err(gval, val) < ASM_TOL
    assert rel_err(rhs.cpu().numpy(), orhs) < ASM_TOL


def test_fused_bc_equals_separate_apply_and_oracle(cuda):
    xy, m, A, rhs, bc, (rp, col, val, orhs, bn, bv) = _setup()
    g.assemble_poisson(m, A, rhs, g.RHS_SINSIN, 1.0, bc)
    fused_v, fused_r = A.download()[2], rhs.cpu().numpy()
    g.assemble_poisson(m, A, rhs, g.RHS_SINSIN, 1.0)
    bc.apply(A, rhs)
    sep_v, sep_r = A.download()[2], rhs.cpu().numpy()
    assert np.array_equal(fused_v, sep_v) and np.array_equal(fused_r, sep_r)
    oval, orhs2 = O.apply_bcs(rp, col, val, orhs, bn, bv)
    assert rel_err(fused_v, oval) < ASM_TOL and rel_err(fused_r, orhs2) < ASM_TOL


def test_pcg_jacobi_against_exact_and_oracle(cuda):
    xy, m, A, rhs, bc, (rp, col, val, orhs, bn, bv) = _setup()
    g.assemble_poisson(m, A, rhs, g.RHS_SINSIN, 1.0, bc)
    x = torch.zeros(m.nv, dtype=torch.float64, device="cuda")
    s = g.LinearSolver(A, "cg", "jacobi", tol=1e-10, maxit=2000, criterion=g.CRITERION_REL)
    info = s.solve(A, x, rhs)
    assert info.converged == 1 and info.residual <= 1e-10
    exact = np.sin(np.pi * xy[:, 0]) * np.sin(np.pi * xy[:, 1])
    xs = x.cpu().numpy()
    assert np.abs(xs - exact).max() < 3e-4  # O(h^2) discretisation error at h = 1/64
    oval, orhs2 = O.apply_bcs(rp, col, val, orhs, bn, bv)
    ox, oinfo = O.pcg(rp, col, oval, orhs2, tol=1e-12, maxit=4000, precond="jacobi")
    # both are 1e-10-relative-residual solutions of the same system
    assert rel_err(xs, ox) < 1e-8
    # a repeated solve from the same start gives identical bits (fixed-order reductions)
    x2 = torch.zeros_like(x)
    s.solve(A, x2, rhs)
    assert torch.equal(x, x2)


def test_absolute_criterion_iterations_match_oracle(cuda):
    xy, m, A, rhs, bc, (rp, col, val, orhs, bn, bv) = _setup()
    g.assemble_poisson(m, A, rhs, g.RHS_SINSIN, 1.0, bc)
    x = torch.zeros(m.nv, dtype=torch.float64, device="cuda")
    info = g.LinearSolver(A, "cg", "jacobi", tol=1e-8, maxit=1000).solve(A, x, rhs)
    oval, orhs2 = O.apply_bcs(rp, col, val, orhs, bn, bv)
    ox, oinfo = O.pcg(rp, col, oval, orhs2, tol=1e-8, maxit=1000, precond="jacobi")
    assert info.converged and abs(info.iterations - oinfo.iterations) <= 1
    assert rel_err(x.cpu().numpy(), ox) < 1e-6


def test_not_converged_is_reported(cuda):
    xy, m, A, rhs, bc, _ = _setup()
    g.assemble_poisson(m, A, rhs, g.RHS_SINSIN, 1.0, bc)
    x = torch.zeros(m.nv, dtype=torch.float64, device="cuda")
    info = g.LinearSolver(A, "cg", "jacobi", tol=1e-12, maxit=3).solve(A, x, rhs)
    assert info.converged == 0 and info.iterations == 3
