"""pf2_pcg_jacobi_static: Jacobi-PCG with its work vectors in a fixed device array of the
library, checked against the allocating solver (pf2_solver_create + pf2_solver_solve)."""
import ctypes as C

import numpy as np
import pytest
import torch

import gpupfem2_gb300 as g
from gpupfem2_gb300 import meshgen as mg
from oracle import oracle as O
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

MAX_ROWS = 131072  # PF2_STATIC_MAX_ROWS


def _static(A, x, b, tol, maxit, criterion):
    L = g.lib()
    f = L.pf2_pcg_jacobi_static
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    info = g.SolveInfo()
    st = f(A.h, g._dev(x), g._dev(b), tol, maxit, criterion, C.byref(info), g._stream())
    return st, info


def _system(nx, ny):
    xy, tri = mg.channel(nx, ny, 4.0, 1.0)
    m = g.Mesh2D.from_arrays(xy, tri)
    A = g.SparseMatrixCSR(m)
    area, invJ = O.mesh_geometry(xy, tri)
    rp, col = O.csr_structure(xy.shape[0], tri)
    val, rhs = O.assemble_poisson(xy, tri, area, invJ, rp, col, 1, 1.0)
    diag = np.array([rp[i] + np.searchsorted(col[rp[i]:rp[i + 1]], i) for i in range(rp.size - 1)])
    val[diag] += 1e-2
    A.upload_values(val)
    return m, A, rp, col, val, rhs


@pytest.mark.parametrize("criterion", [g.CRITERION_ABS, g.CRITERION_REL])
def test_static_pcg_matches_allocating_solver_twice(cuda, monkeypatch, criterion):
    """The static entry point runs k_pcg, the allocating solver's kernel when the
    partitioned kernel is off (PF2_CG_PART=0): the same bits; the partitioned kernel (the
    allocating solver's default) sums its reductions in another order and agrees to the
    solve's tolerance."""
    m, A, rp, col, val, rhs = _system(128, 32)
    b = torch.tensor(rhs, device="cuda")
    x_part = torch.zeros_like(b)
    part = g.LinearSolver(A, "cg", "jacobi", tol=1e-8, maxit=5000, criterion=criterion).solve(A, x_part, b)
    monkeypatch.setenv("PF2_CG_PART", "0")
    x_ref = torch.zeros_like(b)
    ref = g.LinearSolver(A, "cg", "jacobi", tol=1e-8, maxit=5000, criterion=criterion).solve(A, x_ref, b)
    assert ref.converged == 1 and part.converged == 1 and abs(part.iterations - ref.iterations) <= 2
    assert rel_err(x_part.cpu().numpy(), x_ref.cpu().numpy()) < 1e-6
    free = []
    xs = [torch.zeros_like(b) for _ in range(3)]  # torch's allocations come before the calls
    for x in xs:  # calls in a row reuse the same storage
        torch.cuda.synchronize()
        st, info = _static(A, x, b, 1e-8, 5000, criterion)
        assert st == g.OK and info.converged == 1 and info.status == 0
        assert info.iterations == ref.iterations
        # same kernel, same block partition, same summation order: the same bits
        assert torch.equal(x, x_ref)
        free.append(torch.cuda.mem_get_info()[0])
    # nothing is allocated per call: the device's free memory (2 MB granularity, enough
    # to see a new cudaMalloc of the 5.3 MB work) stays where the first call left it
    assert free[1] == free[0] and free[2] == free[0]
    ox, oinfo = O.pcg(rp, col, val, rhs, tol=1e-8, maxit=5000, precond="jacobi")
    if criterion == g.CRITERION_ABS:
        assert abs(info.iterations - oinfo.iterations) <= 2
    assert rel_err(x.cpu().numpy(), ox) < 1e-6


def test_static_pcg_rejects_systems_beyond_its_storage(cuda):
    m, A, rp, col, val, rhs = _system(512, 256)  # 131,841 rows
    assert A.rows > MAX_ROWS
    b = torch.tensor(rhs, device="cuda")
    x = torch.zeros_like(b)
    st, _ = _static(A, x, b, 1e-8, 10, g.CRITERION_ABS)
    assert st == g.BAD_INPUT
    L = g.lib()
    L.pf2_last_error.restype = C.c_char_p
    assert b"static work storage" in L.pf2_last_error()
