"""CG / GMRES with Jacobi, ILU(0), IC(0) on a jittered-channel SPD system against the oracle."""
import ctypes as C

import numpy as np
import pytest
import torch

import gpupfem2_gb300 as g
from gpupfem2_gb300 import meshgen as mg
from oracle import oracle as O
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu


def _system(nx=64, ny=16):
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


@pytest.mark.parametrize("kind,pc", [("cg", "none"), ("cg", "jacobi"), ("cg", "ilu"), ("cg", "ic"),
                                     ("gmres", "jacobi"), ("gmres", "ilu"), ("gmres", "none")])
def test_solver_matches_oracle(cuda, kind, pc):
    m, A, rp, col, val, rhs = _system()
    b = torch.tensor(rhs, device="cuda")
    x = torch.zeros_like(b)
    s = g.LinearSolver(A, kind, pc, tol=1e-8, maxit=1000)
    info = s.solve(A, x, b)
    fn = O.pcg if kind == "cg" else O.gmres
    ox, oinfo = fn(rp, col, val, rhs, tol=1e-8, maxit=1000, precond=pc)
    assert info.converged == 1 and oinfo.converged == 1
    assert abs(info.iterations - oinfo.iterations) <= 2
    # both stop at an absolute 1e-8 criterion; the solutions agree to the solve tolerance
    assert rel_err(x.cpu().numpy(), ox) < 1e-6


@pytest.mark.parametrize("pc", ["ilu", "ic"])
def test_preconditioner_apply_matches_oracle(cuda, pc):
    m, A, rp, col, val, rhs = _system(32, 8)
    s = g.LinearSolver(A, "cg", pc)
    s.setup(A)
    src = torch.tensor(rhs, device="cuda")
    dst = torch.empty_like(src)
    s.apply_preconditioner(dst, src)
    f = O.ilu0(rp, col, val) if pc == "ilu" else O.ic0(rp, col, val)
    ref = np.empty_like(rhs)
    tmp = np.empty_like(rhs)
    src_h = np.ascontiguousarray(rhs)
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    O.lib().or_precond_apply.argtypes = [C.c_int, C.c_int] + [C.c_void_p] * 7
    O.lib().or_precond_apply(O.PRECOND[pc], rp.size - 1, p(rp), p(col), p(f), None, p(src_h), p(ref), p(tmp))
    assert rel_err(dst.cpu().numpy(), ref) < 1e-12


def test_gmres_restart_converges(cuda):
    m, A, rp, col, val, rhs = _system()
    b = torch.tensor(rhs, device="cuda")
    x = torch.zeros_like(b)
    info = g.LinearSolver(A, "gmres", "jacobi", tol=1e-8, maxit=2000, restart=20).solve(A, x, b)
    ox, _ = O.pcg(rp, col, val, rhs, tol=1e-10, maxit=2000, precond="jacobi")
    assert info.converged == 1 and rel_err(x.cpu().numpy(), ox) < 1e-6


def test_spmv(cuda):
    m, A, rp, col, val, rhs = _system()
    x = np.random.default_rng(0).uniform(-1, 1, m.nv)
    y = torch.empty(m.nv, dtype=torch.float64, device="cuda")
    g.spmv(A, torch.tensor(x, device="cuda"), y)
    assert rel_err(y.cpu().numpy(), O.spmv(rp, col, val, x)) < 1e-14


@pytest.mark.parametrize("pc,ordering", [("jacobi", 0), ("ic", 0), ("ilu", 0), ("ic", 1), ("ilu", 1)])
def test_mixed_precision_refinement_reaches_fp64_residual(cuda, pc, ordering):
    """FP32 inner CG (FP32 Jacobi or FP32 ILU(0)/IC(0) factors) inside FP64 iterative
    refinement reaches ||b - A x|| <= 1e-8 ||b||, with the residual checked by the
    oracle's FP64 SpMV.  The multicolour order (ordering 1) runs the whole iteration on
    the permuted system's CSR arrays, the natural order the level-scheduled sweeps."""
    m, A, rp, col, val, rhs = _system(128, 32)
    b = torch.tensor(rhs, device="cuda")
    x = torch.zeros_like(b)
    s = g.LinearSolver(A, "cg", pc, tol=1e-8, maxit=5000, criterion=g.CRITERION_REL,
                       precision=g.PRECISION_MIXED, ordering=ordering)
    info = s.solve(A, x, b)
    assert info.converged == 1 and info.outer_iterations >= 2
    xs = x.cpu().numpy()
    res = np.linalg.norm(rhs - O.spmv(rp, col, val, xs)) / np.linalg.norm(rhs)
    assert res <= 1e-8
    x64 = torch.zeros_like(b)
    info64 = g.LinearSolver(A, "cg", "jacobi", tol=1e-8, maxit=5000, criterion=g.CRITERION_REL).solve(A, x64, b)
    assert info64.converged == 1
    assert rel_err(xs, x64.cpu().numpy()) < 1e-6


def test_mixed_precision_on_the_permuted_csr_arrays_matches_the_slot_sweeps(cuda, monkeypatch):
    """Mixed-precision IC(0) CG on the multicolour order: the CSR path (whole iteration
    on B's arrays) and the slot sweeps (PF2_CG_SLOTS=1) reach the same solution, and at
    the iteration limit both keep the accumulated update."""
    m, A, rp, col, val, rhs = _system(128, 32)
    b = torch.tensor(rhs, device="cuda")
    out = {}
    for slots in ("0", "1"):
        monkeypatch.setenv("PF2_CG_SLOTS", slots)
        x = torch.zeros_like(b)
        s = g.LinearSolver(A, "cg", "ic", tol=1e-8, maxit=5000, criterion=g.CRITERION_REL,
                           precision=g.PRECISION_MIXED, ordering=1)
        info = s.solve(A, x, b)
        assert info.converged == 1
        y = torch.zeros_like(b)
        s5 = g.LinearSolver(A, "cg", "ic", tol=1e-30, maxit=5, criterion=g.CRITERION_REL,
                            precision=g.PRECISION_MIXED, ordering=1)
        lim = s5.solve(A, y, b, check=False)
        assert lim.converged == 0 and lim.iterations == 5
        ys, xs = y.cpu().numpy(), x.cpu().numpy()
        # CG lowers the A-norm of the error (not necessarily the residual's 2-norm)
        e5 = ys - xs
        assert np.isfinite(ys).all() and e5 @ O.spmv(rp, col, val, e5) < 0.5 * (xs @ O.spmv(rp, col, val, xs))
        # five FP32 iterations follow five FP64 ones up to FP32 rounding
        y64 = torch.zeros_like(b)
        g.LinearSolver(A, "cg", "ic", tol=1e-30, maxit=5, ordering=1).solve(A, y64, b, check=False)
        assert rel_err(ys, y64.cpu().numpy()) < 1e-4
        out[slots] = (xs, info.iterations, ys)
    assert abs(out["0"][1] - out["1"][1]) <= 3
    assert rel_err(out["0"][0], out["1"][0]) < 1e-6
    assert rel_err(out["0"][2], out["1"][2]) < 1e-4  # five FP32 iterations, two sweep orders


def _greedy_colour_perm(rp, col):
    n = rp.size - 1
    colour = -np.ones(n, int)
    for i in range(n):
        used = {colour[j] for j in col[rp[i]:rp[i + 1]] if j < i}
        c = 0
        while c in used:
            c += 1
        colour[i] = c
    return np.argsort(colour, kind="stable"), colour.max() + 1


@pytest.mark.parametrize("pc", ["ilu", "ic"])
def test_multicolour_preconditioner_matches_oracle_on_the_permuted_matrix(cuda, pc):
    m, A, rp, col, val, rhs = _system(32, 8)
    perm, ncol = _greedy_colour_perm(rp, col)
    assert ncol <= 10
    iperm = np.empty_like(perm)
    iperm[perm] = np.arange(perm.size)
    # B = P A P^T as CSR with sorted columns
    rows = []
    for r in range(perm.size):
        o = perm[r]
        ent = sorted((iperm[col[k]], val[k]) for k in range(rp[o], rp[o + 1]))
        rows.append(ent)
    brp = np.zeros(perm.size + 1, np.int32)
    brp[1:] = np.cumsum([len(e) for e in rows])
    bcol = np.array([c for e in rows for c, _ in e], np.int32)
    bval = np.array([v for e in rows for _, v in e])
    f = O.ilu0(brp, bcol, bval) if pc == "ilu" else O.ic0(brp, bcol, bval)
    src_b = np.ascontiguousarray(rhs[perm])
    out_b, tmp = np.empty_like(src_b), np.empty_like(src_b)
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    O.lib().or_precond_apply.argtypes = [C.c_int, C.c_int] + [C.c_void_p] * 7
    O.lib().or_precond_apply(O.PRECOND[pc], perm.size, p(brp), p(bcol), p(f), None, p(src_b), p(out_b), p(tmp))
    ref = out_b[iperm]
    s = g.LinearSolver(A, "cg", pc, ordering=1)
    s.setup(A)
    src = torch.tensor(rhs, device="cuda")
    dst = torch.empty_like(src)
    s.apply_preconditioner(dst, src)
    assert rel_err(dst.cpu().numpy(), ref) < 1e-12


@pytest.mark.parametrize("pc", ["ilu", "ic"])
def test_multicolour_solve_agrees_with_natural(cuda, pc):
    m, A, rp, col, val, rhs = _system()
    b = torch.tensor(rhs, device="cuda")
    xs = []
    for ordering in (0, 1):
        x = torch.zeros_like(b)
        info = g.LinearSolver(A, "cg", pc, tol=1e-10, maxit=2000, criterion=g.CRITERION_REL,
                              ordering=ordering).solve(A, x, b)
        assert info.converged == 1
        xs.append(x.cpu().numpy())
    assert rel_err(xs[1], xs[0]) < 1e-8


@pytest.mark.parametrize("pc,restart", [("jacobi", 0), ("ilu", 0), ("jacobi", 20)])
def test_gmres_classical_gram_schmidt_twice_matches_oracle(cuda, pc, restart):
    """GMRES with classical Gram-Schmidt applied twice (two batched reductions per
    iteration) converges like the reference's modified Gram-Schmidt."""
    m, A, rp, col, val, rhs = _system()
    b = torch.tensor(rhs, device="cuda")
    x = torch.zeros_like(b)
    info = g.LinearSolver(A, "gmres", pc, tol=1e-8, maxit=2000, restart=restart,
                          orthogonalization=1).solve(A, x, b)
    assert info.converged == 1
    if restart == 0:
        ox, oinfo = O.gmres(rp, col, val, rhs, tol=1e-8, maxit=2000, precond=pc)
        assert abs(info.iterations - oinfo.iterations) <= 2
    ref, _ = O.pcg(rp, col, val, rhs, tol=1e-12, maxit=5000, precond="jacobi")
    assert rel_err(x.cpu().numpy(), ref) < 1e-6


@pytest.mark.parametrize("pc", ["ilu", "ic"])
@pytest.mark.parametrize("band_rows", [None, "256"])
def test_banded_triangular_solves_match_oracle(cuda, pc, band_rows, monkeypatch):
    """Natural order on the 256 x 64 channel (about 320 levels): the banded solve (ranges
    of rows, one block each) gives the oracle's preconditioner, also with more ranges than
    blocks (256-row ranges), and the CG solve converges as the oracle's."""
    if band_rows:
        monkeypatch.setenv("PF2_BAND_ROWS", band_rows)
    m, A, rp, col, val, rhs = _system(256, 64)
    s = g.LinearSolver(A, "cg", pc, tol=1e-8, maxit=2000)
    s.setup(A)
    src = torch.tensor(rhs, device="cuda")
    dst = torch.empty_like(src)
    s.apply_preconditioner(dst, src)
    f = O.ilu0(rp, col, val) if pc == "ilu" else O.ic0(rp, col, val)
    ref, tmp = np.empty_like(rhs), np.empty_like(rhs)
    src_h = np.ascontiguousarray(rhs)
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    O.lib().or_precond_apply.argtypes = [C.c_int, C.c_int] + [C.c_void_p] * 7
    O.lib().or_precond_apply(O.PRECOND[pc], rp.size - 1, p(rp), p(col), p(f), None, p(src_h), p(ref), p(tmp))
    assert rel_err(dst.cpu().numpy(), ref) < 1e-12
    b = torch.tensor(rhs, device="cuda")
    x = torch.zeros_like(b)
    info = s.solve(A, x, b)
    ox, oinfo = O.pcg(rp, col, val, rhs, tol=1e-8, maxit=2000, precond=pc)
    assert info.converged == 1 and abs(info.iterations - oinfo.iterations) <= 2
    assert rel_err(x.cpu().numpy(), ox) < 1e-6


@pytest.mark.parametrize("pc,ordering", [("none", 0), ("jacobi", 0), ("ilu", 0), ("ic", 0), ("ic", 1)])
@pytest.mark.parametrize("criterion", [g.CRITERION_ABS, g.CRITERION_REL])
def test_one_reduction_cg_matches_standard(cuda, pc, ordering, criterion):
    """Chronopoulos-Gear CG (one fused reduction per iteration) reaches the standard
    iteration's solution within the solve tolerance in the same number of iterations, up
    to rounding at the stopping test."""
    m, A, rp, col, val, rhs = _system()
    b = torch.tensor(rhs, device="cuda")
    res = {}
    for variant in (g.CG_STANDARD, g.CG_ONE_REDUCTION):
        x = torch.zeros_like(b)
        s = g.LinearSolver(A, "cg", pc, tol=1e-8, maxit=2000, criterion=criterion, ordering=ordering,
                           cg_variant=variant)
        info = s.solve(A, x, b)
        assert info.converged == 1 and info.status == 0
        res[variant] = (x.cpu().numpy(), info.iterations)
    assert abs(res[0][1] - res[1][1]) <= 2
    assert rel_err(res[1][0], res[0][0]) < 1e-6
    ox, _ = O.pcg(rp, col, val, rhs, tol=1e-8, maxit=2000, precond=pc)
    assert rel_err(res[1][0], ox) < 1e-6


@pytest.mark.parametrize("pc", ["ic", "ilu"])
@pytest.mark.parametrize("criterion", [g.CRITERION_ABS, g.CRITERION_REL])
def test_pipelined_cg_matches_standard(cuda, pc, criterion):
    """Pipelined PCG (one grid-wide step per iteration, ILU(0)/IC(0) on the multicolour
    order, B's CSR arrays): the standard iteration's solution within the solve tolerance
    in the same number of iterations up to rounding at the stopping test."""
    m, A, rp, col, val, rhs = _system(128, 32)
    b = torch.tensor(rhs, device="cuda")
    res = {}
    for variant in (g.CG_STANDARD, g.CG_PIPELINED):
        x = torch.zeros_like(b)
        s = g.LinearSolver(A, "cg", pc, tol=1e-8, maxit=3000, criterion=criterion, ordering=1, cg_variant=variant)
        info = s.solve(A, x, b)
        assert info.converged == 1 and info.status == 0
        res[variant] = (x.cpu().numpy(), info.iterations)
    assert abs(res[0][1] - res[2][1]) <= 3
    assert rel_err(res[2][0], res[0][0]) < 1e-6
    if criterion == g.CRITERION_REL:
        r = rhs - O.spmv(rp, col, val, res[2][0])
        assert np.linalg.norm(r) <= 1e-8 * np.linalg.norm(rhs) * 1.01


def test_pipelined_cg_at_the_limit_and_off_the_csr_path(cuda, monkeypatch):
    m, A, rp, col, val, rhs = _system()
    b = torch.tensor(rhs, device="cuda")
    # seven iterations of each: the same Krylov iterate up to rounding
    xs = {}
    for variant in (g.CG_STANDARD, g.CG_PIPELINED):
        x = torch.zeros_like(b)
        info = g.LinearSolver(A, "cg", "ic", tol=1e-30, maxit=7, ordering=1, cg_variant=variant).solve(
            A, x, b, check=False)
        assert info.converged == 0 and info.iterations == 7
        xs[variant] = x.cpu().numpy()
    assert rel_err(xs[2], xs[0]) < 1e-9
    # slot sweeps (PF2_CG_SLOTS=1, not B's CSR arrays): the standard iteration runs, bit for bit
    monkeypatch.setenv("PF2_CG_SLOTS", "1")
    out = []
    for variant in (g.CG_STANDARD, g.CG_PIPELINED):
        x = torch.zeros_like(b)
        g.LinearSolver(A, "cg", "ic", tol=1e-8, maxit=2000, ordering=1, cg_variant=variant).solve(A, x, b)
        out.append(x.cpu().numpy())
    assert np.array_equal(out[0], out[1])


def test_one_reduction_cg_stops_at_the_limit(cuda):
    m, A, rp, col, val, rhs = _system()
    b = torch.tensor(rhs, device="cuda")
    x = torch.zeros_like(b)
    s = g.LinearSolver(A, "cg", "jacobi", tol=1e-30, maxit=7, cg_variant=g.CG_ONE_REDUCTION)
    info = s.solve(A, x, b, check=False)
    assert info.converged == 0 and info.iterations == 7
    # seven one-reduction iterations equal seven standard ones up to rounding
    y = torch.zeros_like(b)
    g.LinearSolver(A, "cg", "jacobi", tol=1e-30, maxit=7).solve(A, y, b, check=False)
    assert rel_err(x.cpu().numpy(), y.cpu().numpy()) < 1e-10


@pytest.mark.parametrize("pc", ["none", "jacobi"])
@pytest.mark.parametrize("criterion", [g.CRITERION_ABS, g.CRITERION_REL])
def test_bicgstab_matches_oracle(cuda, pc, criterion):
    m, A, rp, col, val, rhs = _system()
    b = torch.tensor(rhs, device="cuda")
    x = torch.zeros_like(b)
    info = g.LinearSolver(A, "bicgstab", pc, tol=1e-10, maxit=2000, criterion=criterion).solve(A, x, b)
    assert info.converged == 1 and info.status == 0
    ox, oinfo = O.pcg(rp, col, val, rhs, tol=1e-12, maxit=5000, precond="jacobi")
    assert rel_err(x.cpu().numpy(), ox) < 1e-6
    r = torch.empty_like(b)
    g.spmv(A, x, r)
    if criterion == g.CRITERION_REL:
        assert float(torch.linalg.norm(b - r)) <= 1e-10 * float(torch.linalg.norm(b)) * (1 + 1e-6)


def test_bicgstab_on_the_nonsymmetric_prediction_system(cuda):
    """The velocity-prediction matrix (outlet edge term: not symmetric) of a flow step:
    BiCGStab and GMRES reach the same solution."""
    xy, tri = mg.channel(64, 16, 4.0, 1.0)
    bu, bv, bp = mg.channel_boundary_nodes(xy, 4.0, 1.0)
    m = g.Mesh2D.from_arrays(xy, tri)
    m.set_channel_boundary_ids(4.0, 1.0)
    eng = g.FlowEngine(m, g.default_params(rho=1.0, mu=0.01, dt=0.005, level=2, n_outer=1), bu, bv, bp)
    eng.seed()
    eng.step()
    A, _ = eng.system(0)
    rp_, col_, val_ = A.download()
    dense = np.zeros((rp_.size - 1,) * 2)
    for i in range(rp_.size - 1):
        dense[i, col_[rp_[i]:rp_[i + 1]]] = val_[rp_[i]:rp_[i + 1]]
    assert np.abs(dense - dense.T).max() > 1e-12  # the outlet term breaks the symmetry
    n = A.rows
    b = torch.tensor(mg.uniform_pm1(3, n), device="cuda")
    x1, x2 = torch.zeros_like(b), torch.zeros_like(b)
    i1 = g.LinearSolver(A, "bicgstab", "jacobi", tol=1e-12, maxit=2000).solve(A, x1, b)
    i2 = g.LinearSolver(A, "gmres", "jacobi", tol=1e-12, maxit=2000).solve(A, x2, b)
    assert i1.converged == 1 and i2.converged == 1
    assert rel_err(x1.cpu().numpy(), x2.cpu().numpy()) < 1e-8


def test_bicgstab_stops_at_the_limit_and_rejects_triangular_preconditioners(cuda):
    m, A, rp, col, val, rhs = _system()
    b = torch.tensor(rhs, device="cuda")
    x = torch.zeros_like(b)
    info = g.LinearSolver(A, "bicgstab", "jacobi", tol=1e-30, maxit=5).solve(A, x, b, check=False)
    assert info.converged == 0 and info.iterations == 5 and np.isfinite(x.cpu().numpy()).all()
    with pytest.raises(g.Pf2Error) as e:
        g.LinearSolver(A, "bicgstab", "ilu")
    assert e.value.status == g.BAD_INPUT


def test_bicgstab_half_step_solution_is_converged(cuda):
    """A diagonal system with power-of-two entries and the Jacobi preconditioner: the
    first half step (alpha = 1) solves it exactly, so s = 0 and t = A M^{-1} s = 0.  That is
    convergence, not a breakdown: x = b / d exactly, reported converged in one iteration."""
    xy, tri = mg.channel(8, 4, 4.0, 1.0)
    m = g.Mesh2D.from_arrays(xy, tri)
    A = g.SparseMatrixCSR(m)
    rp, col, _ = A.download()
    n = rp.size - 1
    d = 2.0 ** np.arange(-3, 5)[np.arange(n) % 8]
    val = np.zeros(col.size)
    for i in range(n):
        val[rp[i] + np.searchsorted(col[rp[i]:rp[i + 1]], i)] = d[i]
    A.upload_values(val)
    rhs = mg.uniform_pm1(7, n)
    for criterion in (g.CRITERION_ABS, g.CRITERION_REL):
        b = torch.tensor(rhs, device="cuda")
        x = torch.zeros_like(b)
        info = g.LinearSolver(A, "bicgstab", "jacobi", tol=1e-10, maxit=50, criterion=criterion).solve(A, x, b)
        assert info.converged == 1 and info.status == 0 and info.iterations == 1
        assert np.array_equal(x.cpu().numpy(), rhs / d)


def test_bicgstab_restarts_an_orthogonal_shadow_residual(cuda):
    """rhat = r0 supported on identity rows that the first iteration zeroes in r: the
    engine restarts the shadow residual as the oracle does and reaches its solution."""
    from tests.helpers import shadow_breakdown_system
    xy, tri, rp, col, val, rhs = shadow_breakdown_system()
    m = g.Mesh2D.from_arrays(xy, tri)
    A = g.SparseMatrixCSR(m)
    A.upload_values(val)
    ox, oinfo = O.bicgstab(rp, col, val, rhs, tol=1e-12, maxit=500, precond="jacobi")
    assert oinfo.converged == 1
    b = torch.tensor(rhs, device="cuda")
    x = torch.zeros_like(b)
    info = g.LinearSolver(A, "bicgstab", "jacobi", tol=1e-12, maxit=500).solve(A, x, b)
    assert info.converged == 1 and info.iterations > 1
    # the dot products round differently (block sums against chunk sums): a few iterations
    assert abs(info.iterations - oinfo.iterations) <= 5
    assert rel_err(x.cpu().numpy(), ox) < 1e-9


@pytest.mark.parametrize("part", ["1", "0"])
def test_barrier_wait_that_runs_out_returns_timeout(cuda, monkeypatch, part):
    """A grid-barrier wait bounded to one poll (PF2_BARRIER_POLLS, read when the solver
    is created; a test knob) gives up before the other blocks arrive: the solve returns
    PF2_TIMEOUT with the record of the block and barrier that gave up, nothing faults, and
    a solver made afterwards with the normal limit solves on the same context.  Both the
    partitioned kernel (the default) and k_pcg (PF2_CG_PART=0)."""
    m, A, rp, col, val, rhs = _system(128, 32)
    b = torch.tensor(rhs, device="cuda")
    monkeypatch.setenv("PF2_CG_PART", part)
    monkeypatch.setenv("PF2_BARRIER_POLLS", "1")
    s = g.LinearSolver(A, "cg", "jacobi", tol=1e-8, maxit=1000)
    monkeypatch.delenv("PF2_BARRIER_POLLS")
    x = torch.zeros_like(b)
    with pytest.raises(g.Pf2Error) as e:
        s.solve(A, x, b)
    assert e.value.status == g.TIMEOUT
    assert "grid barrier timed out in the solver (block" in str(e.value)
    torch.cuda.synchronize()  # the context is still usable
    x = torch.zeros_like(b)
    info = g.LinearSolver(A, "cg", "jacobi", tol=1e-8, maxit=1000).solve(A, x, b)
    assert info.converged == 1 and info.status == 0
    ox, _ = O.pcg(rp, col, val, rhs, tol=1e-8, maxit=1000, precond="jacobi")
    assert rel_err(x.cpu().numpy(), ox) < 1e-6


def _cylinder_system():
    """The Poisson matrix of the quarter-size cylinder mesh (125,364 nodes) with a small
    shift, the size class of the flow's pressure solves."""
    xy, tri = mg.cylinder_channel(nxh=350, nyh=400, nr=12)
    m = g.Mesh2D.from_arrays(xy, tri)
    A = g.SparseMatrixCSR(m)
    area, invJ = O.mesh_geometry(xy, tri)
    rp, col = O.csr_structure(xy.shape[0], tri)
    val, rhs = O.assemble_poisson(xy, tri, area, invJ, rp, col, 1, 1.0)
    diag = np.array([rp[i] + np.searchsorted(col[rp[i]:rp[i + 1]], i) for i in range(rp.size - 1)])
    val[diag] += 1e-2
    A.upload_values(val)
    return m, A, rp, col, val, rhs


def _solve_both(monkeypatch, A, rhs, pc, ordering, parts="", **kw):
    """The same solve by the partitioned kernel (PF2_CG_PART=2: solver creation fails
    unless it applies) and by the kernels it replaces (PF2_CG_PART=0); keyed "1" and "0"."""
    b = torch.tensor(rhs, device="cuda")
    out = {}
    for part in ("2", "0"):
        monkeypatch.setenv("PF2_CG_PART", part)
        if parts:
            monkeypatch.setenv("PF2_CG_PARTS", parts)
        x = torch.zeros_like(b)
        info = g.LinearSolver(A, "cg", pc, ordering=ordering, **kw).solve(A, x, b, check=False)
        out["1" if part == "2" else part] = (x.cpu().numpy(), info)
    return out


@pytest.mark.parametrize("pc,ordering", [("none", 0), ("jacobi", 0), ("ic", 1), ("ilu", 1)])
@pytest.mark.parametrize("parts", ["", "7"])
def test_partitioned_cg_matches_the_other_kernels(cuda, monkeypatch, pc, ordering, parts):
    """The partitioned CG (one part per block with its vectors in shared memory; 4 parts
    of the 2,193-row system, or 7 with PF2_CG_PARTS) against k_pcg / pcg_csr
    (PF2_CG_PART=0) and the oracle, converged to an absolute 1e-12: each row's arithmetic
    is the same, the reductions' order differs, so the solutions agree to 1e-10 and the
    iteration counts within 2."""
    m, A, rp, col, val, rhs = _system(128, 16)
    out = _solve_both(monkeypatch, A, rhs, pc, ordering, parts, tol=1e-12, maxit=5000)
    (xp, ip), (xo, io) = out["1"], out["0"]
    assert ip.converged == 1 and io.converged == 1 and ip.status == 0
    assert abs(ip.iterations - io.iterations) <= 2
    assert rel_err(xp, xo) < 1e-10
    if pc in ("none", "jacobi"):
        ox, oi = O.pcg(rp, col, val, rhs, tol=1e-12, maxit=5000, precond=pc)
        assert oi.converged == 1 and rel_err(xp, ox) < 1e-10


@pytest.mark.parametrize("pc,ordering", [("jacobi", 0), ("ic", 1)])
def test_partitioned_cg_relative_criterion_and_cap(cuda, monkeypatch, pc, ordering):
    """The relative criterion (r.r reduced every iteration) converges like the other
    kernels; at an iteration cap far from convergence (40 iterations) both paths stop with
    the same count, report the same ||r|| / ||b||, and their iterates agree to 1e-9."""
    m, A, rp, col, val, rhs = _system(128, 16)
    out = _solve_both(monkeypatch, A, rhs, pc, ordering, tol=1e-10, maxit=5000, criterion=g.CRITERION_REL)
    (xp, ip), (xo, io) = out["1"], out["0"]
    assert ip.converged == 1 and io.converged == 1 and abs(ip.iterations - io.iterations) <= 2
    assert ip.residual <= 1e-10 and rel_err(xp, xo) < 1e-8
    res = np.linalg.norm(rhs - O.spmv(rp, col, val, xp)) / np.linalg.norm(rhs)
    assert res <= 2e-10
    out = _solve_both(monkeypatch, A, rhs, pc, ordering, tol=1e-30, maxit=40)
    (xp, ip), (xo, io) = out["1"], out["0"]
    assert ip.converged == 0 and io.converged == 0 and ip.iterations == io.iterations == 40
    assert rel_err(xp, xo) < 1e-9


def test_partitioned_cg_on_the_cylinder_mesh(cuda, monkeypatch):
    """IC(0) on the multicolour order, 152 parts (one per SM) of the 125,364-row cylinder
    system: the partitioned kernel and pcg_csr reach the same converged solution (1e-10)
    in the same number of iterations (within 2)."""
    m, A, rp, col, val, rhs = _cylinder_system()
    out = _solve_both(monkeypatch, A, rhs, "ic", 1, tol=1e-12, maxit=20000)
    (xp, ip), (xo, io) = out["1"], out["0"]
    print("cylinder IC(0): partitioned %d iterations, pcg_csr %d, rel diff %.2e" % (
        ip.iterations, io.iterations, rel_err(xp, xo)))
    assert ip.converged == 1 and io.converged == 1 and abs(ip.iterations - io.iterations) <= 2
    assert rel_err(xp, xo) < 1e-10


@pytest.mark.parametrize("pc", ["ic", "ilu"])
@pytest.mark.parametrize("local", ["1", "0"])
def test_partitioned_mixed_cg_matches_the_csr_kernel(cuda, monkeypatch, pc, local):
    """Mixed-precision CG on the parts (FP32 vectors in shared memory, FP32 sweeps and
    SpMV, FP64 refinement; 8 parts of the 4,257-row system, or 7 forced) against the mixed
    kernel on B's CSR arrays (PF2_CG_PART=0): both reach ||b - A x|| <= 1e-8 ||b||
    (checked with the oracle's FP64 SpMV) and agree with the FP64 solution to 1e-6.  With
    the global factors (the default) the iteration counts agree within 10 %; with the
    partition-local factors (PF2_CG_PART_LOCAL=1: one IC(0) / ILU(0) block per part, no
    wait on another part in the sweeps) the solve takes at most 1.6 times the iterations."""
    monkeypatch.setenv("PF2_CG_PART_LOCAL", local)
    m, A, rp, col, val, rhs = _system(128, 32)
    b = torch.tensor(rhs, device="cuda")
    x64 = torch.zeros_like(b)
    g.LinearSolver(A, "cg", "jacobi", tol=1e-12, maxit=20000, criterion=g.CRITERION_REL).solve(A, x64, b)
    x64 = x64.cpu().numpy()
    for parts in ("", "7"):
        if parts:
            monkeypatch.setenv("PF2_CG_PARTS", parts)
        out = _solve_both(monkeypatch, A, rhs, pc, 1, tol=1e-8, maxit=5000, criterion=g.CRITERION_REL,
                          precision=g.PRECISION_MIXED)
        for key, (x, info) in out.items():
            res = np.linalg.norm(rhs - O.spmv(rp, col, val, x)) / np.linalg.norm(rhs)
            print("mixed %s local %s parts %s path %s: %d iterations, %d refinements, residual %.2e" % (
                pc, local, parts or "default", key, info.iterations, info.outer_iterations, res))
            assert info.converged == 1 and info.outer_iterations >= 2 and res <= 1e-8
            assert rel_err(x, x64) < 1e-6
        ip, io = out["1"][1].iterations, out["0"][1].iterations
        if local == "0":
            assert abs(ip - io) <= 0.1 * io + 2
        else:
            assert ip <= 1.6 * io


def test_partitioned_mixed_cg_on_the_cylinder_mesh(cuda, monkeypatch):
    """Mixed IC(0) on the 152 parts of the 125,364-row cylinder system: 1e-8 relative in
    FP64 and within 1e-6 of the FP64 solve, in about as many iterations as the mixed
    kernel on B's CSR arrays."""
    m, A, rp, col, val, rhs = _cylinder_system()
    out = _solve_both(monkeypatch, A, rhs, "ic", 1, tol=1e-8, maxit=20000, criterion=g.CRITERION_REL,
                      precision=g.PRECISION_MIXED)
    b = torch.tensor(rhs, device="cuda")
    x64 = torch.zeros_like(b)
    g.LinearSolver(A, "cg", "ic", tol=1e-12, maxit=20000, criterion=g.CRITERION_REL, ordering=1).solve(A, x64, b)
    x64 = x64.cpu().numpy()
    for key, (x, info) in out.items():
        res = np.linalg.norm(rhs - O.spmv(rp, col, val, x)) / np.linalg.norm(rhs)
        print("cylinder mixed IC(0) path %s: %d iterations, residual %.2e" % (key, info.iterations, res))
        assert info.converged == 1 and res <= 1e-8 and rel_err(x, x64) < 1e-6
    assert abs(out["1"][1].iterations - out["0"][1].iterations) <= 0.1 * out["0"][1].iterations + 2
