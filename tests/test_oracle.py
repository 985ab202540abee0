"""CPU checks of the oracle itself (analytic solutions and factorisation identities)."""
import numpy as np
import pytest

from gpupfem2_gb300 import meshgen as mg
from oracle import oracle as O
from tests.helpers import poisson_square


def _poisson_system(n, rhs_kind=1, lam=1.0):
    xy, tri, bcs = poisson_square(n)
    area, invJ = O.mesh_geometry(xy, tri)
    rp, col = O.csr_structure(xy.shape[0], tri)
    val, rhs = O.assemble_poisson(xy, tri, area, invJ, rp, col, rhs_kind, lam)
    bn = np.array([b for b, _ in bcs], np.int32)
    bv = np.array([v for _, v in bcs])
    val, rhs = O.apply_bcs(rp, col, val, rhs, bn, bv)
    return xy, rp, col, val, rhs


def test_poisson_second_order_convergence():
    errs = []
    for n in (16, 32, 64):
        xy, rp, col, val, rhs = _poisson_system(n)
        x, info = O.pcg(rp, col, val, rhs, tol=1e-12, maxit=2000, precond="jacobi")
        assert info.converged
        exact = np.sin(np.pi * xy[:, 0]) * np.sin(np.pi * xy[:, 1])
        errs.append(np.abs(x - exact).max())
    assert 3.5 < errs[0] / errs[1] < 4.5 and 3.5 < errs[1] / errs[2] < 4.5


def test_csr_sizes_of_the_workloads():
    xy, tri = mg.unit_square(64)
    assert O.csr_structure(xy.shape[0], tri)[1].size == 29057
    xy, tri = mg.channel()
    assert O.csr_structure(xy.shape[0], tri)[1].size == 115649


def _spd_channel():
    xy, tri = mg.channel(16, 8, 2.0, 1.0)
    area, invJ = O.mesh_geometry(xy, tri)
    rp, col = O.csr_structure(xy.shape[0], tri)
    val, rhs = O.assemble_poisson(xy, tri, area, invJ, rp, col, 1, 1.0)
    diag = np.array([rp[i] + np.searchsorted(col[rp[i]:rp[i + 1]], i) for i in range(rp.size - 1)])
    val[diag] += 0.01
    return rp, col, val, rhs


def _dense(rp, col, val, part=None):
    n = rp.size - 1
    A = np.zeros((n, n))
    for i in range(n):
        for k in range(rp[i], rp[i + 1]):
            j = col[k]
            if part == "lower" and j > i:
                continue
            if part == "strict_lower" and j >= i:
                continue
            if part == "upper" and j < i:
                continue
            A[i, j] = val[k]
    return A


def test_ic0_and_ilu0_reproduce_a_on_its_pattern():
    rp, col, val, _ = _spd_channel()
    A = _dense(rp, col, val)
    L = _dense(rp, col, O.ic0(rp, col, val), "lower")
    assert np.abs((L @ L.T - A)[A != 0]).max() < 1e-12
    f = O.ilu0(rp, col, val)
    Lu = _dense(rp, col, f, "strict_lower") + np.eye(A.shape[0])
    U = _dense(rp, col, f, "upper")
    assert np.abs((Lu @ U - A)[A != 0]).max() < 1e-12


@pytest.mark.parametrize("pc", ["none", "jacobi", "ilu", "ic"])
def test_cg_and_gmres_agree(pc):
    rp, col, val, rhs = _spd_channel()
    x, info = O.pcg(rp, col, val, rhs, tol=1e-12, maxit=2000, precond=pc)
    y, info2 = O.gmres(rp, col, val, rhs, tol=1e-12, maxit=500, precond=pc)
    assert info.converged and info2.converged
    A = _dense(rp, col, val)
    xs = np.linalg.solve(A, rhs)
    assert np.abs(x - xs).max() < 1e-8 * np.abs(xs).max()
    assert np.abs(y - xs).max() < 1e-8 * np.abs(xs).max()


def test_ic_preconditioner_cuts_iterations():
    rp, col, val, rhs = _spd_channel()
    nj = O.pcg(rp, col, val, rhs, tol=1e-10, precond="jacobi")[1].iterations
    ni = O.pcg(rp, col, val, rhs, tol=1e-10, precond="ic")[1].iterations
    assert ni < nj


@pytest.mark.parametrize("level", [1, 2, 3, 4])
def test_subcell_centres_map_to_their_subcell(level):
    c = O.subcell_centers(level)
    assert c.shape == (level * level, 3)
    assert np.allclose(c.sum(axis=1), 1.0, atol=1e-15)
    for k in range(level * level):
        assert O.determine_subcell(level, c[k]) == k


def test_seed_and_still_flow_keep_particles():
    xy, tri = mg.channel(8, 4, 2.0, 1.0)
    area, invJ = O.mesh_geometry(xy, tri)
    off, idx = O.neighbors(xy.shape[0], tri)
    P = O.seed(xy, tri, 3)
    assert P["cell"].size == 9 * tri.shape[0]
    z = np.zeros(xy.shape[0])
    Q, nd, na = O.advect(P, xy, tri, invJ, off, idx, z, z, 0.1, 3, 3)
    assert nd == 0 and na == 0 and Q["cell"].size == P["cell"].size
    assert np.array_equal(Q["cell"], P["cell"]) and np.array_equal(Q["x"], P["x"])


def test_uniform_flow_moves_deletes_and_reseeds():
    xy, tri = mg.channel(16, 4, 4.0, 1.0)
    area, invJ = O.mesh_geometry(xy, tri)
    off, idx = O.neighbors(xy.shape[0], tri)
    P = O.seed(xy, tri, 2)
    ux = np.full(xy.shape[0], 1.0)
    uy = np.zeros(xy.shape[0])
    Q, nd, na = O.advect(P, xy, tri, invJ, off, idx, ux, uy, 0.2, 3, 2)
    assert nd > 0 and na > 0
    # every cell has every sub-cell populated after the reseed
    counts = np.bincount(Q["cell"], minlength=tri.shape[0])
    assert counts.min() >= 4
    assert np.all(np.diff(Q["cell"]) >= 0)


def test_bicgstab_restarts_an_orthogonal_shadow_residual():
    """rhat = r0 lives on identity rows that the first iteration zeroes in r, so
    rhat.r = 0 exactly with r != 0: the solve restarts rhat = r and converges to the
    direct solution instead of stopping."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    from tests.helpers import shadow_breakdown_system
    xy, tri, rp, col, val, rhs = shadow_breakdown_system()
    n = rp.size - 1
    A = sp.csr_matrix((val, col, rp), shape=(n, n))
    exact = spl.spsolve(A.tocsc(), rhs)
    for criterion in (0, 1):
        x, info = O.bicgstab(rp, col, val, rhs, tol=1e-12, maxit=500, precond="jacobi", criterion=criterion)
        assert info.converged == 1 and info.iterations > 1
        assert np.abs(x - exact).max() < 1e-9 * np.abs(exact).max()


def test_solver_options_agree_on_a_converged_system():
    """The engine's solver options restated in the oracle (multicolour IC(0)/ILU(0) CG,
    the relative criterion, BiCGStab, GMRES with classical Gram-Schmidt twice) reach the
    natural-order solution of the reference's CG."""
    xy, tri = mg.channel(64, 16, 4.0, 1.0)
    area, invJ = O.mesh_geometry(xy, tri)
    rp, col = O.csr_structure(xy.shape[0], tri)
    val, rhs = O.assemble_poisson(xy, tri, area, invJ, rp, col, 1, 1.0)
    diag = np.array([rp[i] + np.searchsorted(col[rp[i]:rp[i + 1]], i) for i in range(rp.size - 1)])
    val[diag] += 1e-2
    ref, _ = O.pcg(rp, col, val, rhs, tol=1e-13, maxit=5000, precond="jacobi")
    for pc in ("jacobi", "ilu", "ic"):
        for ordering in (0, 1):
            x, info, rel = O.cg(rp, col, val, rhs, tol=1e-11, maxit=5000, precond=pc, ordering=ordering,
                                criterion=1)
            assert info.converged == 1 and rel <= 1e-11
            assert np.abs(x - ref).max() < 1e-9 * np.abs(ref).max()
    x, info = O.bicgstab(rp, col, val, rhs, tol=1e-11, maxit=5000, precond="jacobi", criterion=1)
    assert info.converged == 1 and np.abs(x - ref).max() < 1e-9 * np.abs(ref).max()
    x, info = O.gmres_cgs2(rp, col, val, rhs, tol=1e-11, maxit=2000, precond="jacobi")
    x2, info2 = O.gmres(rp, col, val, rhs, tol=1e-11, maxit=2000, precond="jacobi")
    assert info.converged == 1 and abs(info.iterations - info2.iterations) <= 2
    assert np.abs(x - ref).max() < 1e-8 * np.abs(ref).max()


def test_oracle_flow_with_the_engine_solver_choices():
    """A cylinder flow from rest with BiCGStab for the prediction: every solve of the
    first steps converges (the first prediction system is the one whose shadow residual
    the first iteration makes orthogonal), and the fields agree with GMRES's within the
    solve tolerance."""
    xy, tri = mg.cylinder_channel(nxh=100, nyh=100, nr=6)
    bu, bv, bp = mg.channel_boundary_nodes(xy, 2.2, 0.41, 1.5, cylinder=(0.2, 0.2, 0.05))
    base = dict(rho=1.0, mu=1e-3, dt=5e-4, scheme=1, level=2, n_outer=2, substeps=3, pressure_precond=2,
                calc_loads=1, body_id=3, thickness=0.1, lx=2.2, ly=0.41, has_cylinder=1, cx=0.2, cy=0.2,
                radius=0.05, tol=1e-12, maxit=3000, pressure_tol=1e-13, pressure_maxit=5000, pressure_criterion=1,
                pressure_ordering=1)
    out = {}
    for pred in (1, 2):
        f = O.Flow(xy, tri, O.make_params(prediction_solver=pred, **base), bu, bv, bp)
        for _ in range(2):
            info = f.step()
            assert info.conv_ok == 1 and info.res_pres[0] <= 1e-13
        out[pred] = (f.field("ux"), f.field("p"), info.cx)
    for k in range(2):
        assert np.abs(out[1][k] - out[2][k]).max() <= 1e-9 * np.abs(out[1][k]).max()
    assert abs(out[1][2] - out[2][2]) <= 1e-9 * abs(out[1][2])
