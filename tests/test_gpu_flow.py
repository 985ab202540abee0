"""Whole PFEM-2 steps (cases/Cylinder2D/main.cu:793-880) on the GPU against the oracle,
and the flow systems' assembly kernels one by one."""
import numpy as np
import pytest
import torch

import gpupfem2_gb300 as g
from gpupfem2_gb300 import meshgen as mg
from oracle import oracle as O
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

# Fields of a step: every solve stops at an absolute 1e-8 criterion, and the engine
# and the oracle sum in different orders, so the fields agree to the solver tolerance.
FIELD_TOL = 1e-6


def _channel_case(nx=64, ny=16, level=3, scheme=0, precond=0, n_outer=2):
    xy, tri = mg.channel(nx, ny, 4.0, 1.0)
    bu, bv, bp = mg.channel_boundary_nodes(xy, 4.0, 1.0)
    kw = dict(rho=1.0, mu=0.01, dt=0.005, scheme=scheme, substeps=3, level=level, n_outer=n_outer)
    p = g.default_params(pressure_precond=precond, **kw)
    op = O.make_params(lx=4.0, ly=1.0, pressure_precond=precond, tol=1e-8, **kw)
    return xy, tri, bu, bv, bp, p, op


@pytest.mark.parametrize("scheme,precond", [(0, 0), (1, 0), (0, 1), (1, 2)])
def test_steps_match_oracle(cuda, scheme, precond):
    xy, tri, bu, bv, bp, p, op = _channel_case(scheme=scheme, precond=precond)
    m = g.Mesh2D.from_arrays(xy, tri)
    m.set_channel_boundary_ids(4.0, 1.0)
    eng = g.FlowEngine(m, p, bu, bv, bp)
    eng.seed()
    ref = O.Flow(xy, tri, op, bu, bv, bp)
    for _ in range(3):
        eng.step()
        oi = ref.step()
        info = eng.info()
        assert info.converged == 1 and oi.conv_ok == 1
        assert info.particles == oi.particles
        for name in ("ux", "uy", "p", "pred_x", "pred_y"):
            assert rel_err(eng.field(name), ref.field(name)) < FIELD_TOL, name
    P, R = eng.particles.download(), ref.particles()
    assert np.array_equal(P["cell"], R["cell"])
    assert np.abs(P["x"] - R["x"]).max() < 1e-9


def _flow_arrays(xy, tri):
    x, y = xy[:, 0], xy[:, 1]
    rng = np.random.default_rng(0)
    f = {"ux": 6 * y * (1 - y), "uy": 0.1 * np.sin(np.pi * x), "uxo": 6 * y * (1 - y) * 0.9,
         "uyo": 0.05 * np.cos(x), "pold": 2.0 - 0.5 * x, "px": rng.uniform(0, 1, x.size),
         "py": rng.uniform(-0.1, 0.1, x.size), "pres": 1.5 - 0.4 * x + 0.01 * y}
    return f


def test_flow_assembly_kernels_match_oracle(cuda):
    xy, tri = mg.channel(32, 8, 4.0, 1.0)
    m = g.Mesh2D.from_arrays(xy, tri)
    m.set_channel_boundary_ids(4.0, 1.0)
    area, invJ = O.mesh_geometry(xy, tri)
    rp, col = O.csr_structure(xy.shape[0], tri)
    ids = O.edge_boundary_ids(xy, tri, 4.0, 1.0)
    f = _flow_arrays(xy, tri)
    T = {k: torch.tensor(v, device="cuda") for k, v in f.items()}
    p = g.default_params(rho=1.3, mu=0.02, dt=0.01)
    op = O.make_params(rho=1.3, mu=0.02, dt=0.01)
    nv = xy.shape[0]
    A = [g.SparseMatrixCSR(m) for _ in range(2)]
    r = [torch.zeros(nv, dtype=torch.float64, device="cuda") for _ in range(2)]
    for pold in (None, "pold"):
        g.assemble_velocity_prediction(m, p, T["ux"], T["uy"], T["uxo"], T["uyo"], T[pold] if pold else None,
                                       A[0], A[1], r[0], r[1])
        vx, vy = np.zeros(col.size), np.zeros(col.size)
        bx, by = np.zeros(nv), np.zeros(nv)
        O.lib().or_assemble_prediction(tri.shape[0], xy, tri, area, invJ.ravel(), ids, O.C.byref(op), f["ux"],
                                       f["uy"], f["uxo"], f["uyo"],
                                       f[pold].ctypes.data_as(O.C.c_void_p) if pold else None, rp, col, vx, vy,
                                       bx, by)
        assert rel_err(A[0].download()[2], vx) < 1e-12 and rel_err(A[1].download()[2], vy) < 1e-12
        assert rel_err(r[0].cpu().numpy(), bx) < 1e-12 and rel_err(r[1].cpu().numpy(), by) < 1e-12
        g.assemble_pressure(m, p, T["px"], T["py"], T[pold] if pold else None, A[0], r[0])
        v, b = np.zeros(col.size), np.zeros(nv)
        O.lib().or_assemble_pressure(tri.shape[0], tri, area, invJ.ravel(), O.C.byref(op), f["px"], f["py"],
                                     f[pold].ctypes.data_as(O.C.c_void_p) if pold else None, rp, col, v, b)
        assert rel_err(A[0].download()[2], v) < 1e-12 and rel_err(r[0].cpu().numpy(), b) < 1e-12
        g.assemble_velocity_correction(m, p, T["px"], T["py"], T["pres"], T[pold] if pold else None, A[0], A[1],
                                       r[0], r[1])
        vx, vy = np.zeros(col.size), np.zeros(col.size)
        bx, by = np.zeros(nv), np.zeros(nv)
        O.lib().or_assemble_correction(tri.shape[0], tri, area, invJ.ravel(), O.C.byref(op), f["px"], f["py"],
                                       f["pres"], f[pold].ctypes.data_as(O.C.c_void_p) if pold else None, rp, col,
                                       vx, vy, bx, by)
        assert rel_err(A[0].download()[2], vx) < 1e-12 and rel_err(r[1].cpu().numpy(), by) < 1e-12


def test_prediction_bc_values_match_oracle(cuda):
    xy, tri = mg.channel(32, 8, 4.0, 1.0)
    m = g.Mesh2D.from_arrays(xy, tri)
    area, invJ = O.mesh_geometry(xy, tri)
    bu, bv, bp = mg.channel_boundary_nodes(xy, 4.0, 1.0)
    f = _flow_arrays(xy, tri)
    p = g.default_params(rho=1.3, dt=0.01)
    op = O.make_params(rho=1.3, dt=0.01)
    src, dst = g.DirichletBCs(m.nv, bu), g.DirichletBCs(m.nv, bu)
    node_to_bc = -np.ones(m.nv, np.int32)
    for k, (i, _) in enumerate(bu):
        node_to_bc[i] = k
    bn = np.array([i for i, _ in bu], np.int32)
    bvals = np.array([v for _, v in bu])
    for comp in (0, 1):
        g.prediction_bc_values(m, p, src, dst, torch.tensor(f["pres"], device="cuda"),
                               torch.tensor(f["pold"], device="cuda"), comp)
        out = np.zeros(len(bu))
        O.lib().or_prediction_bc(tri.shape[0], tri, area, invJ.ravel(), O.C.byref(op), f["pres"],
                                 f["pold"].ctypes.data_as(O.C.c_void_p), len(bu), bn, bvals, node_to_bc, comp, out)
        assert rel_err(g.bc_values(dst).cpu().numpy(), out) < 1e-12


def test_body_loads_match_oracle(cuda):
    xy, tri = mg.cylinder_channel(nxh=100, nyh=100, nr=6)
    m = g.Mesh2D.from_arrays(xy, tri)
    m.set_channel_boundary_ids(2.2, 0.41, (0.2, 0.2, 0.05))
    ids = O.edge_boundary_ids(xy, tri, 2.2, 0.41, (0.2, 0.2, 0.05))
    area, invJ = O.mesh_geometry(xy, tri)
    x, y = xy[:, 0], xy[:, 1]
    ux, uy, pr = 1.5 * np.sin(3 * y), 0.2 * np.cos(5 * x), 1.0 - 0.3 * x + 0.2 * y * y
    p = g.default_params(mu=1e-3, body_boundary_id=3, thickness=0.1)
    op = O.make_params(mu=1e-3, body_id=3, thickness=0.1, cx=0.2, cy=0.2)
    cx, cy = g.body_loads(m, p, torch.tensor(ux, device="cuda"), torch.tensor(uy, device="cuda"),
                          torch.tensor(pr, device="cuda"))
    ref = np.zeros(2)
    O.lib().or_body_loads(tri.shape[0], xy, tri, invJ.ravel(), ids, O.C.byref(op), ux, uy, pr, ref)
    assert abs(cx - ref[0]) < 1e-12 * max(1.0, abs(ref[0])) and abs(cy - ref[1]) < 1e-12 * max(1.0, abs(ref[1]))


def test_learned_guess_keeps_the_solution(cuda):
    """Pressure solves started from the learned guess (trained online on the first
    steps) reach the same converged fields as solves started from the previous
    pressure: the solver, with its relative 1e-8 test, stays the judge."""
    xy, tri, bu, bv, bp, p, op = _channel_case()
    m = g.Mesh2D.from_arrays(xy, tri)
    m.set_channel_boundary_ids(4.0, 1.0)
    runs = {}
    for x0 in (0, 1):
        prm = g.default_params(rho=1.0, mu=0.01, dt=0.005, scheme=0, substeps=3, level=3, n_outer=2,
                               pressure_precond=0, pressure_criterion=1, pressure_x0=x0, learn_steps=4,
                               learn_rate=1e-3)
        eng = g.FlowEngine(m, prm, bu, bv, bp)
        eng.seed()
        used = 0
        for _ in range(8):
            eng.step()
            inf = eng.info()
            assert inf.converged == 1 and inf.status == 0
            used += inf.guess_used
        runs[x0] = (eng.field("p"), eng.field("ux"), used)
    assert rel_err(runs[1][0], runs[0][0]) < 1e-6 and rel_err(runs[1][1], runs[0][1]) < 1e-6
    assert runs[0][2] == 0


@pytest.mark.parametrize("option", ["bicgstab", "one_reduction"])
def test_solver_options_keep_the_step(cuda, option):
    """BiCGStab for the velocity prediction, or one-reduction CG for the pressure and
    correction solves: the same fields as the reference's solvers to the solve tolerance."""
    xy, tri, bu, bv, bp, p, op = _channel_case()
    m = g.Mesh2D.from_arrays(xy, tri)
    m.set_channel_boundary_ids(4.0, 1.0)
    runs = []
    for alt in (False, True):
        kw = dict(rho=1.0, mu=0.01, dt=0.005, scheme=0, substeps=3, level=3, n_outer=2, pressure_precond=2,
                  pressure_ordering=1)
        if alt:
            kw.update(prediction_solver=g.SOLVER_BICGSTAB if option == "bicgstab" else g.SOLVER_GMRES,
                      cg_variant=g.CG_ONE_REDUCTION if option == "one_reduction" else g.CG_STANDARD)
        eng = g.FlowEngine(m, g.default_params(**kw), bu, bv, bp)
        eng.seed()
        for _ in range(3):
            eng.step()
            assert eng.info().converged == 1
        runs.append({f: eng.field(f) for f in ("ux", "uy", "p")})
    for f in ("ux", "uy", "p"):
        assert rel_err(runs[1][f], runs[0][f]) < FIELD_TOL, f


def test_particle_buffers_grow_with_the_flow(cuda):
    """Reseeding only adds particles; an engine created with room for 1.1x the seeded
    particles grows its buffers between steps and repeats, bit for bit, the run of an
    engine created with room to spare."""
    xy, tri, bu, bv, bp, p, op = _channel_case(level=3)
    m = g.Mesh2D.from_arrays(xy, tri)
    m.set_channel_boundary_ids(4.0, 1.0)
    out = []
    for cap in (1.1, 8.0):
        eng = g.FlowEngine(m, p, bu, bv, bp, capacity_factor=cap)
        eng.seed()
        for _ in range(6):
            eng.step()
            assert eng.info().status == 0
        out.append((eng.particles.download(), eng.field("ux"), eng.field("p")))
    (pa, ua, qa), (pb, ub, qb) = out
    assert pa["cell"].size > 1.1 * 9 * tri.shape[0] * 0.75  # the small engine did have to grow
    for k in pa:
        assert np.array_equal(pa[k], pb[k]), k
    assert np.array_equal(ua, ub) and np.array_equal(qa, qb)


def test_particles_reserve_keeps_the_particles(cuda):
    xy, tri = mg.channel(32, 8, 4.0, 1.0)
    m = g.Mesh2D.from_arrays(xy, tri)
    h = g.ParticleHandler2D(m, 3, capacity_factor=1.1)
    h.seed()
    before = h.download()
    h.reserve(10 * tri.shape[0] * 9)
    after = h.download()
    for k in before:
        assert np.array_equal(before[k], after[k]), k
