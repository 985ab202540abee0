"""The engine against the reference's own GPU kernels (compiled from the reference
sources by oracle/build_ref.sh and launched through tests/refgpu.py) on the same
inputs.

Bit for bit: cell areas and inverse Jacobians, seeded particles, one advection
substep with cell location (compared per cell as multisets, since the reference orders
particles by atomics), particle velocity correction.  Within a tolerance: results the
reference sums with floating-point atomics (projection, assembly).
"""
import ctypes as C

import numpy as np
import pytest
import torch

import gpupfem2_gb300 as g
from gpupfem2_gb300 import meshgen as mg
from oracle import oracle as O
from tests import refgpu as R
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

if not R.available():
    pytest.skip("reference kernels not built (oracle/build_ref.sh needs the reference tree)", allow_module_level=True)


@pytest.fixture(scope="module")
def flow_mod(cuda):
    return R.RefModule("ref_flow.cubin")


@pytest.fixture(scope="module")
def poisson_mod(cuda):
    return R.RefModule("ref_poisson.cubin")


MESHES = {"channel": lambda: mg.channel(64, 16, 4.0, 1.0),
          "cylinder": lambda: mg.cylinder_channel(nxh=100, nyh=100, nr=6)}


def ref_geometry(mod, xy, tri):
    nc = tri.shape[0]
    v, c = R.mesh_buffers(xy, tri)
    area = torch.zeros(nc, dtype=torch.float64, device="cuda")
    inv = torch.zeros(4 * nc, dtype=torch.float64, device="cuda")
    mod.launch("kCalculateCellArea", nc, C.c_int(nc), v, c, area)
    mod.launch("kCalculateInvJacobi", nc, C.c_int(nc), v, c, inv)
    torch.cuda.synchronize()
    return area.cpu().numpy(), inv.cpu().numpy().reshape(nc, 4), v, c, inv


@pytest.mark.parametrize("case", list(MESHES))
def test_geometry_bitwise(flow_mod, case):
    xy, tri = MESHES[case]()
    area, inv, *_ = ref_geometry(flow_mod, xy, tri)
    m = g.Mesh2D.from_arrays(xy, tri)
    assert np.array_equal(m.download("area"), area)
    assert np.array_equal(m.download("inv_jacobi"), inv)
    oa, oi = O.mesh_geometry(xy, tri)
    assert np.array_equal(oa, area) and np.array_equal(oi, inv)


def set_particle_constants(mod, level):
    c = O.subcell_centers(level)
    buf = np.zeros((16, 3))
    buf[: level * level] = c
    mod.set_global("subcellCenters", buf.tobytes())
    mod.set_global("particlesPerCell", np.int32(level * level).tobytes())
    mod.set_global("subcellsPerDim", np.int32(level).tobytes())
    mod.set_global("subcellStep", np.float64(1.0 / level).tobytes())


def to_aos(P):
    a = np.zeros(P["cell"].size, R.PARTICLE)
    for k in ("x", "y", "l0", "l1", "l2", "u", "v"):
        a[k] = P[k]
    a["cell"] = P["cell"]
    a["id"] = np.arange(P["cell"].size)
    return a


@pytest.mark.parametrize("level", [2, 3, 4])
def test_seed_bitwise(flow_mod, level):
    xy, tri = MESHES["channel"]()
    nc = tri.shape[0]
    set_particle_constants(flow_mod, level)
    v, c = R.mesh_buffers(xy, tri)
    parts = torch.zeros(nc * level * level * 96, dtype=torch.uint8, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    flow_mod.launch("kSeedParticlesIntoCell", nc, C.c_int(nc), v, c, parts, cnt)
    ref = R.host(parts, R.PARTICLE)
    ref = ref[np.lexsort((ref["id"], ref["cell"]))]
    m = g.Mesh2D.from_arrays(xy, tri)
    ph = g.ParticleHandler2D(m, level)
    ph.seed()
    P = ph.download()
    for k in ("x", "y", "l0", "l1", "l2", "cell"):
        assert np.array_equal(P[k], ref[k].astype(P[k].dtype)), k


def _key_rows(P, idx=None):
    cols = [P[k] for k in ("cell", "x", "y", "l0", "l1", "l2")]
    rows = np.stack([np.asarray(cl, np.float64).view(np.int64) if cl.dtype == np.float64
                     else cl.astype(np.int64) for cl in cols], axis=1)
    if idx is not None:
        rows = rows[idx]
    return rows[np.lexsort(rows.T[::-1])]


@pytest.mark.parametrize("dt", [0.02, 0.15])
def test_one_substep_bitwise(flow_mod, dt):
    """Lockstep: the same particle state and velocity field through one substep of the
    reference (kAdvectParticles, kCheckParticleInCell, kCheckParticleInNeighbors) and of
    the engine; survivors compared per cell as multisets of exact bits."""
    xy, tri = MESHES["channel"]()
    nc, nv = tri.shape[0], xy.shape[0]
    level = 3
    set_particle_constants(flow_mod, level)
    # a state with particles off the centroids: seed, then one engine step of a field
    x, y = xy[:, 0], xy[:, 1]
    ux = 1.0 + 0.5 * np.sin(2 * np.pi * y)
    uy = 0.3 * np.cos(np.pi * x) * np.sin(np.pi * y)
    m = g.Mesh2D.from_arrays(xy, tri)
    ph = g.ParticleHandler2D(m, level, capacity_factor=3.0)
    ph.seed()
    tux, tuy = torch.tensor(ux, device="cuda"), torch.tensor(uy, device="cuda")
    ph.advect(tux, tuy, 0.05, 3)
    P0 = ph.download()
    # reference substep
    area, inv, v, c, invt = ref_geometry(flow_mod, xy, tri)
    off, idx = O.neighbors(nv, tri)
    n = P0["cell"].size
    parts = R.dev(to_aos(P0))
    vel = R.ptr_array(tux, tuy)
    flow_mod.launch("kAdvectParticles", n, C.c_int(n), c, parts, vel, C.c_double(dt))
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    lst = torch.zeros(n, dtype=torch.int32, device="cuda")
    flow_mod.launch("kCheckParticleInCell", n, C.c_int(n), v, c, invt, parts, cnt, lst)
    nout = int(cnt.item())
    dcnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    dl = torch.zeros(max(n, 1), dtype=torch.int32, device="cuda")
    if nout:
        flow_mod.launch("kCheckParticleInNeighbors", nout, C.c_int(nout), v, c, invt, R.dev(off), R.dev(idx), parts,
                        lst, dcnt, dl)
    ref = R.host(parts, R.PARTICLE)
    deleted = set(dl.cpu().numpy()[: int(dcnt.item())].tolist())
    keep = np.array([i for i in range(n) if i not in deleted], dtype=np.int64)
    refP = {k: ref[k] for k in ("x", "y", "l0", "l1", "l2")}
    refP["cell"] = ref["cell"].astype(np.int64)
    # engine substep (its population check may add particles at sub-cell centroids)
    ph.advect(tux, tuy, dt, 1)
    P1 = ph.download()
    cen = O.subcell_centers(level)
    fresh = np.zeros(P1["cell"].size, bool)
    for k in range(level * level):
        fresh |= (P1["l0"] == cen[k, 0]) & (P1["l1"] == cen[k, 1]) & (P1["l2"] == cen[k, 2])
    assert nout > 0
    assert np.array_equal(_key_rows(refP, keep), _key_rows(P1, np.nonzero(~fresh)[0]))


def test_velocity_correction_bitwise(flow_mod):
    xy, tri = MESHES["channel"]()
    level = 2
    set_particle_constants(flow_mod, level)
    m = g.Mesh2D.from_arrays(xy, tri)
    ph = g.ParticleHandler2D(m, level)
    ph.seed()
    x, y = xy[:, 0], xy[:, 1]
    f = [torch.tensor(a, device="cuda") for a in (np.sin(x) + y, np.cos(y) * x, 0.5 * np.sin(x), 0.1 * y)]
    ph.init_velocity(f[2], f[3])
    P0 = ph.download()
    parts = R.dev(to_aos(P0))
    v, c = R.mesh_buffers(xy, tri)
    n = P0["cell"].size
    flow_mod.launch("kCorrectParticleVelocity", n, C.c_int(n), c, parts, R.ptr_array(f[0], f[1]),
                    R.ptr_array(f[2], f[3]))
    ref = R.host(parts, R.PARTICLE)
    ph.correct(f[0], f[1], f[2], f[3])
    P1 = ph.download()
    assert np.array_equal(P1["u"], ref["u"]) and np.array_equal(P1["v"], ref["v"])


def test_projection(flow_mod):
    xy, tri = MESHES["channel"]()
    nv = xy.shape[0]
    m = g.Mesh2D.from_arrays(xy, tri)
    ph = g.ParticleHandler2D(m, 3)
    ph.seed()
    x, y = xy[:, 0], xy[:, 1]
    ux, uy = torch.tensor(1 + 0.2 * np.sin(3 * y), device="cuda"), torch.tensor(0.1 * np.cos(x), device="cuda")
    ph.init_velocity(ux, uy)
    ph.advect(ux, uy, 0.05, 3)
    P = ph.download()
    n = P["cell"].size
    parts = R.dev(to_aos(P))
    v, c = R.mesh_buffers(xy, tri)
    px, py, w = (torch.zeros(nv, dtype=torch.float64, device="cuda") for _ in range(3))
    outx, outy = torch.zeros_like(px), torch.zeros_like(px)
    flow_mod.launch("kProjectParticleVelocityOntoGrid", n, C.c_int(n), c, parts, R.ptr_array(px, py), w)
    flow_mod.launch("kFinalizeVelocityProjection", nv, C.c_int(nv), R.ptr_array(outx, outy), R.ptr_array(px, py), w)
    gx, gy = torch.empty_like(px), torch.empty_like(px)
    ph.project(gx, gy)
    # the reference sums with atomics in arbitrary order
    assert rel_err(gx.cpu().numpy(), outx.cpu().numpy()) < 1e-13
    assert rel_err(gy.cpu().numpy(), outy.cpu().numpy()) < 1e-13


def _quadrature_constants(mod):
    c3, w = np.zeros(9), np.zeros(3)
    O.lib().or_face_quadrature.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
    O.lib().or_face_quadrature(1, c3.ctypes.data_as(C.c_void_p), w.ctypes.data_as(C.c_void_p))
    face = np.zeros(13, R.GAUSS2D)
    face["x"][:3], face["y"][:3], face["z"][:3], face["w"][:3] = c3[0::3], c3[1::3], c3[2::3], w
    edge = np.zeros(13, R.GAUSS1D)
    edge["c"][:2] = [-0.577350269189626, 0.577350269189626]
    edge["w"][:2] = [1.0, 1.0]
    mod.set_global("faceQuadratureFormula", face.tobytes())
    mod.set_global("faceQuadraturePointsNum", np.int32(3).tobytes())
    mod.set_global("edgeQuadratureFormula", edge.tobytes())
    mod.set_global("edgeQuadraturePointsNum", np.int32(2).tobytes())


def test_poisson_assembly(poisson_mod):
    xy, tri = mg.channel(64, 16, 4.0, 1.0)
    nc, nv = tri.shape[0], xy.shape[0]
    _quadrature_constants(poisson_mod)
    m = g.Mesh2D.from_arrays(xy, tri)
    A = g.SparseMatrixCSR(m)
    rp, col, _ = A.download()
    area, inv = m.download("area"), m.download("inv_jacobi")
    v, c = R.mesh_buffers(xy, tri)
    val = torch.zeros(col.size, dtype=torch.float64, device="cuda")
    rhs = torch.zeros(nv, dtype=torch.float64, device="cuda")
    poisson_mod.launch("kIntegrateOverCell", nc, C.c_int(nc), v, c, R.dev(area), R.dev(inv), R.dev(rp), R.dev(col),
                       val, rhs)
    grhs = torch.zeros(nv, dtype=torch.float64, device="cuda")
    g.assemble_poisson(m, A, grhs, g.RHS_GAUSSIAN, 0.5)
    assert rel_err(A.download()[2], val.cpu().numpy()) < 1e-12
    assert rel_err(grhs.cpu().numpy(), rhs.cpu().numpy()) < 1e-12


def test_flow_assembly(flow_mod):
    xy, tri = mg.channel(64, 16, 4.0, 1.0)
    nc, nv = tri.shape[0], xy.shape[0]
    _quadrature_constants(flow_mod)
    sp = R.SimParams(rho=1.3, mu=0.02, dt=0.01)
    flow_mod.set_global("simParams", bytes(sp))
    m = g.Mesh2D.from_arrays(xy, tri)
    m.set_channel_boundary_ids(4.0, 1.0)
    ids = m.download("edge_ids")
    mats = [g.SparseMatrixCSR(m) for _ in range(2)]
    rp, col, _ = mats[0].download()
    area, inv = m.download("area"), m.download("inv_jacobi")
    v, c = R.mesh_buffers(xy, tri)
    x, y = xy[:, 0], xy[:, 1]
    F = {k: torch.tensor(a, device="cuda") for k, a in dict(
        ux=6 * y * (1 - y), uy=0.1 * np.sin(np.pi * x), uxo=5 * y * (1 - y), uyo=0.05 * np.cos(x),
        pold=2.0 - 0.5 * x, pres=1.5 - 0.4 * x + 0.01 * y, px=1 + 0.1 * np.sin(x * y), py=0.2 * np.cos(y)).items()}
    p = g.default_params(rho=1.3, mu=0.02, dt=0.01)
    drp, dcol = R.dev(rp), R.dev(col)
    zeros = lambda n: torch.zeros(n, dtype=torch.float64, device="cuda")  # noqa: E731
    for pold in (None, F["pold"]):
        vals, rhss = [zeros(col.size) for _ in range(2)], [zeros(nv) for _ in range(2)]
        flow_mod.launch("kIntegrateVelocityPrediction", nc, C.c_int(nc), v, c, R.dev(area), R.dev(inv), R.dev(ids),
                        R.ptr_array(F["ux"], F["uy"]), R.ptr_array(F["uxo"], F["uyo"]), R.ptr_array(drp, drp),
                        R.ptr_array(dcol, dcol), R.ptr_array(*vals), R.ptr_array(*rhss), pold)
        gr = [zeros(nv) for _ in range(2)]
        g.assemble_velocity_prediction(m, p, F["ux"], F["uy"], F["uxo"], F["uyo"], pold, mats[0], mats[1], gr[0], gr[1])
        for k in range(2):
            assert rel_err(mats[k].download()[2], vals[k].cpu().numpy()) < 1e-12
            assert rel_err(gr[k].cpu().numpy(), rhss[k].cpu().numpy()) < 1e-12
        val, rhs = zeros(col.size), zeros(nv)
        flow_mod.launch("kIntegratePressureEquation", nc, C.c_int(nc), v, c, R.dev(area), R.dev(inv),
                        R.ptr_array(F["px"], F["py"]), drp, dcol, val, rhs, pold)
        g.assemble_pressure(m, p, F["px"], F["py"], pold, mats[0], gr[0])
        assert rel_err(mats[0].download()[2], val.cpu().numpy()) < 1e-12
        assert rel_err(gr[0].cpu().numpy(), rhs.cpu().numpy()) < 1e-12
        vals, rhss = [zeros(col.size) for _ in range(2)], [zeros(nv) for _ in range(2)]
        flow_mod.launch("kIntegrateVelocityCorrection", nc, C.c_int(nc), v, c, R.dev(area), R.dev(inv),
                        R.ptr_array(F["px"], F["py"]), F["pres"], R.ptr_array(drp, drp), R.ptr_array(dcol, dcol),
                        R.ptr_array(*vals), R.ptr_array(*rhss), pold)
        g.assemble_velocity_correction(m, p, F["px"], F["py"], F["pres"], pold, mats[0], mats[1], gr[0], gr[1])
        for k in range(2):
            assert rel_err(mats[k].download()[2], vals[k].cpu().numpy()) < 1e-12
            assert rel_err(gr[k].cpu().numpy(), rhss[k].cpu().numpy()) < 1e-12


def test_edge_ids_and_loads(flow_mod):
    xy, tri = MESHES["cylinder"]()
    nc = tri.shape[0]
    _quadrature_constants(flow_mod)
    flow_mod.set_global("simParams", bytes(R.SimParams(rho=1.0, mu=1e-3, dt=5e-4)))
    v, c = R.mesh_buffers(xy, tri)
    ids = torch.zeros(3 * nc, dtype=torch.int32, device="cuda")
    flow_mod.launch("kSetEdgeBoundaryIDs", nc, C.c_int(nc), v, c, ids)
    m = g.Mesh2D.from_arrays(xy, tri)
    m.set_channel_boundary_ids(2.2, 0.41, (0.2, 0.2, 0.05))
    assert np.array_equal(m.download("edge_ids").ravel(), ids.cpu().numpy())
    # body loads on a smooth synthetic field
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    flow_mod.launch("kCountBodyEdges", nc, C.c_int(nc), C.c_int(3), c, ids, cnt, None)
    nb = int(cnt.item())
    cnt.zero_()
    edges = torch.zeros(2 * nb, dtype=torch.int32, device="cuda")
    flow_mod.launch("kCountBodyEdges", nc, C.c_int(nc), C.c_int(3), c, ids, cnt, edges)
    x, y = xy[:, 0], xy[:, 1]
    ux, uy = torch.tensor(1.5 * np.sin(3 * y), device="cuda"), torch.tensor(0.2 * np.cos(5 * x), device="cuda")
    pr = torch.tensor(1.0 - 0.3 * x + 0.2 * y * y, device="cuda")
    loads = torch.zeros(4 * nb, dtype=torch.float64, device="cuda")
    inv = torch.tensor(m.download("inv_jacobi").ravel(), device="cuda")
    flow_mod.launch("kCalculateBodyForces", nb, C.c_int(nb), v, c, inv, edges, R.ptr_array(ux, uy), pr, loads)
    F = loads.cpu().numpy().reshape(nb, 4).sum(axis=0)
    coeff = 2.0 / (1.0 * 1.0 * 1.0 * 0.1)
    cx, cy = (F[0] + F[2]) * coeff, (F[1] + F[3]) * coeff
    p = g.default_params(mu=1e-3, body_boundary_id=3, thickness=0.1)
    gx, gy = g.body_loads(m, p, ux, uy, pr)
    assert abs(gx - cx) < 1e-12 * max(1, abs(cx)) and abs(gy - cy) < 1e-12 * max(1, abs(cy))
