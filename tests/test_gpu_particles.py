"""ParticleHandler2D on the GPU against the oracle.

Cell indices, per-cell counts, positions and barycentric coordinates are compared bit
for bit (the oracle orders particles by cell exactly as the engine does); the
projected node velocity within a tolerance (its sums are associated differently).
"""
import numpy as np
import pytest
import torch

import gpupfem2_gb300 as g
from gpupfem2_gb300 import meshgen as mg
from oracle import oracle as O
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

KEYS = ("x", "y", "l0", "l1", "l2", "u", "v", "cell")


def _mesh(nx=32, ny=8, lx=4.0, ly=1.0):
    xy, tri = mg.channel(nx, ny, lx, ly)
    return xy, tri, g.Mesh2D.from_arrays(xy, tri)


def _field(xy, t=0.0):
    x, y = xy[:, 0], xy[:, 1]
    ux = 1.0 + 0.5 * np.sin(2 * np.pi * y + t)
    uy = 0.3 * np.cos(np.pi * x) * np.sin(np.pi * y)
    return ux, uy


def _assert_same(P, R, keys=KEYS):
    assert P["cell"].size == R["cell"].size
    for k in keys:
        assert np.array_equal(P[k], R[k]), k


@pytest.mark.parametrize("level", [1, 2, 3, 4])
def test_seed_bitwise(cuda, level):
    xy, tri, m = _mesh()
    ph = g.ParticleHandler2D(m, level)
    ph.seed()
    _assert_same(ph.download(), O.seed(xy, tri, level))


@pytest.mark.parametrize("level,dt", [(2, 0.05), (3, 0.2), (4, 0.12)])
def test_advect_locate_reseed_bitwise(cuda, level, dt):
    xy, tri, m = _mesh()
    area, invJ = O.mesh_geometry(xy, tri)
    off, idx = O.neighbors(xy.shape[0], tri)
    ph = g.ParticleHandler2D(m, level, capacity_factor=3.0)
    ph.seed()
    R = O.seed(xy, tri, level)
    deleted = added = 0
    for step in range(4):
        ux, uy = _field(xy, 0.7 * step)
        tux, tuy = torch.tensor(ux, device="cuda"), torch.tensor(uy, device="cuda")
        ph.advect(tux, tuy, dt, 3)
        R, nd, na = O.advect(R, xy, tri, invJ, off, idx, ux, uy, dt, 3, level, cap=3 * R["cell"].size)
        deleted += nd
        added += na
        P = ph.download()
        _assert_same(P, R)
    assert deleted > 0 and added > 0  # the outlet deletes, the inlet reseeds


def test_projection_and_correction(cuda):
    xy, tri, m = _mesh()
    area, invJ = O.mesh_geometry(xy, tri)
    off, idx = O.neighbors(xy.shape[0], tri)
    ph = g.ParticleHandler2D(m, 3)
    ph.seed()
    ux, uy = _field(xy)
    tux, tuy = torch.tensor(ux, device="cuda"), torch.tensor(uy, device="cuda")
    ph.init_velocity(tux, tuy)
    R = O.seed(xy, tri, 3)
    R["u"], R["v"] = O.correct_velocity(R, tri, ux, uy)
    _assert_same(ph.download(), R)
    ph.advect(tux, tuy, 0.1, 3)
    R, _, _ = O.advect(R, xy, tri, invJ, off, idx, ux, uy, 0.1, 3, 3)
    px = torch.empty_like(tux)
    py = torch.empty_like(tux)
    ph.project(px, py)
    ox, oy = O.project(R, tri, xy.shape[0])
    # per-cell partial sums, then per-node sums: a different association than the
    # oracle's particle-order accumulation
    assert rel_err(px.cpu().numpy(), ox) < 1e-13 and rel_err(py.cpu().numpy(), oy) < 1e-13
    nx, ny = ux * 1.1, uy - 0.2
    ph.correct(torch.tensor(nx, device="cuda"), torch.tensor(ny, device="cuda"), tux, tuy)
    R["u"], R["v"] = O.correct_velocity(R, tri, nx, ny, ux, uy)
    _assert_same(ph.download(), R)
    # projection after a correction uses the corrected velocities
    ph.project(px, py)
    ox, oy = O.project(R, tri, xy.shape[0])
    assert rel_err(px.cpu().numpy(), ox) < 1e-13


def test_upload_round_trip_and_order(cuda):
    xy, tri, m = _mesh(16, 4)
    R = O.seed(xy, tri, 2)
    perm = np.random.default_rng(1).permutation(R["cell"].size)
    shuffled = {k: v[perm] for k, v in R.items()}
    ph = g.ParticleHandler2D(m, 2)
    ph.upload(shuffled)
    P = ph.download()
    order = np.argsort(shuffled["cell"], kind="stable")
    _assert_same(P, {k: v[order] for k, v in shuffled.items()})


def test_capacity_overflow_is_reported(cuda):
    xy, tri, m = _mesh(16, 4)
    ph = g.ParticleHandler2D(m, 2, capacity_factor=1.1)
    R = O.seed(xy, tri, 2)
    big = {k: np.concatenate([v, v]) for k, v in R.items()}
    with pytest.raises(g.Pf2Error) as e:
        ph.upload(big)
    assert e.value.status == g.OVERFLOW
