"""Checkpoint / restart of particles, the learned guess's network and whole flow engines:
a run restarted from a checkpoint repeats the uninterrupted run bit for bit, and a
checkpoint that does not fit the receiving object is rejected."""
import numpy as np
import pytest
import torch

import gpupfem2_gb300 as g
from gpupfem2_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu

FIELDS = ("ux", "uy", "ux_old", "uy_old", "pred_x", "pred_y", "p", "p_old")


def _case(scheme, x0):
    xy, tri = mg.channel(64, 16, 4.0, 1.0)
    bu, bv, bp = mg.channel_boundary_nodes(xy, 4.0, 1.0)
    m = g.Mesh2D.from_arrays(xy, tri)
    m.set_channel_boundary_ids(4.0, 1.0)
    prm = g.default_params(rho=1.0, mu=0.01, dt=0.005, scheme=scheme, substeps=3, level=3, n_outer=2,
                           pressure_precond=1, pressure_x0=x0, learn_steps=3, learn_rate=1e-3)
    return m, prm, bu, bv, bp


def _state(eng):
    P = eng.particles.download()
    return {**{f: eng.field(f) for f in FIELDS}, **{"part_" + k: v for k, v in P.items()}}


@pytest.mark.parametrize("scheme,x0", [(0, 0), (1, 1)])
def test_flow_restart_repeats_the_run(cuda, tmp_path, scheme, x0):
    m, prm, bu, bv, bp = _case(scheme, x0)
    whole = g.FlowEngine(m, prm, bu, bv, bp)
    whole.seed()
    for _ in range(5):
        whole.step()
    ref = _state(whole)
    first = g.FlowEngine(m, prm, bu, bv, bp)
    first.seed()
    for _ in range(2):
        first.step()
    path = tmp_path / "flow.ckpt"
    first.save(path)
    del first
    resumed = g.FlowEngine(m, prm, bu, bv, bp)
    resumed.load(path)
    for _ in range(3):
        resumed.step()
        assert resumed.info().converged == 1
    got = _state(resumed)
    for k, v in ref.items():
        assert np.array_equal(got[k], v), k


def test_particles_checkpoint_continues_exactly(cuda, tmp_path):
    xy, tri = mg.channel(32, 8, 4.0, 1.0)
    m = g.Mesh2D.from_arrays(xy, tri)
    x, y = xy[:, 0], xy[:, 1]
    ux = torch.tensor(6 * y * (1 - y), device="cuda")
    uy = torch.tensor(0.2 * np.sin(np.pi * x), device="cuda")
    a = g.ParticleHandler2D(m, 3)
    a.seed()
    a.init_velocity(ux, uy)
    a.advect(ux, uy, 0.02, 3)
    a.save(tmp_path / "p.ckpt")
    b = g.ParticleHandler2D(m, 3)
    b.load(tmp_path / "p.ckpt")
    Pa, Pb = a.download(), b.download()
    for k in Pa:
        assert np.array_equal(Pa[k], Pb[k]), k
    # projection right after the load reads the saved cell segments
    na = [torch.zeros_like(ux) for _ in range(2)]
    nb = [torch.zeros_like(ux) for _ in range(2)]
    a.project(*na)
    b.project(*nb)
    assert torch.equal(na[0], nb[0]) and torch.equal(na[1], nb[1])
    for h in (a, b):
        h.advect(ux, uy, 0.02, 3)
    Pa, Pb = a.download(), b.download()
    for k in Pa:
        assert np.array_equal(Pa[k], Pb[k]), k


def test_network_checkpoint_continues_training(cuda, tmp_path):
    xy, tri = mg.channel(32, 8, 4.0, 1.0)
    m = g.Mesh2D.from_arrays(xy, tri)
    n = xy.shape[0]
    gen = torch.Generator(device="cuda").manual_seed(0)
    feat = torch.rand(n * 5, device="cuda", generator=gen) - 0.5
    target = torch.rand(n, device="cuda", generator=gen) - 0.5
    a = g.LearnedGuess(m, seed=3)
    for _ in range(3):
        a.train_step(feat, target)
    b = g.LearnedGuess(m, seed=3)
    b.train_step(feat, target)
    b.save(tmp_path / "net.ckpt")
    c = g.LearnedGuess(m, seed=11)
    c.load(tmp_path / "net.ckpt")
    assert np.array_equal(c.params(), b.params())
    for _ in range(2):
        c.train_step(feat, target)  # the AdamW moments and step count came along
    assert np.array_equal(c.params(), a.params())
    ya, yc = torch.empty(n, device="cuda"), torch.empty(n, device="cuda")
    a.forward(feat, ya)
    c.forward(feat, yc)
    assert torch.equal(ya, yc)


def test_checkpoints_that_do_not_fit_are_rejected(cuda, tmp_path):
    xy, tri = mg.channel(32, 8, 4.0, 1.0)
    m = g.Mesh2D.from_arrays(xy, tri)
    h3 = g.ParticleHandler2D(m, 3)
    h3.seed()
    path = tmp_path / "p.ckpt"
    h3.save(path)
    with pytest.raises(g.Pf2Error) as e:  # another level
        g.ParticleHandler2D(m, 2).load(path)
    assert e.value.status == g.BAD_INPUT and "level" in str(e.value)
    small = g.Mesh2D.from_arrays(*mg.channel(16, 8, 4.0, 1.0))
    with pytest.raises(g.Pf2Error) as e:  # another mesh
        g.ParticleHandler2D(small, 3).load(path)
    assert e.value.status == g.BAD_INPUT and "cells" in str(e.value)
    with pytest.raises(g.Pf2Error) as e:  # another kind of object
        g.LearnedGuess(m).load(path)
    assert e.value.status == g.BAD_INPUT and "kind" in str(e.value)
    data = path.read_bytes()
    cut = tmp_path / "cut.ckpt"
    cut.write_bytes(data[: len(data) // 2])
    with pytest.raises(g.Pf2Error) as e:
        g.ParticleHandler2D(m, 3).load(cut)
    assert e.value.status == g.BAD_INPUT and "truncated" in str(e.value)
    longer = tmp_path / "long.ckpt"
    longer.write_bytes(data + b"\0")
    with pytest.raises(g.Pf2Error) as e:
        g.ParticleHandler2D(m, 3).load(longer)
    assert e.value.status == g.BAD_INPUT and "after the last section" in str(e.value)
    with pytest.raises(g.Pf2Error) as e:
        g.ParticleHandler2D(m, 3).load(tmp_path / "missing.ckpt")
    assert e.value.status == g.IO_ERROR
