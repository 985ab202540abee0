"""The learned-guess network on the GPU (BF16 tensor-core MLPs, FP32 accumulation)
against the FP64 oracle: outputs, gradients, and a training run that lowers the loss.
BF16 rounding of weights and activations bounds the agreement: outputs within 2e-2 and
gradients within 5e-2, both relative in the 2-norm."""
import numpy as np
import pytest
import torch

import gpupfem2_gb300 as g
from gpupfem2_gb300 import meshgen as mg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _case(nx=40, ny=12):
    xy, tri = mg.channel(nx, ny, 4.0, 1.0)
    m = g.Mesh2D.from_arrays(xy, tri)
    rp, col = O.csr_structure(xy.shape[0], tri)
    rng = np.random.default_rng(5)
    x, y = xy[:, 0] / 4.0, xy[:, 1]
    feat = np.stack([x, y, np.sin(3 * x) * y, np.cos(2 * y) - x, rng.normal(scale=0.3, size=x.size)], axis=1)
    t = np.sin(2 * np.pi * x) * y * (1 - y) + 0.1 * feat[:, 3]
    return m, rp, col, feat, t


def _nrel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_forward_and_gradient_match_oracle(cuda):
    m, rp, col, feat, t = _case()
    net = g.LearnedGuess(m, seed=1)
    rng = np.random.default_rng(2)
    theta = rng.normal(scale=0.15, size=net.n_params).astype(np.float32)
    net.set_params(theta)
    f = torch.tensor(feat, dtype=torch.float32, device="cuda")
    y = torch.empty(m.nv, dtype=torch.float32, device="cuda")
    net.forward(f, y)
    oy, _ = O.mpnn_forward(rp, col, feat.astype(np.float32).astype(np.float64), theta.astype(np.float64))
    assert _nrel(y.cpu().numpy(), oy) < 2e-2
    tt = torch.tensor(t, dtype=torch.float32, device="cuda")
    loss = net.train_step(f, tt, apply=False)
    og, oloss = O.mpnn_backward(rp, col, feat.astype(np.float32).astype(np.float64), theta.astype(np.float64),
                                t.astype(np.float32).astype(np.float64))
    assert abs(loss - oloss) < 3e-2 * oloss
    gg = net.grad()
    assert _nrel(gg, og) < 5e-2
    # every parameter block is exercised
    blocks = [(0, 320), (320, 384), (384, 384 + 8256), (net.n_params - 65, net.n_params - 1), (net.n_params - 1,
                                                                                              net.n_params)]
    for a, b in blocks:
        assert _nrel(gg[a:b], og[a:b]) < 8e-2, (a, b)
    assert np.array_equal(net.params(), theta)


def test_training_lowers_the_loss_and_is_deterministic(cuda):
    m, rp, col, feat, t = _case()
    f = torch.tensor(feat, dtype=torch.float32, device="cuda")
    tt = torch.tensor(t, dtype=torch.float32, device="cuda")
    runs = []
    for _ in range(2):
        net = g.LearnedGuess(m, seed=7)
        losses = [net.train_step(f, tt, lr=3e-3) for _ in range(150)]
        runs.append((losses, net.params()))
    losses = runs[0][0]
    assert losses[-1] < 0.25 * losses[0]
    assert runs[0][0] == runs[1][0] and np.array_equal(runs[0][1], runs[1][1])


def test_tcgen05_layer_matches_mma_sync(cuda, monkeypatch):
    """The forward layer on tcgen05 (tensor-memory accumulator, 128 nodes per CTA; the
    default) against the mma.sync layer (PF2_MPNN_MMA=sync) on a graph whose last tile is
    ragged: the same BF16 products summed in FP32 in another order."""
    m, rp, col, feat, t = _case(64, 24)
    assert m.nv % 128 != 0
    rng = np.random.default_rng(4)
    theta = None
    outs = {}
    f = torch.tensor(feat, dtype=torch.float32, device="cuda")
    for mode in ("tcgen05", "sync"):
        if mode == "sync":
            monkeypatch.setenv("PF2_MPNN_MMA", "sync")
        else:
            monkeypatch.delenv("PF2_MPNN_MMA", raising=False)
        net = g.LearnedGuess(m, seed=3)
        if theta is None:
            theta = rng.normal(scale=0.15, size=net.n_params).astype(np.float32)
        net.set_params(theta)
        y = torch.empty(m.nv, dtype=torch.float32, device="cuda")
        net.forward(f, y)
        net.params()  # synchronises and reports a tensor-core wait that ran out
        outs[mode] = y.cpu().numpy()
    assert np.isfinite(outs["tcgen05"]).all()
    assert _nrel(outs["tcgen05"], outs["sync"]) < 1e-3
    oy, _ = O.mpnn_forward(rp, col, feat.astype(np.float32).astype(np.float64), theta.astype(np.float64))
    assert _nrel(outs["tcgen05"], oy) < 2e-2
