"""The learned-guess network of the oracle: analytic gradients against central finite
differences (FP64), and AdamW against a direct restatement."""
import numpy as np

from gpupfem2_gb300 import meshgen as mg
from oracle import oracle as O


def _graph():
    xy, tri = mg.channel(6, 3, 2.0, 1.0)
    rp, col = O.csr_structure(xy.shape[0], tri)
    rng = np.random.default_rng(3)
    feat = rng.normal(size=(xy.shape[0], O.MPNN_IN))
    t = rng.normal(size=xy.shape[0])
    theta = rng.normal(scale=0.2, size=O.mpnn_param_count())
    return rp, col, feat, t, theta


def test_param_count():
    assert O.mpnn_param_count() == 64 * 5 + 64 + 3 * (64 * 128 + 64) + 64 + 1


def test_backward_matches_finite_differences():
    rp, col, feat, t, theta = _graph()
    g, loss = O.mpnn_backward(rp, col, feat, theta, t)
    _, loss2 = O.mpnn_forward(rp, col, feat, theta, t)
    assert abs(loss - loss2) < 1e-14 * max(1, abs(loss))
    rng = np.random.default_rng(0)
    idx = np.concatenate([rng.choice(theta.size, 60, replace=False), [theta.size - 1, theta.size - 2]])
    h = 1e-6
    for k in idx:
        tp, tm = theta.copy(), theta.copy()
        tp[k] += h
        tm[k] -= h
        fd = (O.mpnn_forward(rp, col, feat, tp, t)[1] - O.mpnn_forward(rp, col, feat, tm, t)[1]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g[k])) + 1e-9, k


def test_adamw_step():
    theta = np.array([1.0, -2.0, 0.5])
    g = np.array([0.1, -0.3, 0.0])
    m, v = np.zeros(3), np.zeros(3)
    ref = theta.copy()
    O.adamw(theta, g, m, v, 1, lr=1e-3, wd=0.01)
    mh = 0.1 * g / 0.1
    vh = 0.001 * g * g / 0.001
    ref -= 1e-3 * (mh / (np.sqrt(vh) + 1e-8) + 0.01 * ref)
    assert np.allclose(theta, ref, rtol=0, atol=1e-15)
