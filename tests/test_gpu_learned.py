"""What the trained network of the learned pressure start gains (no reference counterpart).

The learned start (PF2_X0_LEARNED, csrc/guess.cu) is x0 = p^n + D c, D = [d0, h_1 .. h_8]:
d0 the network's predicted increment, h_k the last pressure increments of the run, c the
Galerkin coefficients in the energy norm.  The network's output layer starts at zero, so
an untrained network gives d0 = 0 and the start is the projection onto the history alone:
the method without the network.

On the 64 x 16 channel (Scheme A, one outer iteration, Jacobi CG to ||r|| <= 1e-8 ||b||)
three runs of 40 steps from rest are compared over steps 21-40:

* the previous pressure as the start (PF2_X0_GIVEN);
* the learned start with the network untrained (rate 0): the history projection;
* the learned start with the network trained online on steps 1-20 (AdamW, rate 1e-3).

And the network itself, trained by the library's own kernels (pf2_mpnn_train_step) on the
same 20 steps' (features, increment) pairs, against the increments of steps 21-40 that
it has not seen.

Measured on a GB300: held-out error of the trained network 0.70 of the increment's norm
(the untrained one 1.0); pressure iterations over steps 21-40: 4,150 from the previous
pressure, 3,731 from the history projection (89.9 %), 3,723 with the trained network (-8);
start residual ||b - A x0|| / ||b - A p^n|| 0.0238 with the history alone, 0.0237 with the
trained network.  So the trained network predicts the increment, but the history projection already
holds the start's gains (its energy-norm error is ~1e-5 of the previous pressure's) and
the network's direction adds almost nothing to it; the test asserts exactly that much.
"""
import numpy as np
import pytest
import torch

import gpupfem2_gb300 as g
from gpupfem2_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu

STEPS, LEARN = 40, 20


def _case():
    xy, tri = mg.channel(64, 16, 4.0, 1.0)
    bu, bv, bp = mg.channel_boundary_nodes(xy, 4.0, 1.0)
    m = g.Mesh2D.from_arrays(xy, tri)
    m.set_channel_boundary_ids(4.0, 1.0)
    return xy, m, bu, bv, bp


def _params(x0, rate):
    return g.default_params(rho=1.0, mu=0.01, dt=0.005, scheme=0, substeps=3, level=3, n_outer=1,
                            pressure_precond=0, pressure_criterion=1, pressure_x0=x0, learn_steps=LEARN,
                            learn_rate=rate)


def _wrap(ptr, n):
    class _A:
        __cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False), "version": 3}

    return torch.as_tensor(_A(), device="cuda")


def _run(m, bu, bv, bp, x0, rate, record=False):
    eng = g.FlowEngine(m, _params(x0, rate), bu, bv, bp)
    eng.seed()
    its, ratios, used, pairs = [], [], 0, []
    p_prev = np.zeros(m.nv)
    for s in range(STEPS):
        p = eng.field("p")
        eng.step()
        inf = eng.info()
        assert inf.converged == 1 and inf.status == 0
        its.append(inf.it_pressure[0])
        if s >= LEARN:
            used += inf.guess_used
            if inf.guess_residual[0] > 0:
                ratios.append(inf.guess_residual[1] / inf.guess_residual[0])
        if record:
            _, rhs = eng.system(2)
            pairs.append((p_prev, p, _wrap(rhs, m.nv).cpu().numpy().copy(), eng.field("p")))
        p_prev = p
    return np.array(its), ratios, used, pairs


def _features(xy, p_prev, p, b):
    """The network's inputs as csrc/guess.cu forms them."""
    def scale(a):  # max |a|, or 1 for a zero field
        s = np.abs(a).max()
        return s if s > 1e-300 else 1.0

    lo = xy.min(0)
    L = max(np.ptp(xy[:, 0]), np.ptp(xy[:, 1]))
    d = p - p_prev
    sd = scale(d)
    f = np.stack([(xy[:, 0] - lo[0]) / L, (xy[:, 1] - lo[1]) / L, b / scale(b), p / scale(p), d / sd], 1)
    return torch.tensor(f.astype(np.float32).ravel(), device="cuda"), sd


def test_what_the_trained_network_gains(cuda):
    xy, m, bu, bv, bp = _case()
    it_prev, _, used_prev, pairs = _run(m, bu, bv, bp, g.X0_GIVEN, 0.0, record=True)
    it_hist, ratio_hist, used_hist, _ = _run(m, bu, bv, bp, g.X0_LEARNED, 0.0)
    it_net, ratio_net, used_net, _ = _run(m, bu, bv, bp, g.X0_LEARNED, 1e-3)

    # the network alone: trained on steps 1-20 by the library's kernels, tested on 21-40
    nets = {"trained": g.LearnedGuess(m, seed=0x5EED), "untrained": g.LearnedGuess(m, seed=0x5EED)}
    for p_prev, p, b, p_new in pairs[:LEARN]:
        f, sd = _features(xy, p_prev, p, b)
        nets["trained"].train_step(f, torch.tensor(((p_new - p) / sd).astype(np.float32), device="cuda"), lr=1e-3)
    err = {k: [] for k in nets}
    for p_prev, p, b, p_new in pairs[LEARN:]:
        f, sd = _features(xy, p_prev, p, b)
        want = (p_new - p) / sd
        for k, net in nets.items():
            y = torch.empty(m.nv, dtype=torch.float32, device="cuda")
            net.forward(f, y)
            err[k].append(np.linalg.norm(y.cpu().numpy() - want) / np.linalg.norm(want))
    e_tr, e_un = float(np.mean(err["trained"])), float(np.mean(err["untrained"]))

    n_prev, n_hist, n_net = int(it_prev[LEARN:].sum()), int(it_hist[LEARN:].sum()), int(it_net[LEARN:].sum())
    print("\nheld-out increment error: trained %.3f, untrained %.3f" % (e_tr, e_un))
    print("pressure iterations, steps %d-%d: previous pressure %d, history projection (untrained) %d (%.1f %%), "
          "with the trained network %d (%.1f %% of the previous; %+d against the history alone)"
          % (LEARN + 1, STEPS, n_prev, n_hist, 100.0 * n_hist / n_prev, n_net, 100.0 * n_net / n_prev,
             n_net - n_hist))
    print("start residual ||b - A x0|| / ||b - A p^n|| (mean): history %.4f, trained network %.4f; "
          "steps where the network's direction got a coefficient: %d of %d"
          % (np.mean(ratio_hist), np.mean(ratio_net), used_net, STEPS - LEARN))

    # the untrained network's output is zero: its start is the history projection alone
    assert e_un == pytest.approx(1.0, abs=1e-6) and used_hist == 0 and used_prev == 0
    # training teaches the network the increments of steps it has not seen
    assert e_tr < 0.8
    # the history projection saves iterations against the previous pressure ...
    assert n_hist <= 0.95 * n_prev
    # ... and the trained network's direction keeps that (it costs no iterations)
    assert n_net <= n_hist + max(2, 0.02 * n_hist)
