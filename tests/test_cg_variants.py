"""The algebra behind the GPU CG variants, checked on the CPU with the oracle's IC(0)
factor (or_ic0, the reference's csric02 restated) on a small Poisson system:

* r.z = |L^{-1} r|^2 for z = L^{-T} L^{-1} r, which lets the IC(0) iteration on the
  permuted CSR arrays reduce r.z right after the forward sweep (three grid-wide steps);
* pipelined PCG (Ghysels and Vanroose, Parallel Computing 40 (2014), Algorithm 4), the
  recurrences of `k_pcg_pipe`, gives the standard PCG iterates up to rounding.

Both PCG forms below are test-local restatements of the published iterations."""
import numpy as np
import scipy.sparse as sp
from scipy.sparse.linalg import spsolve_triangular

from gpupfem2_gb300 import meshgen as mg
from oracle import oracle as O


def _system():
    xy, tri = mg.channel(24, 8, 4.0, 1.0)
    area, invJ = O.mesh_geometry(xy, tri)
    rp, col = O.csr_structure(xy.shape[0], tri)
    val, rhs = O.assemble_poisson(xy, tri, area, invJ, rp, col, 1, 1.0)
    n = rp.size - 1
    diag = np.array([rp[i] + np.searchsorted(col[rp[i]:rp[i + 1]], i) for i in range(n)])
    val[diag] += 1e-2
    A = sp.csr_matrix((val, col, rp), shape=(n, n))
    f = O.ic0(rp, col, val)
    rows = np.repeat(np.arange(n), np.diff(rp))
    low = col <= rows
    L = sp.csr_matrix((f[low], (rows[low], col[low])), shape=(n, n))
    return A, L, rhs


def _apply(L, v):
    t = spsolve_triangular(L, v, lower=True)
    return spsolve_triangular(L.T.tocsr(), t, lower=False), t


def _pcg(A, L, b, iters):
    x = np.zeros_like(b)
    r = b.copy()
    z, _ = _apply(L, r)
    p = z.copy()
    g = r @ z
    for _ in range(iters):
        q = A @ p
        a = g / (p @ q)
        x += a * p
        r -= a * q
        z, _ = _apply(L, r)
        gn = r @ z
        p = z + (gn / g) * p
        g = gn
    return x


def _pipelined(A, L, b, iters):
    x = np.zeros_like(b)
    r = b.copy()
    u, _ = _apply(L, r)
    w = A @ u
    zv = np.zeros_like(b)
    q = np.zeros_like(b)
    s = np.zeros_like(b)
    p = np.zeros_like(b)
    g_old = a_old = None
    for i in range(iters + 1):
        g, d = r @ u, w @ u
        if i == iters:
            break
        m, _ = _apply(L, w)
        nv = A @ m
        if i == 0:
            beta, a = 0.0, g / d
        else:
            beta = g / g_old
            a = g / (d - beta * g / a_old)
        zv = nv + beta * zv
        q = m + beta * q
        s = w + beta * s
        p = u + beta * p
        x += a * p
        r -= a * s
        u -= a * q
        w -= a * zv
        g_old, a_old = g, a
    return x


def test_rz_equals_squared_forward_result():
    A, L, rhs = _system()
    r = rhs - A @ (0.3 * np.ones_like(rhs))
    z, t = _apply(L, r)
    assert abs(r @ z - t @ t) <= 1e-12 * abs(r @ z)


def test_pipelined_pcg_follows_standard_pcg():
    A, L, rhs = _system()
    for k in (1, 5, 20):
        xs, xp = _pcg(A, L, rhs, k), _pipelined(A, L, rhs, k)
        assert np.linalg.norm(xp - xs) <= 1e-9 * np.linalg.norm(xs)
    # both reach the solution
    x = _pipelined(A, L, rhs, 200)
    assert np.linalg.norm(rhs - A @ x) <= 1e-9 * np.linalg.norm(rhs)
