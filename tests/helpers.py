"""Shared helpers of the parity tests: workloads and comparisons."""
import numpy as np

from gpupfem2_gb300 import meshgen as mg


def poisson_square(n=64):
    xy, tri = mg.unit_square(n)
    bcs = mg.square_boundary_nodes(xy)
    return xy, tri, bcs


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def csr_dense_rows(rp, col, val):
    return [dict(zip(col[rp[i]:rp[i + 1]].tolist(), val[rp[i]:rp[i + 1]].tolist())) for i in range(rp.size - 1)]


def shadow_breakdown_system(nx=32, ny=8):
    """A nonsymmetric system on which BiCGStab's shadow residual rhat = r0 becomes
    orthogonal to r after the first iteration: the Poisson matrix of a channel (plus a
    small shift) with the rows of the boundary nodes made identity rows while their
    columns stay in the other rows, and a right-hand side on those rows alone.  With the
    Jacobi preconditioner (1 on those rows) the first step gives alpha = 1 and zeroes r
    on the boundary rows, the whole support of rhat.  The same structure arises in the
    first velocity prediction of a flow from rest when the Dirichlet columns are kept.
    Returns (xy, tri, rowptr, col, val, rhs)."""
    from oracle import oracle as O
    xy, tri = mg.channel(nx, ny, 4.0, 1.0)
    area, invJ = O.mesh_geometry(xy, tri)
    rp, col = O.csr_structure(xy.shape[0], tri)
    val, _ = O.assemble_poisson(xy, tri, area, invJ, rp, col, 1, 1.0)
    n = rp.size - 1
    bnodes = [i for i, _ in mg.channel_boundary_nodes(xy, 4.0, 1.0)[0]]
    rhs = np.zeros(n)
    g = mg.uniform_pm1(5, n)
    for i in range(n):
        val[rp[i] + np.searchsorted(col[rp[i]:rp[i + 1]], i)] += 1e-2
    for i in bnodes:
        val[rp[i]:rp[i + 1]] = 0.0
        val[rp[i] + np.searchsorted(col[rp[i]:rp[i + 1]], i)] = 1.0
        rhs[i] = g[i]
    return xy, tri, rp, col, val, rhs
