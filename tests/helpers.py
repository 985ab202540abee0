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
