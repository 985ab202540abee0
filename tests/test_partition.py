"""The row partition of the partitioned CG solve (pf2_graph_parts, host code): every row in
one of the parts, part sizes within one row per bisection level of each other, the same
parts on every call, a compact cut on the cylinder meshes, and disconnected graphs."""
import ctypes as C

import numpy as np
import pytest

import gpupfem2_gb300 as g
from gpupfem2_gb300 import meshgen as mg
from oracle import oracle as O


def parts(rp, col, P):
    f = g.lib().pf2_graph_parts
    f.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    f.restype = C.c_int
    rp = np.ascontiguousarray(rp, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    out = np.full(rp.size - 1, -1, np.int32)
    st = f(rp.size - 1, rp.ctypes.data, col.ctypes.data, P, out.ctypes.data)
    return st, out


def boundary_fraction(rp, col, part):
    rows = np.repeat(np.arange(rp.size - 1), np.diff(rp))
    bnd = np.zeros(rp.size - 1, bool)
    bnd[rows[part[rows] != part[col]]] = True
    return bnd.mean()


@pytest.mark.parametrize("P", [1, 2, 7, 152])
def test_parts_cover_the_rows_and_balance(P):
    xy, tri = mg.cylinder_channel(nxh=350, nyh=400, nr=12)
    rp, col = O.csr_structure(xy.shape[0], tri)
    st, part = parts(rp, col, P)
    assert st == 0
    sizes = np.bincount(part, minlength=P)
    assert part.min() == 0 and part.max() == P - 1 and sizes.sum() == rp.size - 1
    levels = int(np.ceil(np.log2(P))) if P > 1 else 0
    assert sizes.max() - sizes.min() <= max(1, levels)
    assert np.array_equal(part, parts(rp, col, P)[1])


def test_cut_is_compact_on_the_cylinder_mesh():
    """152 parts (one per SM) of the quarter-size cylinder mesh's 125,364 nodes: 14 % of
    the rows have a neighbour in another part (measured 0.140); one part per row band of
    a column-by-column numbering would cut most rows."""
    xy, tri = mg.cylinder_channel(nxh=350, nyh=400, nr=12)
    rp, col = O.csr_structure(xy.shape[0], tri)
    st, part = parts(rp, col, 152)
    assert st == 0 and boundary_fraction(rp, col, part) < 0.16


def test_disconnected_graph():
    """Two separate channels in one pattern: the breadth-first order continues in the
    other component, and every part is still filled."""
    xy, tri = mg.channel(16, 4, 4.0, 1.0)
    n = xy.shape[0]
    tri2 = np.concatenate([tri, tri + n])
    rp, col = O.csr_structure(2 * n, tri2)
    st, part = parts(rp, col, 5)
    assert st == 0
    sizes = np.bincount(part, minlength=5)
    assert sizes.min() > 0 and sizes.sum() == 2 * n


def test_bad_input_is_rejected():
    rp = np.array([0, 1], np.int32)
    col = np.array([0], np.int32)
    assert parts(rp, col, 0)[0] == g.BAD_INPUT
    assert parts(rp, np.array([3], np.int32), 1)[0] == g.BAD_INPUT
