"""The multicolour order of the ILU(0)/IC(0) sweeps (pf2_multicolour_order, host code):
a proper colouring, colours contiguous in the permutation, and Kempe-chain trimming of
greedy colouring's tail (four colours on the cylinder meshes)."""
import ctypes as C

import numpy as np
import pytest

import gpupfem2_gb300 as g
from gpupfem2_gb300 import meshgen as mg
from oracle import oracle as O


def order(rp, col, kempe):
    n = rp.size - 1
    L = g.lib()
    f = L.pf2_multicolour_order
    f.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    rp = np.ascontiguousarray(rp, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    perm = np.empty(n, np.int32)
    nc, ns = C.c_int(), C.c_int()
    assert f(n, rp.ctypes.data, col.ctypes.data, int(kempe), perm.ctypes.data, C.byref(nc), C.byref(ns), None) == 0
    starts = np.empty(ns.value, np.int32)
    assert f(n, rp.ctypes.data, col.ctypes.data, int(kempe), perm.ctypes.data, C.byref(nc), C.byref(ns),
             starts.ctypes.data) == 0
    return perm, nc.value, starts


def check_groups(rp, col, perm, starts, independent):
    n = rp.size - 1
    assert np.array_equal(np.sort(perm), np.arange(n))
    assert starts[0] == 0 and starts[-1] == n and np.all(np.diff(starts) > 0)
    group = np.empty(n, np.int64)
    for gi in range(starts.size - 1):
        group[perm[starts[gi]:starts[gi + 1]]] = gi
        if independent:  # one colour per group: its rows keep their order
            assert np.all(np.diff(perm[starts[gi]:starts[gi + 1]]) > 0)
    if independent:  # no edge inside a group: each group is one colour
        rows = np.repeat(np.arange(n), np.diff(rp))
        off = rows != col
        assert not np.any(group[rows[off]] == group[col[off]])


@pytest.mark.parametrize("name,make", [("quarter", lambda: mg.cylinder_channel(nxh=350, nyh=400, nr=12)),
                                       ("channel", lambda: mg.channel())])
def test_kempe_gives_four_colours_on_the_2d_meshes(name, make):
    xy, tri = make()
    rp, col = O.csr_structure(xy.shape[0], tri)
    perm, nc, starts = order(rp, col, kempe=True)
    assert nc <= 4 and starts.size == nc + 1
    check_groups(rp, col, perm, starts, independent=True)


def test_greedy_tail_is_swept_with_the_last_colour():
    xy, tri = mg.cylinder_channel(nxh=350, nyh=400, nr=12)
    rp, col = O.csr_structure(xy.shape[0], tri)
    perm, nc, starts = order(rp, col, kempe=False)
    assert nc == 6 and starts.size == 5  # two thin tail colours merged into the fourth group
    check_groups(rp, col, perm, starts, independent=False)
    # the permutation is greedy colouring's, colour by colour
    n = rp.size - 1
    color = -np.ones(n, int)
    for i in range(n):
        nb = col[rp[i]:rp[i + 1]]
        used = set(color[nb[nb < i]])
        c = 0
        while c in used:
            c += 1
        color[i] = c
    assert np.array_equal(perm, np.lexsort((np.arange(n), color)))


def test_3d_pattern_is_coloured_properly():
    xyz, tet = mg.box_tets(8, 6, 4)
    rp, col = O.csr_structure_3d(xyz.shape[0], tet)
    perm, nc, starts = order(rp, col, kempe=True)
    # groups after the trimmed colours are single colours as well
    check_groups(rp, col, perm, starts, independent=True)
    assert nc == starts.size - 1


@pytest.mark.parametrize("name,make", [("quarter", lambda: mg.cylinder_channel(nxh=350, nyh=400, nr=12)),
                                       ("channel", lambda: mg.channel()),
                                       ("square", lambda: mg.unit_square(64))])
@pytest.mark.parametrize("kempe", [True, False])
def test_oracle_restates_the_engine_colouring(name, make, kempe):
    """The oracle's multicolour order (its restatement of greedy colouring with Kempe
    trimming) is the engine's permutation, so the oracle can run the pressure solve
    with the engine's IC(0)/ILU(0) ordering."""
    xy, tri = make()
    rp, col = O.csr_structure(xy.shape[0], tri)
    perm, nc, starts = order(rp, col, kempe=kempe)
    operm, ostarts = O.multicolour_order(rp, col, kempe=kempe)
    assert np.array_equal(perm, operm)
    if kempe:
        assert np.array_equal(starts, ostarts)
