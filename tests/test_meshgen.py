"""The deterministic workload generator and the DAT format."""
import os

import numpy as np

from gpupfem2_gb300 import meshgen as mg


def test_sizes():
    xy, tri = mg.unit_square(64)
    assert xy.shape == (4225, 2) and tri.shape == (8192, 3)
    xy, tri = mg.channel()
    assert xy.shape == (16705, 2) and tri.shape == (32768, 3)


def test_jitter_is_deterministic_and_bounded():
    a, ta = mg.channel()
    b, tb = mg.channel()
    assert np.array_equal(a, b) and np.array_equal(ta, tb)
    base, _ = mg.structured_rectangle(256, 64, 4.0, 1.0)
    d = np.abs(a - base).max()
    assert 0 < d <= 0.2 * (1.0 / 64) + 1e-15


def test_all_triangles_counter_clockwise():
    for xy, tri in (mg.unit_square(8), mg.channel(32, 8)):
        a, b, c = xy[tri[:, 0]], xy[tri[:, 1]], xy[tri[:, 2]]
        cr = (b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])
        assert (cr > 0).all()


def test_dat_round_trip_is_exact_and_has_no_trailing_newline(tmp_path):
    xy, tri = mg.channel(16, 4)
    p = os.path.join(tmp_path, "m.dat")
    mg.write_dat(p, xy, tri)
    raw = open(p, "rb").read()
    assert not raw.endswith(b"\n")
    xy2, tri2 = mg.read_dat(p)
    assert np.array_equal(xy, xy2) and np.array_equal(tri, tri2)


def test_splitmix64_known_values():
    # splitmix64 seeded with 0: the generator's first outputs
    z = mg.splitmix64(0, 3)
    assert [int(v) for v in z] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def test_uniform_refinement_quadruples():
    xy, tri = mg.unit_square(4)
    x2, t2 = mg.refine_uniform(xy, tri)
    assert t2.shape[0] == 4 * tri.shape[0]
    assert x2.shape[0] == xy.shape[0] + (3 * tri.shape[0] + 16) // 2
