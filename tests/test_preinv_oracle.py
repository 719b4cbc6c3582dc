"""The oracle's restatement of the pre-inverted EoS lookup
(src/eos_interpolator.cpp:531-739): linear fields are reproduced exactly
inside every tile (the property unit_tests/eos_interpolator_test.cpp:44-135
checks for the interpolator), densities are clamped to 0.001 and taken by
absolute value. CPU only."""
import numpy as np

import preinv_oracle as P

LO, HI, N = (-2, -3, -3, -2), (0, -2, -3, -2), 6


def linear_table():
    xyz = P.node_coordinates(LO, HI, N)
    coef = np.arange(1, 12)[:, None] * np.array([1.0, -2.0, 0.5, 3.0])[None, :] / 7.0
    return xyz, xyz @ coef.T + np.arange(11) * 0.25, coef


def test_linear_fields_are_exact():
    xyz, vals, coef = linear_table()
    rng = np.random.default_rng(5)
    nt, mn, st = P.tile_geometry(LO, HI, N)
    # random points inside each decade of every axis
    pts = []
    for _ in range(200):
        q = []
        for k in range(4):
            j = rng.integers(nt[k])
            q.append(mn[k][j] * (1.0 + 8.9 * rng.random()))
        pts.append(q)
    pts = np.array(pts)
    got = P.lookup(vals, LO, HI, N, pts)
    ref = pts @ coef.T + np.arange(11) * 0.25
    assert np.max(np.abs(got - ref) / (np.abs(ref) + 1e-12)) < 1e-12


def test_clamping_and_symmetry():
    xyz, vals, coef = linear_table()
    q = np.array([[0.05, -0.004, 0.0005, 0.03], [0.05, 0.004, 0.001, 0.03]])
    got = P.lookup(vals, LO, HI, N, q)
    assert np.array_equal(got[0], got[1])
