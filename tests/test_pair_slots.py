"""The pair-slot model of ccake_gb300.traffic_model (the counts behind the
choice of per-particle candidate lists over staged cell tiles), on small
lattices with the benchmark's h = 2 dx."""
import numpy as np
import pytest

pytest.importorskip("scipy")
from ccake_gb300 import traffic_model as TM


def test_pair_slots_2d_lattice():
    xs = 0.05 * np.arange(60)
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    r = TM.pair_slots(np.column_stack([X.ravel(), Y.ravel()]), 0.1)
    # lattice points with i^2 + j^2 <= 16 other than the centre; within 2.2 h:
    # i^2 + j^2 <= 19.36
    assert r["in_2h"] == 48.0
    assert r["candidates"] == 60.0
    # the candidate list walks the fewest slots; the staged designs 2-4x more
    assert 2 * r["candidates"] < min(r["cluster"], r["stencil"], r["warp_union"])
    assert r["stencil"] <= r["warp_union"]


def test_pair_slots_3d_lattice():
    xs = 0.1 * np.arange(24)
    es = 0.06 * np.arange(20)
    E, Y, X = np.meshgrid(es, xs, xs, indexing="ij")
    r = TM.pair_slots(np.column_stack([X.ravel(), Y.ravel(), E.ravel()]), 0.2)
    assert r["in_2h"] > 400
    assert r["in_2h"] < r["candidates"] < min(r["cluster"], r["stencil"], r["warp_union"])
