"""Pre-inverted (s, rho) -> thermodynamics tables on the GPU
(ccake_preinverted_*): the generated nodes equal the batched inversion at
the node densities from the generator's seed (same algorithm, bit for bit),
lookups equal the oracle's restatement of the reference's interpolation on
the same tables (bit for bit), interpolation error against the inversion,
and a hydro run that takes its thermodynamics from the tables."""
import numpy as np
import pytest

from ccake_gb300 import api, ics
import preinv_oracle as P

pytestmark = pytest.mark.gpu

LO, HI = (-1, -2, -3, -2), (0, -1, -3, -2)


def gpu_cdiag():
    return api.GpuHydro(ics.RunConfig(eos_kind=1, thermo_mode=1))


def test_nodes_equal_batched_inversion_and_lookup_equals_oracle():
    g = gpu_cdiag()
    N = 5
    g.preinverted_build(LO, HI, N)
    vals = g.preinverted_values()
    xyz = P.node_coordinates(LO, HI, N)
    assert vals.shape == (len(xyz), 11)
    seeds = np.tile([750.0 / 197.0, 0, 0, 0], (len(xyz), 1))
    x, th, st, _ = g.eos_invert(1, xyz, seeds)
    assert np.all(st >= 0)
    # th16: T muB muS muQ p s rhoB rhoS rhoQ e w cs2 dwds dwdB dwdS dwdQ
    ref = th[:, [0, 1, 3, 2, 9, 4, 11, 12, 13, 15, 14]]
    assert np.array_equal(vals, ref)
    rng = np.random.default_rng(3)
    q = np.column_stack([10 ** rng.uniform(-1.2, 1.1, 300), rng.choice([-1, 1], 300) * 10 ** rng.uniform(-2.5, 0.2, 300),
                         10 ** rng.uniform(-3.5, -2.5, 300), 10 ** rng.uniform(-2, -1.05, 300)])
    assert np.array_equal(g.preinverted_lookup(q), P.lookup(vals, LO, HI, N, q))


def test_interpolation_error_against_inversion():
    g = gpu_cdiag()
    g.preinverted_build(LO, HI, 20)
    rng = np.random.default_rng(4)
    n = 2000
    q = np.column_stack([10 ** rng.uniform(-1, 0.999, n), 10 ** rng.uniform(-2, -0.001, n),
                         np.full(n, 10 ** -2.5), 10 ** rng.uniform(-2, -1.001, n)])
    look = g.preinverted_lookup(q)
    x, th, st, _ = g.eos_invert(1, q, np.tile([750.0 / 197.0, 0, 0, 0], (n, 1)))
    assert np.all(st >= 0)
    relT = np.abs(look[:, 0] / th[:, 0] - 1)
    rele = np.abs(look[:, 4] / th[:, 9] - 1)
    # the generator's grid steps by half the decade's lower edge (10^(e+1) / 20),
    # so the interpolation is coarsest at the bottom of each decade
    assert relT.max() < 1e-2 and rele.max() < 3e-2
    assert np.median(relT) < 1e-3


def test_hydro_with_preinverted_tables():
    p, rc = ics.hotspots_2d(n_side=48, n_hot=6, seed=7)
    ref = api.GpuHydro(rc)
    ref.load(p)
    ref.initialize()
    ref.step(5)
    g = api.GpuHydro(rc)
    g.load(p)
    g.initialize()
    g.preinverted_build((-3, -3, -3, -3), (1, 0, 0, 0), 12)
    g.preinverted_use(True)
    g.step(5)
    T, Tr = g.get("T"), ref.get("T")
    assert np.all(np.isfinite(T))
    assert np.median(np.abs(T / Tr - 1)) < 1e-2
    g.preinverted_use(False)
    g.step(1)
