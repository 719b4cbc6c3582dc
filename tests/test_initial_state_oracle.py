"""The oracle's initial viscous state (src/sph_workstation.cpp:1350-1430):
input_initial_shear keeps the IC's pi^{ij} (the extensive form is pi^{ij} /
sigma, and pi^{mu nu} is rebuilt from it), bulk_from_trace sets Pi = trace - p."""
import dataclasses

import numpy as np

from ccake_gb300 import ics
import oracle_py as O


def test_initial_shear_and_bulk_from_trace():
    p, rc = ics.hotspots_2d(n_side=20, n_hot=2, seed=11)
    rc = dataclasses.replace(rc, zeta_over_s=0.02)
    trace = 0.9 * p.e / 3.0
    pi = np.zeros((6, p.n))
    pi[0] = 0.05 * p.e * np.cos(3.0 * p.x)
    pi[3] = -pi[0]
    pi[1] = 0.02 * p.e
    o = O.OracleRun(p, rc)
    o.set_initial_viscous(trace, pi)
    assert o.initialize() == 0
    assert np.allclose(o.get("shv11"), pi[0], rtol=1e-13, atol=1e-16)
    assert np.allclose(o.get("shv12"), pi[1], rtol=1e-13, atol=1e-16)
    assert np.allclose(o.get("shv22"), pi[3], rtol=1e-13, atol=1e-16)
    # u = 0: pi^{00} = pi^{0i} = 0 and pi^{33} = -(pi^{11} + pi^{22}) / tau^2 = 0
    assert np.max(np.abs(o.get("shv00"))) < 1e-15 and np.max(np.abs(o.get("shv01"))) < 1e-15
    # Pi = ext Pi sigma with ext Pi = (trace - p_initial) / sigma; the
    # initial p is that of the input e (the smoothing changes s, not e)
    plain = O.OracleRun(p, rc)
    assert plain.initialize() == 0
    assert np.max(np.abs(plain.get("bulk"))) == 0.0
    assert np.all(o.get("bulk") < 0.0)
    assert o.step(3) == 0 and np.isfinite(o.get("u0")).all()
