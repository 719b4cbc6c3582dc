"""The factorised 3-D kernel on the GPU against the CPU oracle.

With the reference's factorized_kernel option (src/kernel.cpp:129-170) the
3-D kernel is W_2D(r_perp, hT) W_1D(|d eta|, hEta) and its gradient
(dW_2D W_1D along the transverse separation, W_2D dW_1D along d eta); the
neighbour list keeps its 2 hT sphere (src/system_state.cpp:650-719). The
smoothing, the gradient sums (with and without the diffusion sector) and
everything after them run through it in the FP64 form, held to the FP64
form's bar (1e-10 relative, against 1e-6 of a field's range where it
crosses zero, 1e-5 for the diffusion currents).
"""
import dataclasses

import numpy as np
import pytest

from ccake_gb300 import api, ics
import oracle_py as O

pytestmark = pytest.mark.gpu

RTOL = 1e-10
KAPPA = (0.3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.3)


def relerr(a, b, floor=1e-6):
    scale = np.abs(b) + floor * np.max(np.abs(b)) + 1e-300
    return float(np.max(np.abs(a - b) / scale))


def csr_rows(off, idx):
    return [tuple(idx[off[i]:off[i + 1]]) for i in range(len(off) - 1)]


@pytest.mark.parametrize("h_eta,diffusion", [(0.15, False), (0.25, False), (0.15, True)])
def test_factorized_kernel_parity(h_eta, diffusion):
    p, rc = ics.hotspots_3d(n_xy=16, n_eta=12, n_hot=4, seed=3)
    rc = dataclasses.replace(rc, factorized_kernel=1, hEta=h_eta)
    if diffusion:
        rc = dataclasses.replace(rc, using_diffusion=1, kappa_over_T2=KAPPA)
    gpu = api.GpuHydro(rc)
    gpu.load(p)
    orc = O.OracleRun(p, rc)
    go, gi = gpu.neighbours()
    oo, oi = orc.neighbours()
    assert csr_rows(go, gi) == csr_rows(oo, oi)
    gpu.initialize()
    assert orc.initialize() == 0
    for f in ("sigma_lab", "T", "e"):
        assert relerr(gpu.get(f), orc.get(f)) < RTOL, f
    gpu.step(3)
    assert orc.step(3) == 0
    fields = ["x", "y", "eta", "u0", "u1", "u2", "ext_s", "T", "e", "sigma_lab", "ext_shv0", "ext_shv2",
              "ext_shv4", "shv33", "Ez"]
    if diffusion:
        fields += ["ext_B", "qB1", "qB3"]
    for f in fields:
        # the currents start at zero and cross it: against 1e-5 of their range,
        # as in the diffusion sector's own parity tests
        floor = 1e-5 if f[0] == "q" else 1e-6
        assert relerr(gpu.get(f), orc.get(f), floor) < RTOL, f
    # the option changes the evolution: the run with the spherical kernel differs
    plain = api.GpuHydro(dataclasses.replace(rc, factorized_kernel=0))
    plain.load(p)
    plain.initialize()
    plain.step(3)
    assert relerr(plain.get("u2"), orc.get("u2")) > 1e-6


def test_factorized_kernel_rejected_in_the_mixed_form():
    p, rc = ics.hotspots_3d(n_xy=16, n_eta=12, n_hot=4, seed=3)
    with pytest.raises(api.CcakeError):
        api.GpuHydro(dataclasses.replace(rc, factorized_kernel=1, hEta=0.15, precision=1))
