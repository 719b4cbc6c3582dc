"""Diffusion sector on the GPU against the CPU oracle, through the C ABI.

The sector (src/eom_default.cpp:1415-1817 with its coupling into du/dt and
dN/dt, the diffusion sums of src/sph_workstation.cpp:909-967, the alpha
derivatives of src/eos.cpp:337-493, the coefficients of
src/transport_coefficients.cpp and the regulator of
src/sph_workstation.cpp:132-218) runs in the FP64 form. Tolerance: 1e-10
relative per field as in the other parity tests, against the field's own
range where it crosses zero (sums whose terms cancel against 1e-4 of it).
"""
import dataclasses

import numpy as np
import pytest

from ccake_gb300 import api, ics
import oracle_py as O

pytestmark = pytest.mark.gpu

RTOL = 1e-10
GRAD_FLOOR = 1e-4


def relerr(a, b, floor=1e-6):
    scale = np.abs(b) + floor * np.max(np.abs(b)) + 1e-300
    return float(np.max(np.abs(a - b) / scale))


KAPPA = (0.3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.3)


def hotspots_diffusion(dim=2):
    # B and Q carried (rhoB = e/20, rhoQ = 0.4 rhoB), conformal-diagonal EoS,
    # exact Hessian inverse; kappa/T^2 = 0.3 for B and Q (S carries no charge)
    if dim == 2:
        p, rc = ics.hotspots_2d(n_side=40, n_hot=5, seed=11)
    else:
        p, rc = ics.hotspots_3d(n_xy=16, n_eta=12, n_hot=4, seed=3)
    return p, dataclasses.replace(rc, using_diffusion=1, kappa_over_T2=KAPPA)


def baryon_coth():
    # baryon only, conformal EoS with the reference derivative chain,
    # kappa_B from the coth form with tau_q = C_B / T, the regulator on and an
    # initial current part of which it caps
    p, rc = ics.hotspots_2d(n_side=40, n_hot=5, seed=13)
    # e above the regulator's e0 = 0.1 GeV/fm^3 leaves part of the current
    # below its cap; rhoB = 10 e[GeV/fm^3] of the unscaled field puts mu_B/T
    # above the 1e-2 floor of the coth form everywhere
    p = dataclasses.replace(p, e=50.0 * p.e, rhoB=200.0 * p.rhoB, rhoQ=np.zeros_like(p.rhoQ))
    rc = dataclasses.replace(rc, eos_kind=0, thermo_mode=0, using_diffusion=1, diffusion_mode=2,
                             diffusion_relax_mode=1, C_B=0.4, diffusion_regulator=1)
    q = np.zeros((12, p.n))
    q[1] = 12.0 * p.rhoB * np.cos(6.0 * p.x)     # q_B^x
    q[2] = 6.0 * p.rhoB * np.sin(5.0 * p.y)      # q_B^y
    return p, rc, q


def make_pair(p, rc, q=None):
    gpu = api.GpuHydro(rc)
    gpu.load(p)
    orc = O.OracleRun(p, rc)
    if q is not None:
        gpu.set_initial_diffusion(q)
        for c, C in enumerate("BSQ"):
            for m in range(4):
                orc.set(f"in_q{C}{m}", q[4 * c + m])
    gpu.initialize()
    assert orc.initialize() == 0
    return gpu, orc


DIFF_PHASE_FIELDS = ["grad_alpha0B", "grad_alpha1B", "grad_alpha0Q", "grad_alpha1Q", "div_qaB", "div_qaQ",
                     "grad_qaB", "grad_qaQ"]


@pytest.mark.parametrize("case", ["hotspots", "coth"])
def test_diffusion_phase_parity(case):
    if case == "hotspots":
        p, rc = hotspots_diffusion()
        gpu, orc = make_pair(p, rc)
    else:
        p, rc, q = baryon_coth()
        gpu, orc = make_pair(p, rc, q)
    gpu.step(2)
    assert orc.step(2) == 0
    gpu.phase("smooth_fields")
    for ph in ("neighbours", "velocity", "smooth_fields"):
        orc.phase(ph)
    gpu.phase("update_thermo")
    for ph in ("thermo", "reset_pi", "regulate_diffusion"):
        orc.phase(ph)
    # alpha derivatives and q^mu (after the regulator)
    for k in (0, 2, 3, 5, 9, 11):
        assert relerr(gpu.get(f"dalpha{k}"), orc.get(f"dalpha{k}")) < RTOL, k
    for f in ("qB0", "qB1", "qB2", "qQ0", "qQ1", "qQ2"):
        assert relerr(gpu.get(f), orc.get(f), 1e-5) < RTOL, f
    gpu.phase("update_viscosities")
    orc.phase("viscosities")
    gpu.phase("time_derivatives")
    orc.phase("gradients")
    orc.phase("eom")
    fields = ["du_dt0", "du_dt1", "d_ext_s", "d_ext_B", "d_ext_qB0", "d_ext_qB1", "d_ext_qB2"]
    if case == "hotspots":
        fields += ["d_ext_Q", "d_ext_qQ0", "d_ext_qQ1"] + DIFF_PHASE_FIELDS
    else:
        fields += [f for f in DIFF_PHASE_FIELDS if f.endswith("B")]
    for f in fields:
        assert relerr(gpu.get(f), orc.get(f), GRAD_FLOOR) < RTOL, f


@pytest.mark.parametrize("case", ["hotspots2d", "hotspots3d", "coth", "cartesian2d", "cartesian3d"])
def test_diffusion_evolution_parity(case):
    # cartesian: the twin of src/eom_cartesian.cpp:1327-1722 (coord = 1)
    q = None
    if case == "coth":
        p, rc, q = baryon_coth()
        steps = 10
    else:
        p, rc = hotspots_diffusion(3 if case.endswith("3d") else 2)
        steps = 3 if case.endswith("3d") else 10
        if case.startswith("cartesian"):
            rc = dataclasses.replace(rc, coord=1)
    gpu, orc = make_pair(p, rc, q)
    b0 = gpu.get("ext_B")
    gpu.step(steps)
    assert orc.step(steps) == 0
    fields = ["x", "y", "u0", "u1", "ext_s", "ext_B", "T", "e", "muB", "ext_qB0", "ext_qB1", "qB0", "qB1"]
    if case != "coth":
        fields += ["ext_Q", "ext_qQ0", "ext_qQ1", "ext_shv0", "shv00"]
    if case.endswith("3d"):
        fields += ["eta", "u2", "ext_qB2"]
    for f in fields:
        floor = 1e-5 if f[0] in "uq" or f.startswith("ext_q") else 1e-6
        assert relerr(gpu.get(f), orc.get(f), floor) < RTOL, f
    # the sector moves charge: the extensive densities are no longer constant
    assert np.max(np.abs(gpu.get("ext_B") - b0)) > 1e-9 * np.max(np.abs(b0))
    tg, to = gpu.totals(), orc.totals()
    for k in ("S", "B", "Q", "E"):
        assert abs(tg[k] - to[k]) <= 1e-10 * (abs(to[k]) + 1e-30), k


def test_diffusion_numbers_and_system_state(tmp_path):
    p, rc = hotspots_diffusion()
    gpu, orc = make_pair(p, rc)
    gpu.step(3)
    assert orc.step(3) == 0
    gpu.hydro_numbers()
    for f in ("kn_diffB", "kn_diffQ", "ire_diffB", "ire_diffQ", "bulk_knudsen", "theta"):
        assert relerr(gpu.get(f), orc.get(f), 1e-5) < 1e-9, f
    path = tmp_path / "system_state_3.dat"
    gpu.write_system_state(str(path))
    rows = [ln.split() for ln in path.read_text().splitlines()[1:]]
    assert len(rows) == p.n
    # the last six numbers of a row: Knudsen B S Q, inverse Reynolds B S Q
    kn = np.array([float(r[-6]) for r in rows])
    ire = np.array([float(r[-3]) for r in rows])
    assert np.allclose(kn, gpu.get("kn_diffB"), rtol=1e-5, atol=0)
    assert np.allclose(ire, gpu.get("ire_diffB"), rtol=1e-5, atol=0)
    assert np.max(kn) > 0.0


def test_diffusion_off_matches_plain_and_rejects_unsupported():
    # with kappa = 0 and no initial current the sector leaves the evolution as
    # it is without it; the DNMR mode is rejected
    p, rc = ics.hotspots_2d(n_side=32, n_hot=4, seed=5)
    plain = api.GpuHydro(rc)
    plain.load(p)
    plain.initialize()
    plain.step(5)
    zero = api.GpuHydro(dataclasses.replace(rc, using_diffusion=1))
    zero.load(p)
    zero.initialize()
    zero.step(5)
    for f in ("x", "u0", "e", "ext_B"):
        assert relerr(zero.get(f), plain.get(f), 1e-5) < 1e-12, f
    with pytest.raises(api.CcakeError):
        api.GpuHydro(dataclasses.replace(rc, using_diffusion=1, diffusion_mode=1))


def test_diffusion_freeze_out_rows():
    # the hypersurface rows carry the snapshot's q^mu in their twelve
    # diffusion columns (FreezeOut diffout, src/output.cpp:463-474)
    p, rc = ics.hotspots_2d(n_side=40, n_hot=4, seed=11)
    rc = dataclasses.replace(rc, using_diffusion=1, kappa_over_T2=KAPPA, freeze_out_T=0.3 / 0.1973269804,
                             particlization=1, surface=1)
    gpu, orc = make_pair(p, rc)
    for _ in range(3):
        gpu.step(4)
        assert orc.step(4) == 0
    rg, ro = gpu.freeze_out_rows(), orc.freeze_out_rows()
    assert ro.shape[0] >= 3 and rg.shape == ro.shape
    assert np.array_equal(rg[:, :2], ro[:, :2])
    scale = np.abs(ro) + 1e-6 * np.max(np.abs(ro), axis=0) + 1e-300
    assert np.max(np.abs(rg - ro) / scale) < 1e-9
    q = ro[:, -13:-1]
    assert np.max(np.abs(q[:, 1:3])) > 0.0      # q_B^x, q_B^y
