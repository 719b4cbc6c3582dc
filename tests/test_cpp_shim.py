"""The C++ shim (include/ccake_gpu.hpp) compiles against the C ABI, links
against libccake_gpu.so and, on a GPU, runs a short event through the
reference-shaped classes."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = r'''
#include "ccake_gpu.hpp"
#include <cmath>
#include <cstdio>
#include <vector>
int main() {
  ccake_config cfg{};
  cfg.dim = 2; cfg.eos_kind = 0; cfg.zeta_mode = 1; cfg.zeta_cs2_p = 2.0;
  cfg.hT = 0.1; cfg.t0 = 1.0; cfg.dt = 0.001; cfg.eos_c = 15.6269 / 3.0;
  cfg.eos_T0 = cfg.eos_muB0 = cfg.eos_muQ0 = cfg.eos_muS0 = 1.0;
  cfg.xmin = cfg.ymin = -1.0; cfg.etamin = -0.1; cfg.freeze_out_T = 150.0 / 197.3269804;
  const int ns = 40; std::vector<double> x, y, e, z;
  for (int j = 0; j < ns; j++) for (int i = 0; i < ns; i++) {
    double xx = -1.0 + 0.05 * i, yy = -1.0 + 0.05 * j;
    x.push_back(xx); y.push_back(yy); z.push_back(0.0);
    e.push_back(15.6269 * std::pow(1.0 + 0.1 * std::exp(-(xx * xx + yy * yy)), 4));
  }
  ccake_particles_soa soa{(int64_t)x.size(), x.data(), y.data(), nullptr, e.data(), nullptr, nullptr, nullptr,
                          z.data(), z.data(), nullptr};
  ccake::gpu::BSQHydro hydro(cfg, 1.0 + 5.5 * 0.001);
  hydro.read_in_initial_conditions(soa);
  hydro.initialize_hydrodynamics();
  hydro.run();
  ccake_totals tot = hydro.system().conservation();
  std::printf("t=%.6f S=%.12g E=%.12g\n", hydro.system().t(), tot.S, tot.E);
  return (std::fabs(hydro.system().t() - 1.006) < 1e-12) ? 0 : 1;
}
'''


def _compile(tmp_path, link):
    src = tmp_path / "shim.cpp"
    src.write_text(SRC)
    exe = tmp_path / "shim"
    cmd = ["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src)]
    if link:
        libdir = os.path.join(ROOT, "ccake_gb300", "_build")
        cmd += ["-o", str(exe), "-L", libdir, "-lccake_gpu", "-Wl,-rpath," + libdir]
    else:
        cmd += ["-fsyntax-only"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_shim_compiles(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    _compile(tmp_path, link=False)


@pytest.mark.gpu
def test_shim_runs_event(tmp_path):
    from ccake_gb300 import build
    build.build()
    exe = _compile(tmp_path, link=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "t=1.006" in out.stdout


def _write_ic_29(path, p, rc):
    """A 29-column IC file (initial diffusion) of a 2-D hot-spot event with
    an initial shear, a bulk trace and initial baryon currents, in the
    reference's units (GeV/fm^3 for e, the trace and pi^{ij})."""
    hc = 0.1973269804
    trace = 0.9 * p.e / 3.0
    pixx = 0.05 * p.e * np.cos(3.0 * p.x)
    pixy = 0.02 * p.e * np.sin(2.0 * p.y)
    qx = 0.5 * p.rhoB * np.cos(4.0 * p.y)
    with open(path, "w") as fh:
        fh.write(f"#0 0.05 0.05 0.1 0 {float(rc.xmin)!r} {float(rc.ymin)!r} -0.1\n")
        for i in range(p.n):
            row = [p.x[i], p.y[i], 0.0, p.e[i] * hc, p.rhoB[i], 0.0, p.rhoQ[i], 0.0, 0.0, 0.0, trace[i] * hc,
                   pixx[i] * hc, pixy[i] * hc, 0.0, -pixx[i] * hc, 0.0, 0.0,
                   0.0, qx[i], 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0]
            fh.write(" ".join(repr(float(v)) for v in row) + "\n")


SRC_IC = r'''
#include "ccake_gpu.hpp"
#include <cstdio>
int main(int argc, char** argv) {
  ccake_config cfg{};
  cfg.dim = 2; cfg.eos_kind = 1; cfg.thermo_mode = 1; cfg.using_shear = 1; cfg.shear_relax_mode = 1;
  cfg.zeta_mode = 1; cfg.eta_over_s = 0.08; cfg.zeta_over_s = 0.02; cfg.zeta_cs2_A = 1.67552; cfg.zeta_cs2_p = 2.0;
  cfg.hT = 0.1; cfg.hEta = 0.1; cfg.t0 = 1.0; cfg.dt = 0.001; cfg.eos_c = %(eos_c)r;
  cfg.eos_T0 = cfg.eos_muB0 = cfg.eos_muQ0 = cfg.eos_muS0 = 1.0;
  cfg.xmin = %(xmin)r; cfg.ymin = %(ymin)r; cfg.etamin = -0.1; cfg.freeze_out_T = %(tfo)r;
  cfg.using_diffusion = 1; cfg.kappa_over_T2[0] = 0.3; cfg.kappa_over_T2[8] = 0.3;
  cfg.reg_chi0 = 10.0; cfg.reg_e0 = 0.1; cfg.reg_xi0 = 0.01; cfg.reg_rq_max = 1.0;
  ccake_ic_options o{0, 1, 1, 1, 1, 0, 0.0};
  ccake::gpu::BSQHydro hydro(cfg, 1.0 + 2.5 * 0.001);   // three steps
  hydro.read_ccake(argv[1], o, true, true);
  hydro.initialize_hydrodynamics();
  hydro.run();
  ccake_totals tot = hydro.system().conservation();
  std::printf("%%.17g %%.17g %%.17g %%.17g\n", hydro.system().t(), tot.S, tot.B, tot.E);
  return 0;
}
'''


@pytest.mark.gpu
def test_shim_reads_ic_with_initial_state(tmp_path):
    # BSQHydro::read_ccake through the shim with initial diffusion, shear and
    # bulk, against the same run through the Python API and the oracle
    import dataclasses
    from ccake_gb300 import api, build, ics
    import oracle_py as O
    build.build()
    p0, rc = ics.hotspots_2d(n_side=32, n_hot=4, seed=5)
    rc = dataclasses.replace(rc, zeta_over_s=0.02, using_diffusion=1, kappa_over_T2=(0.3, 0, 0, 0, 0, 0, 0, 0, 0.3))
    ic = tmp_path / "ic29.dat"
    _write_ic_29(ic, p0, rc)
    src = tmp_path / "shim_ic.cpp"
    src.write_text(SRC_IC % {"eos_c": float(rc.eos_c), "xmin": float(rc.xmin), "ymin": float(rc.ymin),
                             "tfo": float(rc.freeze_out_T)})
    exe = tmp_path / "shim_ic"
    libdir = os.path.join(ROOT, "ccake_gb300", "_build")
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe), "-L", libdir,
                    "-lccake_gpu", "-Wl,-rpath," + libdir], check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe), str(ic)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    t, S, B, E = (float(v) for v in out.stdout.split())
    # the same inputs through the Python API and the oracle
    p, cols, _ = api.read_ccake_ic(ic, input_initial_diffusion=1)
    q = np.stack([cols[k] for k in ("qB0", "qB1", "qB2", "qB3", "qS0", "qS1", "qS2", "qS3", "qQ0", "qQ1", "qQ2",
                                    "qQ3")])
    pi = np.stack([cols[k] for k in ("pixx", "pixy", "pixeta", "piyy", "piyeta", "pietaeta")])
    g = api.GpuHydro(rc)
    g.load(p)
    g.set_initial_diffusion(q)
    g.set_initial_viscous(cols["bulk"], pi)
    g.initialize()
    g.step(3)
    o = O.OracleRun(p, rc)
    for c, C in enumerate("BSQ"):
        for m in range(4):
            o.set(f"in_q{C}{m}", q[4 * c + m])
    o.set_initial_viscous(cols["bulk"], pi)
    assert o.initialize() == 0
    assert o.step(3) == 0
    tg, to = g.totals(), o.totals()
    assert abs(t - g.t) < 1e-14
    assert (S, B, E) == (tg["S"], tg["B"], tg["E"])
    for k, v in (("S", S), ("B", B), ("E", E)):
        assert abs(v - to[k]) <= 1e-10 * abs(to[k]), k
    assert np.max(np.abs(g.get("qB1"))) > 0 and np.max(np.abs(g.get("bulk"))) > 0
