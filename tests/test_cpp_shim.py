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
