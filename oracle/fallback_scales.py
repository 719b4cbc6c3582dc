"""CPU restatement of how the reference matches the analytic fallbacks of a
tabulated EoS to the table (test infrastructure only):
EquationOfState::set_up_chosen_EOSs, src/eos_initialization.cpp:276-341
(tanh_conformal), :343-403 (conformal) and :404-464 (conformal_diagonal).

With Tmax = 1.1 T_FO and the grid maxima mu_max of each chemical-potential
axis, p(T, mu) the table's interpolated pressure:
  c = p(Tmax, 0, 0, 0) / Tmax^4, T0 = 1 (all three fallbacks);
  tanh_conformal and conformal: mu0 = c^(1/4) mu_max / sqrt(sqrt(p(Tmax, mu_max)) - sqrt(p(Tmax, 0)));
  conformal_diagonal:           mu0 = (c / (p(Tmax, mu_max) - p(Tmax, 0)))^(1/4) mu_max;
an axis whose maximum is 0 keeps mu0 = 1.
"""
import ctypes
from types import SimpleNamespace

import numpy as np

import oracle_py as O


def reference_fallback_scales(n, lo, d, fields, freeze_out_T):
    """(conf5, cdiag5) = (c, T0, muB0, muQ0, muS0) of the conformal (and
    tanh-conformal) and conformal-diagonal fallbacks, from the oracle's table
    lookup (src/interpolatorND.cpp:250-317)."""
    ones = np.ones(5)
    table = O.OracleTable(n, lo, d, fields, ones, ones)
    cfg = O.make_config(SimpleNamespace(eos_kind=2))

    def p_at(x):
        out = np.zeros(17)
        O.lib().orc_eos_full_thermo(ctypes.byref(cfg), table.h, 0, O._dp(np.asarray(x, dtype=np.float64)),
                                    O._dp(out))
        return out[0]

    n = np.asarray(n)
    lo = np.asarray(lo, dtype=np.float64)
    d = np.asarray(d, dtype=np.float64)
    mx = lo + d * (n - 1)
    Tmax = 1.1 * freeze_out_T
    pT = p_at([Tmax, 0.0, 0.0, 0.0])
    c = pT / Tmax ** 4
    conf = [c, 1.0, 1.0, 1.0, 1.0]
    cdiag = [c, 1.0, 1.0, 1.0, 1.0]
    for a in (1, 2, 3):   # muB, muQ, muS
        if abs(mx[a]) < 1e-30:
            continue
        x = [Tmax, 0.0, 0.0, 0.0]
        x[a] = mx[a]
        pv = p_at(x)
        conf[1 + a] = c ** 0.25 * mx[a] / np.sqrt(np.sqrt(pv) - np.sqrt(pT))
        cdiag[1 + a] = (c / (pv - pT)) ** 0.25 * mx[a]
    return np.array(conf), np.array(cdiag)
