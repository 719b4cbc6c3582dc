"""CPU restatement of the reference's pre-inverted EoS lookup (test
infrastructure only): EoS_Interpolator::fill_thermodynamics and
interpolate4D, src/eos_interpolator.cpp:531-739, on tiles laid out by
utilities/generate_eos_table.cpp:196-203 and :296-342.

- densities clamped to max(0.001, s) and max(0.001, |rho|);
- the tile of an axis: the decade of the value, clamped to the tiles present
  (here: the number of tile edges 10^(e_lo + j), j >= 1, at or below it);
- tile minimum 10^e, step 10^(e+1) / N, N nodes an axis;
- cell index floor((x - min) / step) clamped to [0, N - 2] (the reference
  clamps to N - 1 and then reads the +1 corner);
- x_i = ((pos - min) - idx * step) / step; corner c takes the +1 node on
  axis i when bit i of c is set; phi_c = prod_i (bit ? x_i : 1 - x_i) in axis
  order; f = sum_c phi_c theta_c in corner order.

Tables: values[tile][node][11] with tiles and nodes row-major (rhoQ
fastest); variables T, muB, muQ, muS, e, p, cs2, dwds, dwdB, dwdQ, dwdS.
"""
import numpy as np

NVARS = 11


def tile_geometry(exp_lo, exp_hi, N):
    nt = [h - l + 1 for l, h in zip(exp_lo, exp_hi)]
    mn = [[10.0 ** (exp_lo[k] + j) for j in range(nt[k])] for k in range(4)]
    st = [[10.0 ** (exp_lo[k] + j + 1) / N for j in range(nt[k])] for k in range(4)]
    return nt, mn, st


def node_coordinates(exp_lo, exp_hi, N):
    """(s, rhoB, rhoS, rhoQ) of every node in table order (min + i * step)."""
    nt, mn, st = tile_geometry(exp_lo, exp_hi, N)
    out = []
    for t in np.ndindex(*nt):
        for ix in np.ndindex(N, N, N, N):
            out.append([mn[k][t[k]] + ix[k] * st[k][t[k]] for k in range(4)])
    return np.array(out)


def lookup(values, exp_lo, exp_hi, N, sBSQ):
    nt, mn, st = tile_geometry(exp_lo, exp_hi, N)
    tn = N ** 4
    vals = values.reshape(-1, tn, NVARS)
    out = np.zeros((len(sBSQ), NVARS))
    for r, q in enumerate(sBSQ):
        pos = [max(0.001, q[0])] + [max(0.001, abs(v)) for v in q[1:]]
        t, idx, x = [], [], []
        for k in range(4):
            tk = sum(1 for j in range(1, nt[k]) if pos[k] >= mn[k][j])
            m, d = mn[k][tk], st[k][tk]
            ik = int(np.floor((pos[k] - m) / d))
            ik = min(max(ik, 0), N - 2)
            t.append(tk)
            idx.append(ik)
            x.append(((pos[k] - m) - ik * d) / d)
        tile = ((t[0] * nt[1] + t[1]) * nt[2] + t[2]) * nt[3] + t[3]
        f = np.zeros(NVARS)
        for c in range(16):
            ph = 1.0
            for i in range(4):
                ph = ph * (x[i] if (c >> i) & 1 else 1.0 - x[i])
            node = (((idx[0] + (c & 1)) * N + idx[1] + ((c >> 1) & 1)) * N + idx[2] + ((c >> 2) & 1)) * N + \
                idx[3] + ((c >> 3) & 1)
            f = f + ph * vals[tile, node]
        out[r] = f
    return out
