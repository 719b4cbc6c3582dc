"""The reference's semi-analytic viscous Gubser tables (fixture extracted by
tests/golden/make_gubser_golden.py) and the comparison of an SPH state with
them along the lines y = 0 and y = x.

Particles of the lattice centred on the origin that start on either line stay
on it (the flow is radially symmetric), so the SPH fields are read along the
line by linear interpolation in x between those particles.
"""
import json
import os

import numpy as np

HBARC_GEVFM = 0.1973269804
PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gubser_semianalytic.json")
FIELDS = ("T", "ux", "uy", "pixx", "piyy", "pixy", "t2pee")


def load():
    with open(PATH) as fh:
        doc = json.load(fh)
    return {(t["line"], t["tau"]): np.asarray(t["rows"]) for t in doc["tables"]}


def sph_fields(get, tau):
    """The table's columns from a state accessor get(name) (GPU or oracle), in GeV units."""
    hc = HBARC_GEVFM
    return {"T": get("T") * hc, "ux": get("u0"), "uy": get("u1"), "pixx": get("shv11") * hc,
            "piyy": get("shv22") * hc, "pixy": get("shv12") * hc, "t2pee": get("shv33") * hc * tau * tau}


def line_errors(table, line, x, y, fields, dx, xlim):
    """Max |SPH - table| over the table's points with |x| <= xlim, per field,
    divided by the field's largest magnitude in the table (T is checked
    relative to the local value)."""
    sel = np.abs(y) < 0.25 * dx if line == "y=0" else np.abs(x - y) < 0.25 * dx
    xs = x[sel]
    order = np.argsort(xs)
    xs = xs[order]
    pts = np.abs(table[:, 0]) <= xlim
    out = {}
    for col, f in enumerate(FIELDS, start=2):
        ref = table[pts, col]
        scale = np.max(np.abs(table[:, col]))
        if scale == 0.0:
            continue
        v = np.interp(table[pts, 0], xs, fields[f][sel][order])
        if f == "T":
            out[f] = float(np.max(np.abs(v - ref) / ref))
        else:
            out[f] = float(np.max(np.abs(v - ref)) / scale)
    return out
