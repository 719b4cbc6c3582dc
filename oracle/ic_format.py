"""CPU restatement of the reference's "ccake" initial-condition reader (test
infrastructure only): BSQHydro::read_ccake, src/BSQHydro.cpp:206-425.

- line 1 is the header: after its first '#', eight numbers
  "<ignored> dx dy deta <ignored> xmin ymin etamin" (:239-249);
- later lines: blank lines and lines whose first non-blank character is '#'
  are skipped (:255-256); a data line holds 17 numbers (x y eta e|s rhoB rhoS
  rhoQ ux uy ueta bulk pixx pixy pixeta piyy piyeta pietaeta), 29 with
  initial diffusion (+ qB^0..3 qS^0..3 qQ^0..3) (:258-263);
- e is divided by hbar c = 0.1973269804 GeV fm unless the input is entropy;
  the five pi^{ij} and the bulk pressure are divided by hbar c (:264-285);
- a disabled charge reads as zero, its diffusion too (:341-380);
- a cell is kept when e > e_cutoff / hbar c, with entropy input when the
  ideal pion gas energy 3C (s/4C)^{4/3}, C = 3 pi^2 / 90, is (:398-407).

Returns the columns in file order under the names of COLUMNS.
"""
import math

HBARC_GEV = 0.1973269804
COLUMNS = ("x", "y", "eta", "e", "rhoB", "rhoS", "rhoQ", "ux", "uy", "ueta", "bulk", "pixx", "pixy", "pixeta",
           "piyy", "piyeta", "pietaeta", "qB0", "qB1", "qB2", "qB3", "qS0", "qS1", "qS2", "qS3", "qQ0", "qQ1",
           "qQ2", "qQ3")


def read_ccake(path, input_as_entropy=False, input_initial_diffusion=False, charges=(1, 1, 1), e_cutoff=0.0):
    cols = {c: [] for c in COLUMNS}
    with open(path) as fh:
        header = fh.readline()
        head = header[header.index("#") + 1:].split()
        grid = tuple(float(head[k]) for k in (1, 2, 3, 5, 6, 7))
        ncol = 29 if input_initial_diffusion else 17
        C = 3.0 * math.pi ** 2 / 90.0
        eps_of_s = (3.0 * C) * math.pow(1.0 / (4.0 * C), 4.0 / 3.0)
        for line in fh:
            t = line.strip()
            if not t or t.startswith("#"):
                continue
            parts = t.split()
            if len(parts) < ncol:
                raise ValueError("short data line")
            v = [float(x) for x in parts[:ncol]] + [0.0] * (29 - ncol)
            if not input_as_entropy:
                v[3] /= HBARC_GEV
            for k in range(10, 17):
                v[k] /= HBARC_GEV
            for c in range(3):
                if not charges[c]:
                    v[4 + c] = 0.0
                    for m in range(4):
                        v[17 + 4 * c + m] = 0.0
            e_check = eps_of_s * math.pow(v[3], 4.0 / 3.0) if input_as_entropy else v[3]
            if not (e_check > e_cutoff / HBARC_GEV):
                continue
            for k, c in enumerate(COLUMNS):
                cols[c].append(v[k])
    return cols, grid
