"""The CPU reference of the seed network: its FP64 backward against central
finite differences of its FP64 loss, and the BF16-emulating form against
the FP64 one (no GPU)."""
import numpy as np

import mlp_reference as M


def test_fp64_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = M.random_params(1).astype(np.float64)
    X = rng.normal(size=(37, 4))
    Y = rng.normal(size=(37, 4))
    g, _ = M.gradient(p, X, Y, bf=False)
    idx = rng.choice(M.N_PARAMS, 60, replace=False)
    idx = np.concatenate([idx, [0, 255, 256, 4415, 8639, 8640, 8899]])
    for i in idx:
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (M.loss(pp, X, Y) - M.loss(pm, X, Y)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 * max(1.0, abs(g[i])) + 1e-9, i


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, 1.0 + 2 ** -9, -3.140625, 1e-30], dtype=np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0 + 2 ** -7 or r[1] == 1.0   # exactly half way: even mantissa wins
    assert r[1] == 1.0
    assert r[2] == 1.0 + 2 ** -7                  # above half way rounds up
    assert r[3] == 1.0                            # below half way rounds down
    assert r[4] == -3.140625
    assert abs(r[5] / 1e-30 - 1) < 2 ** -8


def test_bf16_form_close_to_fp64():
    rng = np.random.default_rng(4)
    p = M.random_params(2)
    X = rng.normal(size=(256, 4))
    Y = rng.normal(size=(256, 4))
    g64, _ = M.gradient(p, X, Y, bf=False)
    g16, _ = M.gradient(p, X, Y, bf=True)
    cos = g64 @ g16 / np.linalg.norm(g64) / np.linalg.norm(g16)
    assert cos > 0.999
