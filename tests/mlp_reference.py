"""CPU reference of the learned-seed network (test infrastructure only).

4-64-64-64-4 tanh MLP, parameters in the library's FP32 block layout
(W1 [64][4], b1, W2 [64][64], b2, W3 [64][64], b3, W4 [4][64], b4), loss =
mean over rows and outputs of (o - y)^2. `forward`/`gradient` with bf16=True
round every tensor-core operand (inputs, weights, hidden activations, dL/do
and the back-propagated dL/dz of layers 3 and 2) to BF16 with round to
nearest even, as the GPU kernels do, and accumulate in float64; the
CUDA-core parts (dW1, dW4, the biases) use the unrounded FP32 values the GPU
uses there. With bf16=False everything is float64 (the exact model).
"""
import numpy as np

SHAPES = [("W1", (64, 4)), ("b1", (64,)), ("W2", (64, 64)), ("b2", (64,)), ("W3", (64, 64)), ("b3", (64,)),
          ("W4", (4, 64)), ("b4", (4,))]
N_PARAMS = 8900


def unpack(p):
    out, o = {}, 0
    for name, sh in SHAPES:
        n = int(np.prod(sh))
        out[name] = np.asarray(p[o:o + n], dtype=np.float64).reshape(sh)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SHAPES])


def bf16(x):
    """Round to BF16 (nearest even), returned as float64."""
    x = np.asarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def _r(x, on):
    return bf16(x) if on else np.asarray(x, dtype=np.float64)


def forward(p, X, bf=True):
    P = unpack(p)
    a0 = _r(X, bf)
    h1 = np.tanh(a0 @ _r(P["W1"], bf).T + P["b1"])
    a1 = _r(h1, bf)
    h2 = np.tanh(a1 @ _r(P["W2"], bf).T + P["b2"])
    a2 = _r(h2, bf)
    h3 = np.tanh(a2 @ _r(P["W3"], bf).T + P["b3"])
    a3 = _r(h3, bf)
    o = a3 @ _r(P["W4"], bf).T + P["b4"]
    return o, (a0, a1, a2, a3)


def gradient(p, X, Y, bf=True):
    """(grad block, sum of squared errors)."""
    P = unpack(p)
    n = X.shape[0]
    o, (a0, a1, a2, a3) = forward(p, X, bf)
    e = o - Y
    dO = 2.0 * e / (4.0 * n)
    g = {"W4": dO.T @ a3, "b4": dO.sum(0)}
    dz3 = (_r(dO, bf) @ _r(P["W4"], bf)) * (1.0 - a3 * a3)
    g["W3"] = _r(dz3, bf).T @ a2
    g["b3"] = dz3.sum(0)
    dz2 = (_r(dz3, bf) @ _r(P["W3"], bf)) * (1.0 - a2 * a2)
    g["W2"] = _r(dz2, bf).T @ a1
    g["b2"] = dz2.sum(0)
    dz1 = (_r(dz2, bf) @ _r(P["W2"], bf)) * (1.0 - a1 * a1)
    g["W1"] = dz1.T @ a0
    g["b1"] = dz1.sum(0)
    return pack(g), float((e * e).sum())


def loss(p, X, Y):
    o, _ = forward(p, X, bf=False)
    return float(((o - Y) ** 2).mean())


def random_params(seed=0, scale=1.0):
    rng = np.random.default_rng(seed)
    d = {}
    for name, sh in SHAPES:
        if name.startswith("W"):
            a = np.sqrt(6.0 / (sh[0] + sh[1])) * scale
            d[name] = rng.uniform(-a, a, sh)
        else:
            d[name] = rng.normal(0.0, 0.1, sh)
    return pack(d).astype(np.float32)
