"""CPU reference of the closure network (bl_mlp.cu) for the gradient checks.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the tensor-
core kernels.  Never used by the product.

The network is 10 -> 64 -> 64 -> 2 with SiLU, parameters in the library's
layout (W1[64][10], b1[64], W2[64][64], b2[64], W3[2][64], b3[2]) and the
loss sum over samples and outputs of (y - t)^2 / (2 n).  ``forward`` and
``gradient`` evaluate it in FP64; with ``bf16=True`` every operand of a
matrix product is first rounded to BF16 (round to nearest even) exactly
where the GPU kernels round it, so the GPU results differ from these only
by the order of the FP32 sums.  ``numeric_gradient`` is the central-
difference check of the analytic FP64 gradient.
"""
import numpy as np

NI, NH, NO = 10, 64, 2
SHAPES = [("W1", (NH, NI)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)),
          ("W3", (NO, NH)), ("b3", (NO,))]
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(p):
    out, k = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[k:k + n], dtype=np.float64).reshape(shape)
        k += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).reshape(-1) for name, _ in SHAPES])


def init_params(seed=0):
    """Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases."""
    rng = np.random.default_rng(seed)
    d = {}
    for name, shape in SHAPES:
        if name.startswith("W"):
            lim = 1.0 / np.sqrt(shape[1])
            d[name] = rng.uniform(-lim, lim, shape)
        else:
            d[name] = np.zeros(shape)
    return pack(d).astype(np.float32)


def bf16(a):
    """Round float32 values to the nearest BF16 (ties to even), as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _silu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return z * s, s


def forward(p, x, bf=False):
    w = unpack(p)
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    x = np.asarray(x, dtype=np.float64)
    z1 = r(x) @ r(w["W1"]).T + w["b1"]
    h1, s1 = _silu(z1)
    if bf:
        h1 = h1.astype(np.float32)
    z2 = r(h1) @ r(w["W2"]).T + w["b2"]
    h2, s2 = _silu(z2)
    if bf:
        h2 = h2.astype(np.float32)
    y = r(h2) @ r(w["W3"]).T + w["b3"]
    return y, (x, z1, h1, s1, z2, h2, s2)


def gradient(p, x, t, bf=False):
    """(loss, gradient) over all samples."""
    w = unpack(p)
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    n = len(x)
    y, (x, z1, h1, s1, z2, h2, s2) = forward(p, x, bf)
    e = y - np.asarray(t, dtype=np.float64)
    loss = 0.5 * np.sum(e * e) / n
    dy = e / n
    if bf:
        dy = dy.astype(np.float32)
    dh2 = r(dy) @ r(w["W3"])
    dz2 = dh2 * s2 * (1.0 + z2 * (1.0 - s2))
    if bf:
        dz2 = dz2.astype(np.float32)
    dh1 = r(dz2) @ r(w["W2"])
    dz1 = dh1 * s1 * (1.0 + z1 * (1.0 - s1))
    if bf:
        dz1 = dz1.astype(np.float32)
    g = {"W1": r(dz1).T @ r(x), "b1": np.sum(dz1, axis=0),
         "W2": r(dz2).T @ r(h1), "b2": np.sum(dz2, axis=0),
         "W3": r(dy).T @ r(h2), "b3": np.sum(dy, axis=0)}
    return loss, pack(g)


def numeric_gradient(p, x, t, idx, h=1e-6):
    """Central differences of the FP64 loss at the parameter indices idx."""
    p = np.asarray(p, dtype=np.float64)
    out = []
    for i in idx:
        a, b = p.copy(), p.copy()
        a[i] += h
        b[i] -= h
        la, _ = gradient(a, x, t)
        lb, _ = gradient(b, x, t)
        out.append((la - lb) / (2 * h))
    return np.array(out)
