"""The CPU reference of the closure network (oracle/mlp.py): its analytic
gradient agrees with central differences, so it can check the GPU kernels."""
import numpy as np

from oracle import mlp


def test_reference_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = mlp.init_params(seed=1).astype(np.float64)
    p[mlp.NH * mlp.NI:mlp.NH * mlp.NI + mlp.NH] = rng.normal(0, 0.1, mlp.NH)  # nonzero b1
    x = rng.normal(0, 1, (37, mlp.NI))
    t = rng.normal(0, 1, (37, mlp.NO))
    _, g = mlp.gradient(p, x, t)
    idx = rng.choice(mlp.NPARAM, 60, replace=False)
    num = mlp.numeric_gradient(p, x, t, idx)
    assert np.allclose(g[idx], num, rtol=1e-5, atol=1e-8), np.max(np.abs(g[idx] - num))


def test_bf16_rounding_is_round_to_nearest_even():
    v = np.array([1.0, 1.0 + 2**-8, 1.0 + 3 * 2**-9, -2.5, 3.0e-3], dtype=np.float32)
    r = mlp.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2**-7 and r[3] == -2.5
    assert abs(r[4] - 3.0e-3) <= 3.0e-3 * 2**-8
