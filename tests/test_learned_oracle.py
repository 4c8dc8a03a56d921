"""CPU checks of the learned classifier's oracle (oracle/mlp.py).

The oracle's analytic gradient is checked against central finite differences
of its own float64 loss; the float32/BF16 restatement of the device
arithmetic is checked against the float64 one; the model serialisation
against the library's size.
"""
import numpy as np

from oracle import mlp
from rabbitqcplus_gb300 import capi


def test_gradient_formulas_match_finite_differences():
    rng = np.random.default_rng(3)
    m = mlp.random_model(5)
    x = rng.normal(0, 1, (40, mlp.F))
    y = rng.integers(0, 2, 40)
    g = mlp.gradients64(m, x, y)
    v = mlp.flatten(m)
    idx = np.concatenate([rng.choice(mlp.NPARAMS, 60, replace=False), [mlp.NPARAMS - 1]])
    h = 1e-6
    for i in idx:
        vp, vm = v.copy(), v.copy()
        vp[i] += h
        vm[i] -= h
        num = (mlp.loss64(mlp.unflatten(m, vp), x, y) - mlp.loss64(mlp.unflatten(m, vm), x, y)) / (2 * h)
        assert abs(num - g[i]) <= 1e-6 + 1e-5 * abs(num), (i, num, g[i])


def test_bf16_restatement_close_to_float64():
    rng = np.random.default_rng(4)
    m = mlp.random_model(6)
    x = rng.uniform(0, 1, (500, mlp.F)).astype(np.float32)
    y = rng.integers(0, 2, 500)
    loss, g = mlp.gradients(m, x, y)
    g64 = mlp.gradients64(m, mlp.bf16(x), y)
    assert abs(loss - mlp.loss64(m, mlp.bf16(x), y)) < 1e-2
    cos = float(g @ g64 / np.linalg.norm(g) / np.linalg.norm(g64))
    assert cos > 0.999


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2**-8, 1.0 + 2**-9, 1.0 + 3 * 2**-9, -2.5, 0.0], np.float32)
    r = mlp.bf16(x)
    # 1 + 2^-8 is halfway between 1 and 1 + 2^-7: ties go to the even mantissa (1.0)
    assert r.tolist() == [1.0, 1.0, 1.0, 1.0078125, -2.5, 0.0]


def test_serialization_round_trip_and_size():
    m = mlp.random_model(7)
    b = mlp.serialize(m)
    assert len(b) == capi.gpu_lib().cg_classifier_size()
    m2 = mlp.parse(b)
    for k in ("w1", "w2", "w3", "b1", "b2"):
        assert np.array_equal(m[k], m2[k]), k
    assert m["b3"] == m2["b3"]
