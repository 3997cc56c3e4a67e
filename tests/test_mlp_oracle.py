"""The CPU restatement of the alpha-guess MLP (the checker of the CUDA
training kernels): analytic gradient against central finite differences,
and the bfloat16 rounding it uses to emulate the tensor-core inference."""
import numpy as np

from oracle import mlp


class M:
    pass


def model(n_in=27, seed=0):
    rng = np.random.default_rng(seed)
    m = M()
    m.input_scale = rng.uniform(0.5, 2.0, n_in)
    m.w1 = rng.standard_normal((32, n_in)) / np.sqrt(n_in)
    m.b1 = rng.standard_normal(32) * 0.1
    m.w2 = rng.standard_normal((32, 32)) / np.sqrt(32)
    m.b2 = rng.standard_normal(32) * 0.1
    m.w3 = rng.standard_normal(32) / np.sqrt(32)
    m.b3 = 0.1
    m.output_scale = 0.05
    return m


def test_analytic_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    X = rng.standard_normal((64, 27))
    t = 2.0 + 0.05 * rng.standard_normal(64)
    m = model()
    _, g = mlp.loss_and_grad(m, X, t)
    for name in ("w1", "b1", "w2", "b2", "w3"):
        arr = getattr(m, name)
        for k in range(5):
            idx = tuple(rng.integers(0, s) for s in arr.shape)
            old = arr[idx]
            arr[idx] = old + 1e-6
            lp = mlp.loss_only(m, X, t)
            arr[idx] = old - 1e-6
            lm = mlp.loss_only(m, X, t)
            arr[idx] = old
            assert abs(g[name][idx] - (lp - lm) / 2e-6) <= 1e-6 * max(1.0, abs(g[name][idx]))


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -9, 1.0 + 3 * 2 ** -9, -2.5, 3.140625], np.float32)
    r = mlp.bf16(x)
    assert r[0] == 1.0
    # ties to even: 1 + 2^-8 is exactly half an ulp (ulp = 2^-7) above 1 -> 1
    assert r[1] == 1.0
    assert r[2] == 1.0
    assert r[3] == 1.0 + 2 ** -7
    assert r[4] == -2.5 and r[5] == 3.140625
