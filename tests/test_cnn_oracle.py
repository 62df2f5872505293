"""The network oracle's analytic gradients against finite differences (CPU)."""
import numpy as np
import pytest

from oracle import cnn_oracle as co


def test_param_count():
    p = co.init_params(0)
    assert p.size == sum(9 * i * o + o for i, o in zip(co.CIN, co.COUT)) == 22281


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.1415926], dtype=np.float32)
    r = co.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0          # tie to even
    assert r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-7


def test_conv_is_cross_correlation():
    x = np.zeros((1, 1, 5, 5))
    x[0, 0, 2, 2] = 1.0
    w = np.zeros((9, 1, 1))
    w[0, 0, 0] = 1.0                             # tap (ky, kx) = (0, 0)
    out = co.conv(x, w)
    assert out[0, 0, 3, 3] == 1.0 and out.sum() == 1.0


def test_input_and_weight_grads_are_adjoint():
    rng = np.random.default_rng(1)
    x = rng.normal(size=(2, 3, 6, 7))
    w = rng.normal(size=(9, 3, 4))
    g = rng.normal(size=(2, 4, 6, 7))
    lhs = np.sum(co.conv(x, w) * g)
    assert abs(lhs - np.sum(x * co.conv_input_grad(g, w))) < 1e-9
    assert abs(lhs - np.sum(w * co.conv_weight_grad(x, g))) < 1e-9


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(2)
    p = co.init_params(3, scale=1.0)
    x = rng.normal(size=(2, 4, 5, 6))
    target = rng.normal(size=(2, 9, 5, 6)) * 0.1
    loss, g = co.gradients(p, x, target, bf16_rounding=False)
    idx = rng.choice(p.size, size=40, replace=False)
    idx = np.concatenate([idx, [p.size - 1, p.size - 10, 0, 9 * 4 * 32 + 3]])
    eps = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += eps
        pm[k] -= eps
        lp, _ = co.gradients(pp, x, target, bf16_rounding=False)
        lm, _ = co.gradients(pm, x, target, bf16_rounding=False)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)) + 1e-9, (k, fd, g[k])
