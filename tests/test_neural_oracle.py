"""The CPU oracle of the neural IBL shader (oracle/nn_oracle.py), on its own: encoding values,
BF16 rounding, the analytic gradient against finite differences, Adam against its textbook form
and the record sampler. The GPU kernels are checked against this oracle in test_neural_gpu.py."""
import numpy as np
import pytest

from oracle import nn_oracle as O


def test_encoding_layout():
    x = np.linspace(-1, 1, 12, dtype=np.float32)[None, :]
    f = O.encode(x)
    assert f.shape == (1, 156)
    np.testing.assert_allclose(f[0, 144:156], x[0])
    for k in range(6):
        np.testing.assert_allclose(f[0, 24 * k:24 * k + 24:2], np.sin(2 ** k * np.pi * x[0]), atol=2e-5)
        np.testing.assert_allclose(f[0, 24 * k + 1:24 * k + 24:2], np.cos(2 ** k * np.pi * x[0]), atol=2e-5)


def test_bf16_rounding():
    a = np.array([1.0, 1.00390625, 1.005859375, -2.0, 3.0e-40, 65504.0], np.float32)
    r = O.bf16(a)
    assert r[0] == 1.0 and r[3] == -2.0
    assert r[1] == 1.0                      # halfway 1 + 2^-8: ties to even -> 1.0
    assert r[2] == np.float32(1.0078125)    # above halfway rounds up
    assert np.all(r.view(np.uint32) & 0xFFFF == 0)


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    n = 64
    x = rng.uniform(-1, 1, (n, 12)).astype(np.float32)
    t = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    flat = rng.normal(0, 0.2, O.N_PARAMS).astype(np.float32)
    p = O.unflatten(flat)
    loss, g = O.loss_and_grad(p, x, t, use_bf16=False)
    gf = O.flatten(g)
    idx = rng.choice(O.N_PARAMS, 40, replace=False)
    # central differences of the FP32 loss; a step may cross a ReLU kink, so allow 2 of 40 misses
    h = 1e-3
    bad = []
    for i in idx:
        fp, fm = flat.copy(), flat.copy()
        fp[i] += h
        fm[i] -= h
        lp, _ = O.loss_and_grad(O.unflatten(fp), x, t, use_bf16=False)
        lm, _ = O.loss_and_grad(O.unflatten(fm), x, t, use_bf16=False)
        fd = (lp - lm) / (2 * h)
        if abs(fd - gf[i]) > 1e-2 * abs(gf[i]) + 2e-4:
            bad.append((int(i), fd, float(gf[i])))
    assert len(bad) <= 2, bad


def test_adam_matches_textbook():
    rng = np.random.default_rng(1)
    p = O.unflatten(rng.normal(0, 0.1, O.N_PARAMS).astype(np.float32))
    p64 = {k: v.astype(np.float64) for k, v in p.items()}
    m = {k: np.zeros_like(v) for k, v in p.items()}
    v = {k: np.zeros_like(q) for k, q in p.items()}
    m64 = {k: np.zeros_like(q) for k, q in p64.items()}
    v64 = {k: np.zeros_like(q) for k, q in p64.items()}
    for step in range(1, 4):
        g = O.unflatten(rng.normal(0, 1e-2, O.N_PARAMS).astype(np.float32))
        O.adam_step(p, g, m, v, step, 1e-3)
        for k in O.ORDER:
            m64[k] = 0.9 * m64[k] + 0.1 * g[k]
            v64[k] = 0.999 * v64[k] + 0.001 * g[k].astype(np.float64) ** 2
            p64[k] -= 1e-3 * (m64[k] / (1 - 0.9 ** step)) / (np.sqrt(v64[k] / (1 - 0.999 ** step)) + 1e-8)
    for k in O.ORDER:
        np.testing.assert_allclose(p[k], p64[k], atol=1e-6)


def test_sampler_is_deterministic_and_in_range():
    a = O.sample_indices(7, 3, 1000, 12345)
    b = O.sample_indices(7, 3, 1000, 12345)
    c = O.sample_indices(7, 4, 1000, 12345)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert a.min() >= 0 and a.max() < 12345
    # roughly uniform
    h = np.bincount(O.sample_indices(1, 0, 200000, 10), minlength=10)
    assert h.min() > 19000 and h.max() < 21000


def test_psnr():
    a = np.zeros((4, 4), np.uint8)
    b = a.copy()
    assert O.psnr(a, b) == float("inf")
    b[0, 0] = 16
    assert O.psnr(a, b) == pytest.approx(10 * np.log10(255.0 ** 2 / 16.0))
