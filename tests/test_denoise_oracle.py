"""The denoiser's CPU restatement checked against itself: bf16 rounding,
layouts, and its analytic gradients against central finite differences
of an unrounded float64 evaluation of the same network (no GPU)."""
import numpy as np
import pytest

import denoise_oracle as D


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7, 1.0 + 3 * 2 ** -8, -2.5, 0.0], np.float32)
    y = D.bf16(x)
    # ties go to even: 1 + 2^-8 -> 1, 1 + 3 * 2^-8 -> 1 + 2^-6
    assert list(y) == [1.0, 1.0, 1.0 + 2 ** -7, 1.0 + 2 ** -6, -2.5, 0.0]


def test_parameter_count_is_about_1_9_million():
    assert 1_850_000 < D.num_params() < 2_000_000


def test_input_gradient_is_the_adjoint_of_the_convolution():
    rng = np.random.default_rng(1)
    x = rng.normal(size=(2, 8, 8, 16)).astype(np.float32)
    w = rng.normal(size=(8, 3, 3, 16)).astype(np.float32)
    dy = rng.normal(size=(2, 8, 8, 8)).astype(np.float32)
    # <conv(x), dy> == <x, conv_input_grad(dy)>; <conv(x), dy> == <w, conv_weight_grad(dy, x)>
    lhs = float((D.conv(x, w) * dy).sum(dtype=np.float64))
    assert abs(lhs - float((x * D.conv_input_grad(dy, w)).sum(dtype=np.float64))) < 1e-3 * abs(lhs) + 1e-3
    assert abs(lhs - float((w * D.conv_weight_grad(dy, x)).sum(dtype=np.float64))) < 1e-3 * abs(lhs) + 1e-3


def test_pool_and_upsample_gradients():
    rng = np.random.default_rng(2)
    x = rng.normal(size=(1, 4, 4, 3)).astype(np.float32)
    dy = rng.normal(size=(1, 2, 2, 3)).astype(np.float32)
    g = D.maxpool_grad(x, dy)
    assert np.allclose(g.sum(axis=(1, 2)), dy.sum(axis=(1, 2)), atol=1e-6)
    assert np.count_nonzero(g) == np.count_nonzero(dy)
    u = rng.normal(size=(1, 4, 4, 3)).astype(np.float32)
    assert np.allclose((D.upsample(dy) * u).sum(), (dy * D.upsample_grad(u)).sum(), atol=1e-4)


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(3)
    params = D.init_params(4)
    params[np.arange(len(params)) % 7 == 0] += 0.01  # non-zero biases too
    x = rng.uniform(0, 1, (1, 8, 8, 16)).astype(np.float32)
    x[..., 10:] = 0
    target = rng.uniform(0, 2, (1, 8, 8, 3)).astype(np.float32)
    _, g, _ = D.loss_and_grads(params, x, target)
    off, picks = 0, []
    for cin, cout in D.LAYERS:  # the largest weight gradient of every layer
        n = cout * 9 * cin
        picks.append(off + int(np.argmax(np.abs(g[off:off + n]))))
        off += n + cout
    good = 0
    for i in picks:
        h = 1e-3
        p1, p2 = params.copy(), params.copy()
        p1[i] += h
        p2[i] -= h
        fd = (D.exact_loss(p1, x, target) - D.exact_loss(p2, x, target)) / (2 * h)
        good += abs(fd - g[i]) <= 0.05 * abs(g[i]) + 1e-5
    assert good >= len(picks) - 1  # the L1 kink may catch one
