"""The guiding network's CPU oracle (oracle/lmoracle_guide.py) is pinned by
finite differences: its hand-written backpropagation of the vMF-mixture
loss matches central differences of the loss in FP64."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import lmoracle_guide as og  # noqa: E402

BOX = (-1.0, 0.0, -2.0, 3.0, 2.0, 2.0)


def problem(n, seed):
    g = np.random.default_rng(seed)
    q = np.zeros((n, 9))
    q[:, :3] = g.uniform([-1, 0, -2], [3, 2, 2], size=(n, 3))
    nrm = g.normal(size=(n, 3))
    q[:, 3:6] = nrm / np.linalg.norm(nrm, axis=1, keepdims=True)
    wo = g.normal(size=(n, 3))
    q[:, 6:9] = wo / np.linalg.norm(wo, axis=1, keepdims=True)
    d = g.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    w = g.uniform(0.1, 2.0, size=n)
    return q, d, w


def test_parameter_count():
    assert og.num_params() == 23856


def test_raw_gradient_matches_finite_differences():
    g = np.random.default_rng(3)
    raw = g.normal(size=(5, 40))
    raw[:, 3::5] = g.uniform(-2, 5, size=(5, 8))
    _, d, w = problem(5, 4)
    loss, grad = og.loss_and_raw_grad(raw, d, w)
    eps = 1e-6
    num = np.zeros_like(raw)
    for i in range(raw.shape[0]):
        for j in range(raw.shape[1]):
            a = raw.copy()
            a[i, j] += eps
            b = raw.copy()
            b[i, j] -= eps
            num[i, j] = (og.loss_and_raw_grad(a, d, w)[0] - og.loss_and_raw_grad(b, d, w)[0]) / (2 * eps)
    assert np.allclose(grad, num, rtol=1e-5, atol=1e-8), np.abs(grad - num).max()


def test_parameter_gradient_matches_finite_differences():
    p = og.init_params(7).astype(np.float64)
    p[og.num_params() - 48:og.num_params() - 8] = np.random.default_rng(1).normal(size=40) * 0.3
    q, d, w = problem(6, 8)
    loss, grad = og.gradient(p, q, BOX, d, w)
    g = np.random.default_rng(9)
    idx = np.concatenate([g.choice(p.size, 60, replace=False), np.arange(p.size - 48, p.size - 8)])
    eps = 1e-6
    for i in idx:
        a = p.copy()
        a[i] += eps
        b = p.copy()
        b[i] -= eps
        fa = og.gradient(a, q, BOX, d, w)[0]
        fb = og.gradient(b, q, BOX, d, w)[0]
        assert abs((fa - fb) / (2 * eps) - grad[i]) <= 1e-6 + 1e-4 * abs(grad[i]), (i, grad[i], (fa - fb) / (2 * eps))


def test_mixture_is_normalised():
    """The vMF mixture integrates to 1 over the sphere (Fibonacci quadrature)."""
    g = np.random.default_rng(5)
    raw = g.normal(size=(1, 40))
    raw[:, 3::5] = np.array([-3, 0, 2, 4, 1, 3, 0.5, 2.5])
    n = 200000
    k = np.arange(n) + 0.5
    z = 1 - 2 * k / n
    phi = np.pi * (1 + 5 ** 0.5) * k
    r = np.sqrt(1 - z * z)
    d = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)
    lq = og.mixture_logpdf(np.repeat(raw, n, axis=0), d)
    assert abs(np.exp(lq).mean() * 4 * np.pi - 1.0) < 2e-3
