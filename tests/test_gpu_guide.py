"""The guiding network on the tensor cores (lmgpu_guide_*, tcgen05 forward /
backward / Adam kernels) against the FP64 CPU oracle
(oracle/lmoracle_guide.py, itself pinned by finite differences)."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import lmoracle_guide as og  # noqa: E402
from test_oracle_guide import BOX, problem  # noqa: E402

pytestmark = pytest.mark.gpu


def trained_like_params(seed):
    """Initial weights with non-trivial output biases (so every lobe term matters)."""
    p = og.init_params(seed)
    g = np.random.default_rng(seed + 1)
    p[og.num_params() - 48:og.num_params() - 8] = g.normal(size=40).astype(np.float32) * 0.5
    return p


def test_forward_matches_oracle(gpu_lib):
    net = gpu_lib.Guide(BOX, 1)
    p = trained_like_params(11)
    net.set_params(p)
    assert np.array_equal(net.params(), p)
    q, _, _ = problem(1000, 12)  # 7 full tiles and a partial one
    raw = net.forward(q).astype(np.float64)
    ref, _, _ = og.forward(p, q, BOX, emulate_bf16=True)
    err = np.linalg.norm(raw - ref) / np.linalg.norm(ref)
    print("forward relative L2 error vs oracle (bf16 emulated)", err)
    assert err < 1e-2, err
    ref64, _, _ = og.forward(p, q, BOX)
    assert np.linalg.norm(raw - ref64) / np.linalg.norm(ref64) < 3e-2
    net.close()


def test_gradient_matches_fp64_oracle(gpu_lib):
    net = gpu_lib.Guide(BOX, 2)
    p = trained_like_params(21)
    net.set_params(p)
    q, d, w = problem(4096 + 77, 22)
    loss, g = net.gradient(q, d, w)
    ref_loss, ref = og.gradient(p, q, BOX, d, w)
    cos = float(g @ ref / (np.linalg.norm(g) * np.linalg.norm(ref)))
    rel = float(np.linalg.norm(g - ref) / np.linalg.norm(ref))
    print("loss", loss, ref_loss, "gradient cosine", cos, "relative L2", rel)
    assert abs(loss - ref_loss) < 1e-2 * abs(ref_loss) + 1e-4
    assert cos > 0.999 and rel < 5e-2, (cos, rel)
    # per layer: every block of the gradient agrees, not just the total
    o = 0
    for rows, cols in og.layer_shapes():
        for size in (rows * cols, rows):
            a, b = g[o:o + size], ref[o:o + size]
            if np.linalg.norm(b) > 0:
                assert np.linalg.norm(a - b) / np.linalg.norm(b) < 0.1, (o, size)
            o += size
    # the padding rows of the output layer get no gradient
    w5 = og.num_params() - 48 - 48 * 64
    assert not g[w5 + 40 * 64:w5 + 48 * 64].any() and not g[-8:].any()
    net.close()


def test_gradient_over_many_tiles_per_cta(gpu_lib):
    """Enough samples that every CTA of the backward accumulates several
    128-sample tiles in tensor memory before its one flush (and a partial
    last tile): the gradient still matches the FP64 oracle, and a second call
    on other samples is not polluted by the first."""
    net = gpu_lib.Guide(BOX, 4)
    p = trained_like_params(31)
    net.set_params(p)
    for seed in (32, 33):
        q, d, w = problem(3 * 160 * 128 + 77, seed)
        loss, g = net.gradient(q, d, w)
        ref_loss, ref = og.gradient(p, q, BOX, d, w)
        cos = float(g @ ref / (np.linalg.norm(g) * np.linalg.norm(ref)))
        rel = float(np.linalg.norm(g - ref) / np.linalg.norm(ref))
        print("samples", q.shape[0], "loss", loss, ref_loss, "gradient cosine", cos, "relative L2", rel)
        assert abs(loss - ref_loss) < 1e-2 * abs(ref_loss) + 1e-4
        assert cos > 0.999 and rel < 5e-2, (cos, rel)
    net.close()


def test_training_fits_a_direction_field(gpu_lib):
    """Online Adam on samples of a position-dependent target (directions
    towards a point, kappa 30): the loss falls and the learned density at
    fresh target samples rises well above uniform."""
    g = np.random.default_rng(5)
    target = np.array([1.0, 1.8, 0.0])

    def batch(n):
        q, _, _ = problem(n, int(g.integers(1 << 30)))
        mu = target - q[:, :3]
        mu /= np.linalg.norm(mu, axis=1, keepdims=True)
        # vMF(mu, 30) samples: perturb and renormalise (close enough for a target)
        d = mu + g.normal(size=mu.shape) * 0.18
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        return q, d, np.ones(n)

    net = gpu_lib.Guide(BOX, 3)
    losses = [net.train_step(*batch(1 << 14), lr=3e-3) for _ in range(300)]
    print("loss first / last", losses[0], np.mean(losses[-20:]))
    assert np.mean(losses[-20:]) < losses[0] - 2.0
    q, d, _ = batch(4096)
    raw = net.forward(q).astype(np.float64)
    mean_pdf = np.exp(og.mixture_logpdf(raw, d)).mean()
    print("mean learned pdf at target samples", mean_pdf, "uniform", 1 / (4 * np.pi))
    assert mean_pdf > 10 / (4 * np.pi)
    net.close()
