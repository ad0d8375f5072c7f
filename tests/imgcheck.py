"""Statistical comparison of two Monte Carlo images with per-pixel variances.

Two unbiased estimates a, b of the same image give z = (a - b) /
sqrt(var_a + var_b) per pixel and channel, approximately standard normal
once each pixel holds enough samples.  Path-tracing estimates are
right-skewed (rare paths carry large throughput): at finite sample counts a
pixel that missed them has both a low value and a low variance estimate, so
per-pixel z is skewed negative.  The bar therefore has two parts:

  per pixel   std(z) in [0.8, 1.2], at most 1.5 % of |z| > 3, |mean z| < 0.25;
  aggregates  (where the central limit theorem holds) every 8 x 8 block mean
              within 4.5 sigma and the image total within 4 sigma, per channel
              -- these catch bias.
"""
import numpy as np


def _z(a, va, b, vb):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    v = np.asarray(va, np.float64) + np.asarray(vb, np.float64)
    m = v > 0
    return (a - b)[m] / np.sqrt(v[m]), m


def _blocks(x, v, f):
    H, W, C = x.shape
    h, w = H // f, W // f
    x = np.asarray(x, np.float64)[: h * f, : w * f].reshape(h, f, w, f, C).mean(axis=(1, 3))
    v = np.asarray(v, np.float64)[: h * f, : w * f].reshape(h, f, w, f, C).sum(axis=(1, 3)) / (f * f) ** 2
    return x, v


def compare(a, va, b, vb):
    z, m = _z(a, va, b, vb)
    v = np.asarray(va, np.float64) + np.asarray(vb, np.float64)
    tot = (np.asarray(a, np.float64).sum(axis=(0, 1)) - np.asarray(b, np.float64).sum(axis=(0, 1))) / np.sqrt(
        v.sum(axis=(0, 1)))
    H, W = np.asarray(a).shape[:2]
    f = max(1, min(H, W) // 8)
    ab, vab = _blocks(a, va, f)
    bb, vbb = _blocks(b, vb, f)
    zb, _ = _z(ab, vab, bb, vbb)
    return {"n": int(m.sum()), "mean_z": float(z.mean()), "std_z": float(z.std()),
            "frac_gt3": float(np.mean(np.abs(z) > 3)), "total_z": [float(x) for x in tot],
            "block_max_abs_z": float(np.abs(zb).max()) if zb.size else 0.0, "zero_both": int(np.sum(~m))}


def assert_same_image(a, va, b, vb, label="", block_limit=4.5):
    """block_limit: the bound on 8 x 8 block means; renderers whose samples
    share random state across pixels (VCM: every eye sample of a pass merges
    with the same photon subpaths) make neighbouring pixels correlated, which
    the per-pixel variances do not capture, and take a wider bound."""
    s = compare(a, va, b, vb)
    assert s["n"] > 0, (label, s)
    assert abs(s["mean_z"]) < 0.25, (label, s)
    assert 0.8 < s["std_z"] < 1.2, (label, s)
    assert s["frac_gt3"] < 0.015, (label, s)
    assert max(abs(x) for x in s["total_z"]) < 4.0, (label, s)
    assert s["block_max_abs_z"] < block_limit, (label, s)
    return s


def assert_same_aggregates(a, va, b, vb, label="", block_limit=4.5):
    """Bias check for low-sample renders, whose per-pixel statistics are not
    yet normal: image totals within 4 sigma and 8 x 8 block means within 4.5
    sigma, per channel."""
    s = compare(a, va, b, vb)
    assert max(abs(x) for x in s["total_z"]) < 4.0, (label, s)
    assert s["block_max_abs_z"] < block_limit, (label, s)
    return s


def relmse(img, ref, eps=1e-2, trim=0.0):
    """Relative MSE of img against ref: mean((img - ref)^2 / (ref^2 + eps)),
    per pixel on the channel mean; trim > 0 drops that fraction of the
    largest per-pixel errors first (outlier-robust form, for images whose
    error is dominated by a few fireflies)."""
    img = np.asarray(img, np.float64)
    ref = np.asarray(ref, np.float64)
    e = ((img - ref) ** 2 / (ref * ref + eps)).reshape(-1, img.shape[-1]).mean(axis=1)
    if trim > 0.0:
        e = np.sort(e)[: max(1, int(round(e.size * (1.0 - trim))))]
    return float(e.mean())
