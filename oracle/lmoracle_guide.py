"""CPU oracle of the path-guiding network (TEST INFRASTRUCTURE ONLY).

An FP64 numpy statement of the network of
lightmetrica-v2_gb300/csrc/guide_net.cuh: the 128-feature input encoding,
the 4 x 64 ReLU MLP, the 8-lobe von Mises-Fisher mixture and the loss
-(1/n) sum w_i log q(d_i), with its gradient by hand-written
backpropagation.  The network has no counterpart in the reference; this
oracle is pinned by finite differences (tests/test_oracle_guide.py) and
checks the tensor-core forward and backward kernels (tests/test_gpu_guide.py).

Parameters are the flat FP32 array of the library (same layout):
W1[64][128] b1[64] W2[64][64] b2 W3 b3 W4 b4 W5[48][64] b5[48].
"""
from __future__ import annotations

import numpy as np

IN, HID, OUT, OUT_USED, LOBES, FREQS = 128, 64, 48, 40, 8, 16
KAPPA_MIN = 0.01


def layer_shapes():
    return [(HID, IN), (HID, HID), (HID, HID), (HID, HID), (OUT, HID)]


def unpack(params: np.ndarray):
    """(W_l, b_l) views of the flat parameter array."""
    p = np.asarray(params, np.float64)
    out, o = [], 0
    for rows, cols in layer_shapes():
        W = p[o:o + rows * cols].reshape(rows, cols)
        o += rows * cols
        b = p[o:o + rows]
        o += rows
        out.append((W, b))
    assert o == p.size
    return out


def num_params() -> int:
    return sum(r * c + r for r, c in layer_shapes())


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to bfloat16 (nearest even) and back."""
    a = np.asarray(x, np.float32).copy()
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def features(queries: np.ndarray, box_lo_hi) -> np.ndarray:
    """(n, 128) input features: sin/cos(2^(f/2) pi u), f = 0..15, of the
    box-normalised position per axis (axis-major, frequency, then sin/cos),
    normal, outgoing direction, zeros."""
    q = np.asarray(queries, np.float64).reshape(-1, 9)
    lo = np.asarray(box_lo_hi[:3], np.float64)
    hi = np.asarray(box_lo_hi[3:], np.float64)
    u = (q[:, :3] - lo) / np.where(hi - lo > 0, hi - lo, 1.0)
    f = np.zeros((q.shape[0], IN))
    for d in range(3):
        for k in range(FREQS):
            a = np.pi * u[:, d] * (2.0 ** (k // 2)) * (np.sqrt(2.0) if k % 2 else 1.0)
            f[:, d * 2 * FREQS + 2 * k] = np.sin(a)
            f[:, d * 2 * FREQS + 2 * k + 1] = np.cos(a)
    f[:, 6 * FREQS:6 * FREQS + 3] = q[:, 3:6]
    f[:, 6 * FREQS + 3:6 * FREQS + 6] = q[:, 6:9]
    return f


def forward(params, queries, box_lo_hi, emulate_bf16: bool = False):
    """Raw outputs (n, 40) and the activations [x, h1..h4] and
    pre-activations [z1..z5].  emulate_bf16 rounds what the tensor cores read
    (inputs, weights, hidden activations) to bfloat16."""
    layers = unpack(params)
    r = bf16 if emulate_bf16 else (lambda a: a)
    h = r(features(queries, box_lo_hi))
    acts, pre = [h], []
    for li, (W, b) in enumerate(layers):
        z = h @ r(W).T + b
        pre.append(z)
        if li < 4:
            h = r(np.maximum(z, 0.0))
            acts.append(h)
    return pre[-1][:, :OUT_USED], acts, pre


def softplus(x):
    return np.where(x > 20.0, x, np.log1p(np.exp(np.minimum(x, 20.0))))


def lobes(raw: np.ndarray):
    raw = np.asarray(raw, np.float64).reshape(-1, LOBES, 5)
    m = raw[:, :, :3]
    nm = np.maximum(np.linalg.norm(m, axis=2), 1e-6)
    mu = m / nm[:, :, None]
    braw = raw[:, :, 3]
    b = np.clip(braw, -20.0, 4000.0)
    kappa = KAPPA_MIN + softplus(b)
    sig = np.where((braw > -20.0) & (braw < 4000.0), 1.0 / (1.0 + np.exp(-b)), 0.0)
    a = raw[:, :, 4]
    logw = a - (a.max(axis=1, keepdims=True) + np.log(np.exp(a - a.max(axis=1, keepdims=True)).sum(axis=1,
                                                                                                   keepdims=True)))
    return mu, kappa, logw, nm, sig


def vmf_log_norm(k):
    return np.log(k / (2.0 * np.pi * -np.expm1(-2.0 * k)))


def mixture_logpdf(raw, dirs):
    mu, kappa, logw, _, _ = lobes(raw)
    d = np.asarray(dirs, np.float64).reshape(-1, 1, 3)
    c = (mu * d).sum(axis=2)
    l = logw + vmf_log_norm(kappa) + kappa * (c - 1.0)
    lmax = l.max(axis=1, keepdims=True)
    return (lmax + np.log(np.exp(l - lmax).sum(axis=1, keepdims=True)))[:, 0]


def loss_and_raw_grad(raw, dirs, weights):
    """Mean loss -(1/n) sum w log q and its gradient w.r.t. the raw outputs."""
    raw = np.asarray(raw, np.float64)
    n = raw.shape[0]
    mu, kappa, logw, nm, sig = lobes(raw)
    d = np.asarray(dirs, np.float64).reshape(-1, 1, 3)
    w = np.asarray(weights, np.float64).reshape(-1, 1) / n
    c = (mu * d).sum(axis=2)
    l = logw + vmf_log_norm(kappa) + kappa * (c - 1.0)
    lmax = l.max(axis=1, keepdims=True)
    lq = lmax + np.log(np.exp(l - lmax).sum(axis=1, keepdims=True))
    r = np.exp(l - lq)
    g = np.zeros((n, LOBES, 5))
    s = -w * r * kappa / nm
    g[:, :, :3] = s[:, :, None] * (d - c[:, :, None] * mu)
    dlogc = 1.0 / kappa - np.where(kappa > 40.0, 0.0, 2.0 / np.expm1(2.0 * np.minimum(kappa, 40.0)))
    g[:, :, 3] = -w * r * (dlogc + c - 1.0) * sig
    g[:, :, 4] = -w * (r - np.exp(logw))
    return float((-w[:, 0] * lq[:, 0]).sum()), g.reshape(n, OUT_USED)


def gradient(params, queries, box_lo_hi, dirs, weights):
    """FP64 loss and parameter gradient (flat, the library's layout)."""
    raw, acts, pre = forward(params, queries, box_lo_hi)
    loss, g_raw = loss_and_raw_grad(raw, dirs, weights)
    layers = unpack(params)
    dz = np.zeros((raw.shape[0], OUT))
    dz[:, :OUT_USED] = g_raw
    grads = [None] * 5
    for li in range(4, -1, -1):
        W, _ = layers[li]
        h = acts[li]
        grads[li] = (dz.T @ h, dz.sum(axis=0))
        if li > 0:
            dh = dz @ W
            dz = dh * (pre[li - 1] > 0.0)
    flat = []
    for gW, gb in grads:
        flat.append(gW.ravel())
        flat.append(gb)
    return loss, np.concatenate(flat)


def init_params(seed: int) -> np.ndarray:
    """A seeded He-uniform initialisation (for tests; the library has its own)."""
    g = np.random.default_rng(seed)
    out = []
    for li, (rows, cols) in enumerate(layer_shapes()):
        lim = np.sqrt(6.0 / (102 if li == 0 else cols)) * (0.1 if li == 4 else 1.0)
        W = g.uniform(-lim, lim, size=(rows, cols))
        if li == 4:
            W[OUT_USED:] = 0.0
        out.append(W.ravel())
        out.append(np.zeros(rows))
    return np.concatenate(out).astype(np.float32)
