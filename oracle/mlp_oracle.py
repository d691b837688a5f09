"""CPU restatement of the learned guide (the MLP of include/pgx.h's
pgx_mlp_* functions and its von Mises-Fisher mixture) — TEST
INFRASTRUCTURE ONLY: tests/ use it as the checker of the tensor-core
forward and backward kernels; the product never imports it.

The reference has no learned component, so there is nothing to pin this
file to but its own mathematics: `loss_and_grad(..., exact=True)` runs in
float64 without any rounding and its analytic gradient is checked against
central finite differences (tests/test_mlp_oracle.py).  With exact=False it
rounds where the GPU rounds — inputs, weights and every hidden activation to
bfloat16 (round to nearest even, through float32), the loss gradient and the
back-propagated activation gradients to bfloat16 — and accumulates in
float64.
"""
from __future__ import annotations

import numpy as np

IN, HID, OUT, LAYERS, LOBES, FREQ = 80, 64, 40, 6, 8, 12
KAPPA_MIN = 0.01
DIMS = [(80, 64), (64, 64), (64, 64), (64, 64), (64, 64), (64, 40)]  # (k, n)


def param_offsets():
    offs, o = [], 0
    for k, n in DIMS:
        offs.append((o, o + n * k))
        o += n * k + n
    return offs, o


OFFSETS, NPARAMS = param_offsets()
assert NPARAMS == 24424


def unpack(params: np.ndarray):
    Ws, bs = [], []
    for (k, n), (ow, ob) in zip(DIMS, OFFSETS):
        Ws.append(params[ow:ow + n * k].reshape(n, k).astype(np.float64))
        bs.append(params[ob:ob + n].astype(np.float64))
    return Ws, bs


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to bfloat16 (nearest, ties to even) through float32."""
    f = np.asarray(x, np.float64).astype(np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    out = r.view(np.float32).astype(np.float64)
    nan = np.isnan(f)
    out[nan] = np.nan
    return out


def encode(queries: np.ndarray, bmin, bmax) -> np.ndarray:
    """The 80 input features of (position, normal, wo) queries (n x 9)."""
    q = np.asarray(queries, np.float64).reshape(-1, 9)
    bmin = np.asarray(bmin, np.float64)
    inv = 1.0 / (np.asarray(bmax, np.float64) - bmin)
    t = np.clip((q[:, 0:3] - bmin) * inv, 0.0, 1.0)
    feats = np.zeros((len(q), IN))
    for c in range(3):
        for j in range(FREQ):
            a = np.pi * (2.0 ** j) * t[:, c]
            feats[:, c * 24 + 2 * j] = np.sin(a)
            feats[:, c * 24 + 2 * j + 1] = np.cos(a)
    feats[:, 72:75] = q[:, 3:6]
    feats[:, 75:78] = q[:, 6:9]
    return feats


def forward(params, queries, bmin, bmax, exact: bool = False):
    """Raw outputs (n x 40) and each layer's input (for the backward pass)."""
    Ws, bs = unpack(np.asarray(params, np.float32))
    rnd = (lambda x: x) if exact else bf16
    x = rnd(encode(queries, bmin, bmax))
    acts = [x]
    for l in range(LAYERS):
        z = x @ rnd(Ws[l]).T + bs[l]
        if l < LAYERS - 1:
            x = rnd(np.maximum(z, 0.0))
            acts.append(x)
        else:
            return z, acts


def softplus(x):
    return np.where(x > 20.0, x, np.log1p(np.exp(np.minimum(x, 20.0))))


def mixture(raw: np.ndarray):
    """Lobe weights (n x 8), unit means (n x 8 x 3), concentrations (n x 8)."""
    raw = np.asarray(raw, np.float64)
    a = raw[:, 0:8]
    w = np.exp(a - a.max(axis=1, keepdims=True))
    w /= w.sum(axis=1, keepdims=True)
    m = raw[:, 8:32].reshape(-1, 8, 3)
    ln = np.linalg.norm(m, axis=2, keepdims=True)
    mu = m / np.maximum(ln, 1e-300)
    kappa = softplus(raw[:, 32:40]) + KAPPA_MIN
    return w, mu, kappa, ln[..., 0]


def vmf(mu, kappa, d):
    """vMF densities of direction(s) d (n x 3) per lobe: n x 8."""
    cosv = np.einsum("nij,nj->ni", mu, d)
    norm = kappa / (2.0 * np.pi * (-np.expm1(-2.0 * kappa)))
    return norm * np.exp(kappa * (cosv - 1.0)), cosv


def mixture_pdf(raw, d):
    w, mu, kappa, _ = mixture(raw)
    v, _ = vmf(mu, kappa, np.asarray(d, np.float64).reshape(-1, 3))
    return (w * v).sum(axis=1)


def loss_grad_raw(raw, wi, weight):
    """Per-sample loss -weight*log q(wi) and d loss / d raw (n x 40)."""
    raw = np.asarray(raw, np.float64)
    wi = np.asarray(wi, np.float64).reshape(-1, 3)
    weight = np.asarray(weight, np.float64).reshape(-1)
    w, mu, kappa, ln = mixture(raw)
    v, cosv = vmf(mu, kappa, wi)
    q = np.maximum((w * v).sum(axis=1), 1e-300)
    g = -weight / q
    d = np.zeros_like(raw)
    d[:, 0:8] = g[:, None] * w * (v - q[:, None])
    s = g[:, None] * w * v * kappa / np.maximum(ln, 1e-300)
    d[:, 8:32] = (s[:, :, None] * (wi[:, None, :] - cosv[:, :, None] * mu)).reshape(-1, 24)
    dlk = 1.0 / kappa - 2.0 / np.expm1(2.0 * kappa) + (cosv - 1.0)
    sig = 1.0 / (1.0 + np.exp(-raw[:, 32:40]))
    d[:, 32:40] = g[:, None] * w * v * dlk * sig
    return -weight * np.log(q), d


def loss_and_grad(params, samples, bmin, bmax, exact: bool = False):
    """Loss sum_i w_i (-log q(wi_i)) / sum_i w_i and its gradient with respect
    to the parameters, for samples with fields position, normal, wo, wi,
    weight (numpy structured array or dict of arrays)."""
    pos = np.asarray(samples["position"], np.float64)
    q = np.concatenate([pos, np.asarray(samples["normal"], np.float64), np.asarray(samples["wo"], np.float64)],
                       axis=1)
    wgt = np.asarray(samples["weight"], np.float64)
    scale = 1.0 / wgt.sum()
    raw, acts = forward(params, q, bmin, bmax, exact)
    li, d = loss_grad_raw(raw, samples["wi"], wgt * scale)
    rnd = (lambda x: x) if exact else bf16
    Ws, _ = unpack(np.asarray(params, np.float32))
    grad = np.zeros(NPARAMS)
    dy = rnd(d)
    for l in range(LAYERS - 1, -1, -1):
        (k, n), (ow, ob) = DIMS[l], OFFSETS[l]
        grad[ow:ow + n * k] = (dy.T @ acts[l]).reshape(-1)
        grad[ob:ob + n] = dy.sum(axis=0)
        if l > 0:
            dx = dy @ rnd(Ws[l])
            dy = rnd(dx * (acts[l] > 0))
    return li.sum(), grad


def sample(raw, u3):
    """Mixture sample with uniforms (lobe, cos, azimuth), as the GPU does."""
    w, mu, kappa, _ = mixture(raw)
    u3 = np.asarray(u3, np.float64).reshape(-1, 3)
    cdf = np.cumsum(w, axis=1)
    pick = np.minimum((u3[:, :1] >= cdf[:, :-1]).sum(axis=1), LOBES - 1)
    idx = np.arange(len(u3))
    m, k = mu[idx, pick], kappa[idx, pick]
    cw = np.clip(1.0 + np.log(u3[:, 1] + (1.0 - u3[:, 1]) * np.exp(-2.0 * k)) / k, -1.0, 1.0)
    sw = np.sqrt(np.maximum(0.0, 1.0 - cw * cw))
    phi = 2.0 * np.pi * u3[:, 2]
    sign = np.where(m[:, 2] >= 0, 1.0, -1.0)
    a = -1.0 / (sign + m[:, 2])
    b = m[:, 0] * m[:, 1] * a
    t = np.stack([1.0 + sign * m[:, 0] ** 2 * a, sign * b, -sign * m[:, 0]], 1)
    bt = np.stack([b, sign + m[:, 1] ** 2 * a, -m[:, 1]], 1)
    d = t * (sw * np.cos(phi))[:, None] + bt * (sw * np.sin(phi))[:, None] + m * cw[:, None]
    return d / np.linalg.norm(d, axis=1, keepdims=True)


def init_params(seed: int = 1) -> np.ndarray:
    """Random parameters for tests (not the device initialisation)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAMS, np.float32)
    for l, ((k, n), (ow, ob)) in enumerate(zip(DIMS, OFFSETS)):
        a = np.sqrt(6.0 / k) * (0.5 if l == LAYERS - 1 else 1.0)
        p[ow:ow + n * k] = rng.uniform(-a, a, n * k)
        p[ob:ob + n] = rng.uniform(-0.1, 0.1, n)
    return p
