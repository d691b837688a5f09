"""Pins the CPU restatement of the learned guide (oracle/mlp_oracle.py) to
its own mathematics: the analytic gradient of the exact (float64) loss
against central finite differences, the mixture pdf's normalisation and the
sampler's distribution.  CPU only."""
from __future__ import annotations

import numpy as np

from oracle import mlp_oracle as mo

BMIN, BMAX = np.array([-1.0, 0.0, -2.0]), np.array([3.0, 2.0, 1.0])


def _samples(n, seed):
    rng = np.random.default_rng(seed)
    s = {
        "position": rng.uniform(BMIN, BMAX, (n, 3)),
        "normal": rng.standard_normal((n, 3)),
        "wo": rng.standard_normal((n, 3)),
        "wi": rng.standard_normal((n, 3)),
        "weight": rng.uniform(0.1, 2.0, n),
    }
    for k in ("normal", "wo", "wi"):
        s[k] /= np.linalg.norm(s[k], axis=1, keepdims=True)
    return s


def test_exact_gradient_matches_finite_differences():
    p = mo.init_params(3).astype(np.float64)
    s = _samples(64, 4)
    _, g = mo.loss_and_grad(p, s, BMIN, BMAX, exact=True)
    rng = np.random.default_rng(5)
    idx = rng.choice(mo.NPARAMS, 40, replace=False)
    # include bias entries and the last layer explicitly
    idx = np.concatenate([idx, [mo.OFFSETS[5][1] + 3, mo.OFFSETS[0][1] + 7, mo.OFFSETS[5][0] + 100]])

    def loss_of(params):
        # forward in float64 with params taken as float64 (no float32 cast)
        Ws, bs = [], []
        for (k, n), (ow, ob) in zip(mo.DIMS, mo.OFFSETS):
            Ws.append(params[ow:ow + n * k].reshape(n, k))
            bs.append(params[ob:ob + n])
        q = np.concatenate([s["position"], s["normal"], s["wo"]], axis=1)
        x = mo.encode(q, BMIN, BMAX)
        for l in range(mo.LAYERS):
            z = x @ Ws[l].T + bs[l]
            x = np.maximum(z, 0.0) if l < mo.LAYERS - 1 else z
        li, _ = mo.loss_grad_raw(x, s["wi"], s["weight"] / s["weight"].sum())
        return li.sum()

    h = 1e-6
    for i in idx:
        e = np.zeros(mo.NPARAMS)
        e[i] = h
        fd = (loss_of(p + e) - loss_of(p - e)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_raw_gradient_matches_finite_differences():
    rng = np.random.default_rng(7)
    raw = rng.standard_normal((16, 40)) * 1.5
    wi = rng.standard_normal((16, 3))
    wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    w = rng.uniform(0.5, 1.5, 16)
    _, d = mo.loss_grad_raw(raw, wi, w)
    h = 1e-6
    for j in range(40):
        e = np.zeros_like(raw)
        e[:, j] = h
        fd = (mo.loss_grad_raw(raw + e, wi, w)[0] - mo.loss_grad_raw(raw - e, wi, w)[0]) / (2 * h)
        np.testing.assert_allclose(d[:, j], fd, rtol=1e-5, atol=1e-7)


def _sphere_grid(n):
    # midpoint rule on (cos theta, phi): equal-area cells of 4 pi / n^2
    c = (np.arange(n) + 0.5) / n * 2.0 - 1.0
    phi = (np.arange(n) + 0.5) / n * 2.0 * np.pi
    cc, pp = np.meshgrid(c, phi, indexing="ij")
    s = np.sqrt(1.0 - cc ** 2)
    return np.stack([s * np.cos(pp), s * np.sin(pp), cc], -1).reshape(-1, 3), 4.0 * np.pi / (n * n)


def test_mixture_pdf_is_normalised():
    rng = np.random.default_rng(9)
    raw = rng.standard_normal((3, 40))
    raw[:, 32:40] = rng.uniform(-2, 4, (3, 8))   # kappa from ~0.1 to ~4
    d, da = _sphere_grid(600)
    for i in range(3):
        p = mo.mixture_pdf(np.repeat(raw[i:i + 1], len(d), 0), d)
        assert abs(p.sum() * da - 1.0) < 2e-3


def test_sampler_follows_pdf():
    rng = np.random.default_rng(11)
    raw = rng.standard_normal((1, 40))
    raw[:, 32:40] = rng.uniform(0, 3, 8)
    n = 200000
    u = rng.random((n, 3))
    d = mo.sample(np.repeat(raw, n, 0), u)
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0)
    # E[f(d)] under the sampler equals the pdf-weighted integral of f
    f = lambda x: (x[:, 2] + 1.0) ** 2 + 0.5 * x[:, 0]
    g, da = _sphere_grid(500)
    exact = (f(g) * mo.mixture_pdf(np.repeat(raw, len(g), 0), g)).sum() * da
    est = f(d).mean()
    assert abs(est - exact) < 4.0 * f(d).std() / np.sqrt(n)


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.0e38, 1e-40, 0.0])
    r = mo.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125  # ties to even, round up
    assert r[5] == 0.0
