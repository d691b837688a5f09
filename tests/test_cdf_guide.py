"""The guide tables that let the environment light sample skip most of its
CDF binary search (pgx_shade.cuh cdf_search_guided, scene.cu
build_cdf_guide), restated in numpy and checked on CPU: for every u the
guided search returns the index of Distribution1D::binarySearch
(Sampling.h:107-123), on CDFs with flat runs, steep steps and the i / n
CDF of an all-zero function.  (The GPU side is covered end to end by the
per-pixel render parity of the environment-lit scenes.)"""
from __future__ import annotations

import numpy as np

F = np.float32


def binary_search(cdf: np.ndarray, u: F) -> int:
    """Distribution1D::binarySearch: the last index whose cdf is <= u,
    clamped to [0, size - 2]."""
    first, it = 0, len(cdf)
    while it > 0:
        half = it // 2
        mid = first + half
        if cdf[mid] <= u:
            first = mid + 1
            it -= half + 1
        else:
            it = half
    return max(min(len(cdf) - 2, first - 1), 0)


def bucket(x: F, k: int) -> int:
    b = int(F(F(x) * F(k)))  # rounded float32 product, truncated
    return min(max(b, 0), k - 1)


def build_guide(cdf: np.ndarray, k: int) -> np.ndarray:
    g = np.zeros(k + 1, np.int64)
    last = -1
    for i, c in enumerate(cdf):
        b = bucket(c, k)
        for j in range(last + 1, b + 1):
            g[j] = i
        last = max(last, b)
    g[last + 1:] = len(cdf)
    return g


def guided_search(cdf: np.ndarray, u: F, g: np.ndarray, k: int) -> int:
    b = bucket(u, k)
    first, it = int(g[b]), int(g[b + 1] - g[b])
    while it > 0:
        half = it // 2
        mid = first + half
        if cdf[mid] <= u:
            first = mid + 1
            it -= half + 1
        else:
            it = half
    return max(min(len(cdf) - 2, first - 1), 0)


def distribution_cdf(func: np.ndarray) -> np.ndarray:
    """Distribution1D's constructor (Sampling.h:130-148) in float32."""
    n = len(func)
    cdf = np.zeros(n + 1, F)
    for i in range(1, n + 1):
        cdf[i] = F(cdf[i - 1] + F(F(func[i - 1]) / F(n)))
    total = cdf[n]
    if total == 0:
        cdf[1:] = (np.arange(1, n + 1, dtype=F) / F(n)).astype(F)
    else:
        cdf[1:] = (cdf[1:] / total).astype(F)
    return cdf


def test_guided_search_equals_binary_search():
    rng = np.random.default_rng(5)
    funcs = []
    n = 512
    f = rng.random(n).astype(F)
    f[100:300] = 0.0                                # flat run
    funcs.append(f)
    g = np.full(n, 1e-3, F)
    g[[7, 8, 400]] = 5e4                            # sun-like spikes
    funcs.append(g)
    funcs.append(np.zeros(n, F))                    # all zero: cdf = i / n
    funcs.append(np.exp(rng.normal(0, 4, n)).astype(F))
    funcs.append(np.zeros(n, F))
    funcs[-1][n // 2] = 1.0                         # a single non-zero bin
    for func in funcs:
        cdf = distribution_cdf(func)
        assert np.all(np.diff(cdf) >= 0)
        k = n
        gt = build_guide(cdf, k)
        assert gt[0] == 0 and gt[k] == len(cdf) and np.all(np.diff(gt) >= 0)
        us = np.concatenate([rng.random(20000).astype(F), cdf[:-1], np.nextafter(cdf[1:], F(0)),
                             np.array([0.0, np.nextafter(F(1), F(0))], F)])
        us = us[(us >= 0) & (us < 1)]
        for u in us:
            assert guided_search(cdf, F(u), gt, k) == binary_search(cdf, F(u)), (u,)


def test_guided_search_is_short():
    """On a smooth CDF the restricted search takes at most a step or two."""
    rng = np.random.default_rng(6)
    cdf = distribution_cdf((rng.random(2048) + 0.5).astype(F))
    gt = build_guide(cdf, 2048)
    assert int(np.max(np.diff(gt))) <= 4
