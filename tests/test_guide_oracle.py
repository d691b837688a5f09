"""The QuadTree guide's CPU restatement (oracle/guide_oracle.py) checked
against its own mathematics, CPU only: the tree's density integrates to 1
over the unit square, refinement follows the 1 % flux rule and the caps,
sampling follows the density, and the cosine sampler's inverse round-trips
through the reference's sampler formula (Materials.h:163-171)."""
from __future__ import annotations

import numpy as np

from oracle import guide_oracle as go

PV = np.dtype([("position", "<f4", 3), ("normal", "<f4", 3), ("wi", "<f4", 3), ("Li", "<f4", 3)])


def lobes_records(n, seed, lobes=6, spread=0.05, bright=None):
    rng = np.random.default_rng(seed)
    r = np.zeros(n, PV)
    r["position"] = rng.uniform(-1, 1, (n, 3))
    r["normal"] = rng.normal(size=(n, 3))
    centres = rng.normal(size=(lobes, 3))
    centres /= np.linalg.norm(centres, axis=1, keepdims=True)
    k = rng.integers(0, lobes, n)
    d = centres[k] + spread * rng.normal(size=(n, 3))
    r["wi"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    r["Li"] = np.exp(rng.normal(0, 1, (n, 1))) * np.ones((1, 3)) if bright is None else bright
    return r


def test_luminance_filters_invalid():
    li = np.array([[1, 1, 1], [0, 0, 0], [-1, 0, 0], [np.nan, 0, 0], [np.inf, 0, 0]], np.float32)
    w = go.luminance(li)
    assert w[0] > 0 and np.all(w[1:] == 0)


def _leaves(tree):
    """(u0, v0, size, probability mass) of every leaf cell of a tree."""
    out = []
    stack = [(0, 0.0, 0.0, 1.0, 1.0)]
    while stack:
        node, u0, v0, size, mass = stack.pop()
        flux, child = tree[node]
        total = sum(flux)
        for c in range(4):
            cu, cv, h = u0 + 0.5 * size * (c & 1), v0 + 0.5 * size * (c >> 1), 0.5 * size
            m = mass * flux[c] / total
            if child[c] >= 0:
                stack.append((child[c], cu, cv, h, m))
            else:
                out.append((cu, cv, h, m))
    return out


def test_tree_density_integrates_to_one():
    """The leaves' masses sum to 1 and quad_pdf at each leaf's centre is its
    mass over its area."""
    tree = go.build_quadtree(lobes_records(900, 1))
    leaves = _leaves(tree)
    assert abs(sum(m for *_, m in leaves) - 1.0) < 1e-12
    for u0, v0, h, m in leaves:
        assert abs(go.quad_pdf(tree, u0 + 0.5 * h, v0 + 0.5 * h) * h * h - m) <= 1e-12 + 1e-9 * m


def test_refinement_rule_and_caps():
    recs = lobes_records(1000, 2, lobes=40, spread=1e-6)
    tree = go.build_quadtree(recs)
    assert len(tree) == go.MAX_NODES  # forty tight lobes exhaust the node budget
    w = np.minimum(go.luminance(recs["Li"]), go.CLAMP_MEDIAN * go.median_bisection(go.luminance(recs["Li"])))
    total = float(w.astype(np.float64).sum())
    depth = {0: 0}
    for i, (flux, child) in enumerate(tree):
        for c in range(4):
            if child[c] >= 0:
                assert flux[c] > 0.01 * total
                depth[child[c]] = depth[i] + 1
    assert max(depth.values()) <= go.MAX_DEPTH - 1
    single = go.build_quadtree(lobes_records(500, 3, lobes=1, spread=0.0))
    assert len(single) == go.MAX_DEPTH  # one direction: a chain down to the depth cap


def test_sampling_follows_density():
    tree = go.build_quadtree(lobes_records(800, 4, lobes=3, spread=0.2))
    rng = np.random.default_rng(0)
    n = 40000
    uv = np.array([go.quad_sample(tree, *rng.random(2)) for _ in range(n)])
    bins = 8
    h, _, _ = np.histogram2d(uv[:, 0], uv[:, 1], bins=bins, range=[[0, 1], [0, 1]])
    expect = np.zeros((bins, bins))
    for u0, v0, sz, m in _leaves(tree):
        # a leaf larger than a bin spreads its mass evenly over the bins it covers
        k = max(1, int(round(sz * bins)))
        i0, j0 = int(u0 * bins + 1e-9), int(v0 * bins + 1e-9)
        expect[i0:i0 + k, j0:j0 + k] += m / (k * k)
    expect *= n
    m = expect > 20
    chi2 = float((((h - expect) ** 2) / np.maximum(expect, 1e-9))[m].sum())
    assert chi2 < 3 * m.sum(), chi2
    for r in rng.random((200, 2)):
        u, v = go.quad_sample(tree, *r)
        assert go.quad_pdf(tree, u, v) > 0


def test_pss_uv_inverts_the_cosine_sampler():
    """u = cos^2 theta, v = phi / 2 pi inverts the sampler theta =
    acos(sqrt(u)), phi = 2 pi v of DiffuseBSDF::sample (Materials.h:147-160)."""
    rng = np.random.default_rng(1)
    n = rng.normal(size=(500, 3)).astype(np.float32)
    uv = rng.uniform(0.02, 0.98, (500, 2))
    fu, fv, fw = go._frame(n)
    th = np.arccos(np.sqrt(uv[:, 0]))
    ph = 2 * np.pi * uv[:, 1]
    loc = np.stack([np.cos(ph) * np.sin(th), np.sin(ph) * np.sin(th), np.cos(th)], 1)
    wi = (fu * loc[:, :1] + fv * loc[:, 1:2] + fw * loc[:, 2:]).astype(np.float32)
    u, v, ok = go.pss_uv(n, wi)
    assert ok.all()
    assert np.abs(u - uv[:, 0]).max() < 1e-4 and np.abs(v - uv[:, 1]).max() < 1e-4


def test_regions_from_a_median_split_tree():
    nodes = np.zeros(7, [("bmin", "<f4", 3), ("bmax", "<f4", 3), ("left", "<i4"), ("right", "<i4"),
                         ("offset", "<i4"), ("used", "<i4")])
    # root 3000 -> 1500 + 1500 -> (750, 750) + (750, 750)
    # interior nodes carry no range of their own (as exported): it comes from the leaves
    spec = [(1, 2, 0, 0), (3, 4, 0, 0), (5, 6, 0, 0), (-1, -1, 0, 750), (-1, -1, 750, 750),
            (-1, -1, 1500, 750), (-1, -1, 2250, 750)]
    for i, (l, r, o, u) in enumerate(spec):
        nodes[i]["left"], nodes[i]["right"], nodes[i]["offset"], nodes[i]["used"] = l, r, o, u
    assert go.regions_from_bvh(nodes, 3000) == [(0, 750, 3), (750, 750, 4), (1500, 750, 5), (2250, 750, 6)]
    assert go.regions_from_bvh(nodes[:1], 800) == [(0, 800, 0)]


def test_mis_compensation():
    """Compensated trees: each leaf's mass is its flux less alpha x the mean
    flux over its area, floored at 0, renormalised; the density still
    integrates to 1 and a uniform tree is left unchanged (nothing would
    remain)."""
    recs = lobes_records(4000, 5, lobes=3, spread=0.1)
    plain = go.build_quadtree(recs)
    comp = go.build_quadtree(recs, compensate=1.0)
    assert [c for _, c in comp] == [c for _, c in plain]
    lp, lc = _leaves(plain), _leaves(comp)
    assert abs(sum(m for *_, m in lc) - 1.0) < 1e-12
    kept = [max(m - h * h, 0.0) for (*_, h, m) in lp]  # mass - alpha * area, alpha = 1
    norm = sum(kept)
    for (u0, v0, h, m), k in zip(lc, kept):
        assert abs(m - k / norm) <= 1e-9
    # the compensated density is sharper where the plain one is high
    assert max(m / (h * h) for *_, h, m in lc) > max(m / (h * h) for *_, h, m in lp)
    # a uniform field: compensation would remove everything, the tree stays
    rng = np.random.default_rng(6)
    u = np.zeros(20000, PV)
    d = rng.normal(size=(20000, 3))
    u["wi"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    u["Li"] = 1.0
    assert go.build_quadtree(u, compensate=1.0) == go.build_quadtree(u)


def test_pdf_weighted_records_do_not_inherit_the_sampler():
    """Records weighted by Lum(Li) |cos| / pdf (what the renderer attaches)
    build the same tree whichever distribution sampled their directions:
    from cosine-sampled directions and from directions drawn by a sharply
    peaked guide, the trees' densities agree (both estimate Li |cos|), while
    the unweighted deposits follow the sampler (the compounding that
    iterated training suffered from)."""
    rng = np.random.default_rng(11)
    n = 200_000
    light = np.array([0.3, 0.2, 0.93])
    light /= np.linalg.norm(light)

    def li_of(w):
        # a bright lobe plus a dim sky, seen from a surface with normal +z
        return 5.0 * np.exp(40.0 * (w @ light - 1.0)) + 0.2

    def cosine(m):
        r1, r2 = rng.random(m), rng.random(m)
        s = np.sqrt(r1)
        w = np.stack([s * np.cos(2 * np.pi * r2), s * np.sin(2 * np.pi * r2), np.sqrt(1 - r1)], 1)
        return w, w[:, 2] / np.pi

    def peaked(m):
        # mixture: 70 % a narrow cone around (-0.6, 0, 0.8), 30 % cosine
        axis = np.array([-0.6, 0.0, 0.8])
        k = 30.0
        pick = rng.random(m) < 0.7
        wc, _ = cosine(m)
        u = rng.random(m)
        ct = 1.0 + np.log(u + (1 - u) * np.exp(-2 * k)) / k   # vMF about +z
        st = np.sqrt(np.maximum(0, 1 - ct * ct))
        ph = 2 * np.pi * rng.random(m)
        loc = np.stack([st * np.cos(ph), st * np.sin(ph), ct], 1)
        # rotate +z to axis
        t = np.cross([0.0, 0.0, 1.0], axis)
        ang = np.arccos(axis[2])
        t /= np.linalg.norm(t)
        K = np.array([[0, -t[2], t[1]], [t[2], 0, -t[0]], [-t[1], t[0], 0]])
        R = np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K
        wv = loc @ R.T
        w = np.where(pick[:, None], wv, wc)
        vmf = k / (2 * np.pi * (1 - np.exp(-2 * k))) * np.exp(k * (w @ axis - 1))
        pdf = 0.7 * vmf + 0.3 * np.maximum(w[:, 2], 0) / np.pi
        keep = w[:, 2] > 0
        return w[keep], pdf[keep]

    probe = rng.normal(size=(4000, 3))
    probe[:, 2] = np.abs(probe[:, 2])
    probe /= np.linalg.norm(probe, axis=1, keepdims=True)
    pu, pv = go.dir_to_uv(probe.astype(np.float32))

    def tree_density(w, weights):
        r = np.zeros(len(w), PV)
        r["wi"] = w
        r["Li"] = 1.0
        t = go.build_quadtree(r, clamp_median=0.0, weights=weights)
        return np.array([go.quad_pdf(t, float(a), float(b)) for a, b in zip(pu, pv)])

    w1, p1 = cosine(n)
    w2, p2 = peaked(n)
    d1 = tree_density(w1, (li_of(w1) * w1[:, 2] / p1).astype(np.float32))
    d2 = tree_density(w2, (li_of(w2) * w2[:, 2] / p2).astype(np.float32))
    # both approximate the same density, Li |cos| (up to the cells' averaging
    # and the noise of 200k samples), where it is large
    target = li_of(probe) * probe[:, 2]
    mask = target > 0.5 * target.max()
    assert mask.sum() > 20
    assert np.median(np.abs(d1[mask] - d2[mask]) / d1[mask]) < 0.25
    # unweighted deposits of the peaked sampler pile up around its axis
    d3 = tree_density(w2, go.luminance(np.repeat(li_of(w2)[:, None], 3, 1)).astype(np.float32))
    near = probe @ np.array([-0.6, 0.0, 0.8]) > 0.95
    assert near.sum() > 20
    assert d3[near].mean() > 3 * d1[near].mean()
