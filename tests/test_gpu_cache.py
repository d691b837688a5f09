"""Radiance cache (point BVH), k-NN and the QuadTree guide on the GPU.

* Point BVH vs the reference's PointBVHNode (Renderer.h:85-142,189-211):
  with distinct coordinates every node holds the same record set; the
  reference's validate() invariants (Renderer.h:144-161) hold in general.
* k-NN vs a float32 brute force (the reference has no cache query).
* Guide: pdf normalisation, sample/pdf consistency, and an unbiased guided
  estimator (same expectation as plain path tracing)."""
from __future__ import annotations

import numpy as np
import pytest

from pathguidingdissertation_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def _records(n, seed=0, ties=False):
    rng = np.random.default_rng(seed)
    r = np.zeros(n, abi.PATH_VERTEX)
    # Distinct coordinates on every axis (a jittered permutation per axis), so
    # every median split is unique and the node sets must match exactly.
    ext = np.array([6.0, 2.0, 4.0])
    pos = np.stack([(rng.permutation(n) + rng.uniform(0.1, 0.9, n)) / n for _ in range(3)], 1) * ext - ext / 2
    if ties:
        pos[: n // 3, 1] = 0.0  # a floor: many equal y coordinates
        pos[n // 3: n // 2] = np.round(pos[n // 3: n // 2], 1)
    r["position"] = pos.astype(np.float32)
    r["normal"] = [0, 1, 0]
    d = rng.normal(size=(n, 3))
    r["wi"] = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    r["Li"][:, 0] = np.arange(n, dtype=np.float32)  # identity
    r["Li"][:, 1] = rng.uniform(0.1, 2.0, n).astype(np.float32)
    return r


def _canonical(nodes, recs, left="left", right="right"):
    ids = recs["Li"][:, 0].astype(np.int64)
    out = []

    def walk(i):
        n = nodes[i]
        if n[left] < 0:
            s = tuple(sorted(ids[n["offset"]:n["offset"] + n["used"]].tolist()))
        else:
            s = tuple(sorted(walk(n[left]) + walk(n[right])))
        out.append(s)
        return s

    walk(0)
    return sorted(out)


def _validate(nodes, recs, eps=1e-4):
    """PointBVHNode::validate (Renderer.h:144-161,213-217)."""
    pos = recs["position"]
    count = 0
    stack = [0]
    while stack:
        i = stack.pop()
        n = nodes[i]
        if n["left"] < 0:
            assert n["used"] <= 8
            p = pos[n["offset"]:n["offset"] + n["used"]]
            assert np.all(p >= n["bmin"] - eps) and np.all(p <= n["bmax"] + eps)
            count += n["used"]
        else:
            assert n["used"] == 0
            for c in (n["left"], n["right"]):
                assert np.all(nodes[c]["bmin"] >= n["bmin"] - eps) and np.all(nodes[c]["bmax"] <= n["bmax"] + eps)
                stack.append(c)
    assert count == len(recs)


@pytest.mark.parametrize("n", [5, 300, 5000, 120000])
def test_point_bvh_matches_reference(ctx, reference, n):
    recs = _records(n, seed=n)
    ctx.cache_build(recs)
    nodes, out = ctx.cache_export()
    r_nodes, r_out = reference.pointbvh(recs)
    assert len(nodes) == len(r_nodes)
    assert _canonical(nodes, out) == _canonical(r_nodes, r_out)
    st = ctx.cache_stats()
    assert st.records == n and st.nodes == len(r_nodes)
    _validate(nodes, out)


def test_point_bvh_invariants_with_ties(ctx):
    recs = _records(30000, seed=3, ties=True)
    ctx.cache_build(recs)
    nodes, out = ctx.cache_export()
    _validate(nodes, out)
    assert sorted(out["Li"][:, 0].tolist()) == list(range(len(recs)))
    st = ctx.cache_stats()
    assert st.leaves == np.sum(nodes["left"] < 0)


@pytest.mark.parametrize("k", [1, 8, 32])
def test_knn_matches_bruteforce(ctx, k):
    recs = _records(20000, seed=7)
    ctx.cache_build(recs)
    _, out = ctx.cache_export()
    rng = np.random.default_rng(1)
    q = (rng.uniform(-0.5, 0.5, (500, 3)) * np.array([6.0, 2.0, 4.0])).astype(np.float32)
    idx, d2 = ctx.cache_knn(q, k)
    p = out["position"]
    for i in range(len(q)):
        d = p - q[i]
        dd = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        order = np.lexsort((np.arange(len(dd)), dd))[:k]
        assert np.array_equal(idx[i], order), i
        assert np.array_equal(d2[i], dd[order])


def test_knn_edge_cases(ctx):
    from pathguidingdissertation_gb300.abi import PgxError
    recs = _records(5, seed=2)
    ctx.cache_build(recs)
    idx, d2 = ctx.cache_knn(np.zeros((3, 3), np.float32), 8)
    assert np.all(idx[:, 5:] == -1) and np.all(np.isinf(d2[:, 5:]))
    with pytest.raises(PgxError):
        ctx.cache_knn(np.zeros((1, 3), np.float32), 65)


def _guided_scene(ctx, desc, depth=8, training="guided_li"):
    ctx.upload(desc)
    ctx.bvh_build()
    ctx.clear()
    if training == "guided_li":
        ctx.render(1, mode=abi.MODE_GUIDED_LI, seed=77, max_depth=depth, record_paths=True)
    else:
        ctx.render(2, mode=abi.MODE_PLAIN, seed=77, max_depth=depth, record_paths=2)
    st = ctx.cache_stats()
    assert st.records > 0
    ctx.clear()


def _uv_grid_dirs(res):
    """Directions at the centres of a res x res grid over the equal-area
    (u, v) square of the guide: u = (cos(theta) + 1) / 2, v = (phi + pi) / 2pi."""
    c = (np.arange(res) + 0.5) / res
    u, v = np.meshgrid(c, c, indexing="ij")
    ct = 2.0 * u.ravel() - 1.0
    st = np.sqrt(np.maximum(0.0, 1.0 - ct * ct))
    phi = 2.0 * np.pi * v.ravel() - np.pi
    return np.stack([st * np.cos(phi), st * np.sin(phi), ct], -1).astype(np.float32)


def test_guide_pdf_normalised_and_consistent(ctx):
    desc = scenes.interior(seed=3, target_tris=20000, n_objects=40, width=96, height=54, env_width=256,
                           env_height=128)
    _guided_scene(ctx, desc)
    _, recs = ctx.cache_export()
    rng = np.random.default_rng(0)
    pts = recs["position"][rng.choice(len(recs), 6, replace=False)]
    # The finest quadtree cells are 2^-10 wide: a 1024^2 grid of cell centres
    # integrates the piecewise-constant pdf exactly.
    grid = _uv_grid_dirs(1024)
    m = len(grid)
    checked = 0
    for x in pts:
        xs = np.repeat(x[None], m, 0)
        pdf = ctx.guide_pdf(xs, grid)
        if pdf.max() == 0:
            continue  # region without recorded flux
        checked += 1
        integral = pdf.astype(np.float64).mean() * 4 * np.pi
        assert abs(integral - 1.0) < 1e-3, integral
        u = rng.random((200000, 2)).astype(np.float32)
        dirs, spdf = ctx.guide_sample(xs[:200000], u)
        again = ctx.guide_pdf(xs[:200000], dirs)
        assert np.allclose(again, spdf, rtol=1e-3, atol=1e-6)
        # First moment of z: sampled mean vs the exact pdf-weighted grid mean.
        z_exact = (grid[:, 2].astype(np.float64) * pdf * 4 * np.pi).mean()
        assert abs(dirs[:, 2].mean() - z_exact) < 0.01
    assert checked > 0


def test_plain_recording_records(ctx):
    """Cache training from the NEE+MIS estimator: Li is finite and positive,
    at most one record per path and depth, and only recorded frames count."""
    desc = scenes.cornell_box(seed=1, width=32, height=32)
    ctx.upload(desc)
    ctx.bvh_build()
    ctx.clear()
    ctx.render(3, mode=abi.MODE_PLAIN, seed=3, max_depth=8, record_paths=1)
    st = ctx.render_stats()
    assert 0 < st.path_vertices <= 32 * 32 * 9
    _, recs = ctx.cache_export()
    assert len(recs) == st.path_vertices
    li = recs["Li"]
    assert np.all(np.isfinite(li)) and np.all(li.min(axis=1) >= 0)
    lum = 0.2126 * li[:, 0] + 0.7152 * li[:, 1] + 0.0722 * li[:, 2]
    assert np.all(lum > 0)
    n1 = len(recs)
    ctx.render(3, mode=abi.MODE_PLAIN, seed=3, max_depth=8, record_paths=3)
    assert ctx.render_stats().path_vertices > 2 * n1


@pytest.mark.parametrize("training", ["guided_li", "plain", "plain_recipe"])
@pytest.mark.parametrize("scene", ["cornell", "interior"])
def test_guided_estimator_unbiased(ctx, scene, training):
    """plain_recipe: the cache of the measured recipe (16,384-record
    regions, conductors narrower than alpha 0.7 left to their BSDF)."""
    if scene == "cornell":
        desc = scenes.cornell_box(seed=1, width=48, height=48)
    else:
        desc = scenes.interior(seed=3, target_tris=20000, n_objects=40, width=48, height=27, env_width=256,
                               env_height=128)
    if training == "plain_recipe":
        ctx.guide_configure(region_records=16384, glossy_alpha=0.7)
        training = "plain"
    _guided_scene(ctx, desc, training=training)
    spp = 1024
    ctx.render(spp, mode=abi.MODE_PLAIN, seed=5, max_depth=8)
    a, a2, _ = ctx.film(squares=True)
    ctx.clear()
    ctx.render(spp, mode=abi.MODE_GUIDED_QUADTREE, seed=6, max_depth=8, guide_fraction=0.5)
    b, b2, _ = ctx.film(squares=True)
    t = 8
    H, W = a.shape[:2]

    def tiles(x):
        return x[: H // t * t, : W // t * t].reshape(H // t, t, W // t, t, 3).sum(axis=(1, 3))

    n = spp * t * t
    ma, mb = tiles(a) / n, tiles(b) / n
    va = np.maximum(tiles(a2) / n - ma * ma, 0) / n
    vb = np.maximum(tiles(b2) / n - mb * mb, 0) / n
    z = np.abs(ma - mb) / np.sqrt(va + vb + 1e-12)
    assert np.mean(z < 4.0) > 0.97, np.sort(z.ravel())[-5:]
    # Whole image: the difference of the two means against its standard error.
    z_total = abs(ma.sum() - mb.sum()) / np.sqrt(va.sum() + vb.sum())
    assert z_total < 4.0, z_total


@pytest.mark.parametrize("scene", ["cornell", "interior"])
def test_pss_guided_estimator_unbiased(ctx, scene):
    """PGX_MODE_GUIDED_PSS: the cache is trained by renders in the mode itself
    (the first unguided, the next guided by the first's primary-sample
    trees); the guided image then agrees with plain path tracing per tile."""
    if scene == "cornell":
        desc = scenes.cornell_box(seed=1, width=48, height=48)
    else:
        desc = scenes.interior(seed=3, target_tris=20000, n_objects=40, width=48, height=27, env_width=256,
                               env_height=128)
    ctx.upload(desc)
    ctx.bvh_build()
    ctx.clear()
    ctx.render(2, mode=abi.MODE_GUIDED_PSS, seed=77, max_depth=8, record_paths=2)
    assert ctx.cache_stats().records > 0
    ctx.clear()
    ctx.render(4, mode=abi.MODE_GUIDED_PSS, seed=78, max_depth=8, record_paths=4, guide_fraction=0.5)
    ctx.clear()
    spp = 1024
    ctx.render(spp, mode=abi.MODE_PLAIN, seed=5, max_depth=8)
    a, a2, _ = ctx.film(squares=True)
    ctx.clear()
    ctx.render(spp, mode=abi.MODE_GUIDED_PSS, seed=6, max_depth=8, guide_fraction=0.5)
    b, b2, _ = ctx.film(squares=True)
    assert not np.array_equal(a, b)
    t = 8
    H, W = a.shape[:2]

    def tiles(x):
        return x[: H // t * t, : W // t * t].reshape(H // t, t, W // t, t, 3).sum(axis=(1, 3))

    n = spp * t * t
    ma, mb = tiles(a) / n, tiles(b) / n
    va = np.maximum(tiles(a2) / n - ma * ma, 0) / n
    vb = np.maximum(tiles(b2) / n - mb * mb, 0) / n
    z = np.abs(ma - mb) / np.sqrt(va + vb + 1e-12)
    assert np.mean(z < 4.0) > 0.97, np.sort(z.ravel())[-5:]
    z_total = abs(ma.sum() - mb.sum()) / np.sqrt(va.sum() + vb.sum())
    assert z_total < 4.0, z_total


def test_pss_cache_refuses_direction_use(ctx):
    """A cache built by a PSS render holds primary-sample trees: the
    direction-space queries and the QuadTree mode refuse it."""
    desc = scenes.cornell_box(seed=1, width=32, height=32)
    ctx.upload(desc)
    ctx.bvh_build()
    ctx.clear()
    ctx.render(2, mode=abi.MODE_GUIDED_PSS, seed=7, max_depth=8, record_paths=2)
    _, recs = ctx.cache_export()
    x = recs["position"][:4].astype(np.float32)
    d = np.tile(np.array([[0.0, 1.0, 0.0]], np.float32), (4, 1))
    with pytest.raises(abi.PgxError):
        ctx.guide_pdf(x, d)
    with pytest.raises(abi.PgxError):
        ctx.render(1, mode=abi.MODE_GUIDED_QUADTREE, seed=7, max_depth=8)
    # a plain recording rebuilds it in direction space
    ctx.render(2, mode=abi.MODE_PLAIN, seed=7, max_depth=8, record_paths=2)
    assert ctx.guide_pdf(x, d).shape == (4,)
