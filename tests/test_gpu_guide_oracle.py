"""pgx's QuadTree guide against its CPU restatement (oracle/guide_oracle.py).

The GPU builds the radiance cache (point BVH, pinned to the reference's
PointBVHNode elsewhere) and one quadtree per region; the exported regions
and trees must equal the oracle's node for node (children identical, flux
within 1e-5 relative), and the guide's pdf and sample queries must agree
with the oracle's: pdf within 1e-5 relative, sampled directions the same
and the GPU's (direction, pdf) pairs consistent with the oracle's tree."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import guide_oracle as go
from pathguidingdissertation_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def _records(n, seed):
    """Positions in a box; directions from 40 tight lobes (deep chains that
    exhaust the 256-cell budget) plus a broad one; log-normal Li with zeros,
    negatives and non-finite values mixed in."""
    rng = np.random.default_rng(seed)
    r = np.zeros(n, abi.PATH_VERTEX)
    r["position"] = rng.uniform(-2, 2, (n, 3))
    r["normal"] = rng.normal(size=(n, 3))
    r["normal"] /= np.linalg.norm(r["normal"], axis=1, keepdims=True)
    centres = rng.normal(size=(40, 3))
    centres /= np.linalg.norm(centres, axis=1, keepdims=True)
    k = rng.integers(0, 40, n)
    spread = np.where(rng.random(n) < 0.25, 0.6, 1e-4)[:, None]
    d = centres[k] + spread * rng.normal(size=(n, 3))
    r["wi"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    li = np.exp(rng.normal(0, 1.5, (n, 1))) * rng.uniform(0.5, 1.5, (n, 3))
    bad = rng.random(n)
    li[bad < 0.05] = 0.0
    li[(bad >= 0.05) & (bad < 0.06)] = -1.0
    li[(bad >= 0.06) & (bad < 0.065), 0] = np.nan
    r["Li"] = li
    return r


def _compare_trees(regions, qnodes, oracle_guide, atol_rel=0.0):
    """atol_rel: absolute flux tolerance as a share of the region's total
    (MIS compensation subtracts nearly equal numbers)."""
    mine = sorted((int(r["first"]), int(r["count"]), int(r["node"])) for r in regions)
    assert mine == oracle_guide.regions
    by_first = {int(r["first"]): r for r in regions}
    n_full = 0
    for (first, count, node), tree in zip(oracle_guide.regions, oracle_guide.trees):
        reg = by_first[first]
        if tree is None:
            assert reg["qroot"] == -1
            continue
        base = int(reg["qroot"])
        assert base >= 0 and base % abi.GUIDE_MAX_QUAD_NODES == 0
        n_full += len(tree) == go.MAX_NODES
        atol = max(atol_rel * sum(tree[0][0]), 1e-30)
        for i, (flux, child) in enumerate(tree):
            q = qnodes[base + i]
            want = [c + base if c >= 0 else -1 for c in child]
            assert list(q["child"]) == want, (first, i)
            np.testing.assert_allclose(q["flux"], flux, rtol=1e-5, atol=atol)
        # nothing else is reachable from the root
        reach, stack = set(), [base]
        while stack:
            i = stack.pop()
            reach.add(i)
            stack += [int(c) for c in qnodes[i]["child"] if c >= 0]
        assert len(reach) == len(tree)
    return n_full


@pytest.mark.parametrize("n,seed", [(700, 1), (9000, 2), (40000, 3)])
def test_quadtrees_match_oracle(ctx, n, seed):
    ctx.upload(scenes.cornell_box(seed=1, width=8, height=8))
    recs = _records(n, seed)
    ctx.cache_build(recs)
    nodes, out = ctx.cache_export()
    regions, qnodes, pss = ctx.guide_export()
    assert not pss
    g = go.Guide(nodes, out)
    full = _compare_trees(regions, qnodes, g)
    assert len(g.regions) == (1 if n <= go.REGION_MAX else len(g.regions)) and len(g.regions) >= 1
    if n > 5000:
        assert full > 0  # the node budget is exercised

    # pdf and sample queries at positions inside and around the records
    rng = np.random.default_rng(seed + 10)
    m = 3000
    pos = np.concatenate([out["position"][rng.integers(0, n, m // 2)],
                          rng.uniform(-3, 3, (m - m // 2, 3))]).astype(np.float32)
    dirs = np.concatenate([out["wi"][rng.integers(0, n, m // 2)], rng.normal(size=(m - m // 2, 3))])
    dirs = (dirs / np.linalg.norm(dirs, axis=1, keepdims=True)).astype(np.float32)
    got = ctx.guide_pdf(pos, dirs)
    want = np.array([g.pdf(p, d) for p, d in zip(pos, dirs)])
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-12)

    u2 = rng.random((m, 2)).astype(np.float32)
    sd, sp = ctx.guide_sample(pos, u2)
    same = 0
    for i in range(m):
        o = g.sample(pos[i], float(u2[i, 0]), float(u2[i, 1]))
        if o is None:
            assert sp[i] == 0
            continue
        d, p = o
        same += np.abs(sd[i] - d).max() < 1e-4
        # the GPU's own sample is consistent with the oracle's tree
        assert abs(g.pdf(pos[i], sd[i]) - sp[i]) <= 1e-5 * max(sp[i], 1e-12) + 1e-12
    assert same >= 0.999 * np.count_nonzero(sp > 0)


def test_primary_sample_quadtrees_match_oracle(ctx):
    """Trees over the diffuse sampler's primary samples, built from the
    records of a PGX_MODE_GUIDED_PSS render of the small interior."""
    desc = scenes.interior(seed=3, target_tris=20000, n_objects=40, width=128, height=72, env_width=256,
                           env_height=128)
    ctx.upload(desc)
    ctx.bvh_build()
    ctx.clear()
    ctx.render(8, mode=abi.MODE_GUIDED_PSS, seed=5, max_depth=8, record_paths=8)
    nodes, out = ctx.cache_export()
    regions, qnodes, pss = ctx.guide_export()
    assert pss and len(out) > 2 * go.REGION_MAX
    _compare_trees(regions, qnodes, go.Guide(nodes, out, pss=True, weights=ctx.cache_weights()))


def test_render_built_quadtrees_match_oracle(ctx):
    """Direction-space trees from the records of a QuadTree-mode render
    guided by an earlier cache: the flux weights Lum(Li) |cos| / pdf the
    renderer attaches to its records go into the trees as the oracle
    builds them."""
    desc = scenes.interior(seed=3, target_tris=20000, n_objects=40, width=128, height=72, env_width=256,
                           env_height=128)
    ctx.upload(desc)
    ctx.bvh_build()
    ctx.clear()
    ctx.render(2, mode=abi.MODE_PLAIN, seed=5, max_depth=8, record_paths=2)
    ctx.clear()
    ctx.render(4, mode=abi.MODE_GUIDED_QUADTREE, seed=6, max_depth=8, record_paths=4)
    nodes, out = ctx.cache_export()
    w = ctx.cache_weights()
    regions, qnodes, pss = ctx.guide_export()
    assert not pss and len(out) > 2 * go.REGION_MAX and len(w) == len(out)
    assert np.count_nonzero(w > 0) > 0.5 * len(w)
    _compare_trees(regions, qnodes, go.Guide(nodes, out, weights=w))


def test_flux_weights(ctx):
    """Host records weigh by Lum(Li); the records of a plain render of an
    all-Lambertian box, whose directions the cosine sampler drew (pdf =
    cos / pi), weigh pi Lum(Li)."""
    ctx.upload(scenes.cornell_box(seed=1, width=8, height=8))
    recs = _records(3000, 4)
    ctx.cache_build(recs)
    _, out = ctx.cache_export()
    np.testing.assert_array_equal(ctx.cache_weights(), go.luminance(out["Li"]))

    ctx.upload(scenes.cornell_box(seed=2, width=48, height=48))
    ctx.bvh_build()
    ctx.clear()
    ctx.render(4, mode=abi.MODE_PLAIN, seed=3, max_depth=6, record_paths=4)
    _, out = ctx.cache_export()
    w = ctx.cache_weights()
    lum = go.luminance(out["Li"]).astype(np.float64)
    ok = lum > 0
    assert ok.sum() > 1000
    np.testing.assert_allclose(w[ok], np.pi * lum[ok], rtol=2e-5)


@pytest.mark.parametrize("params", [
    dict(region_records=4096, refine_fraction=0.005, clamp_median=0.0, uniform_share=0.05),
    dict(region_records=300, refine_fraction=0.03, clamp_median=100.0, uniform_share=0.5),
    dict(region_records=2048, refine_fraction=0.01, clamp_median=10.0, uniform_share=0.2, compensate=1.0),
])
def test_guide_params_match_oracle(ctx, params):
    """pgx_guide_configure: region size, refinement share and flux clamp of
    the next build, uniform share of later queries, against the oracle with
    the same parameters; out-of-range values are refused and change
    nothing."""
    ctx.upload(scenes.cornell_box(seed=1, width=8, height=8))
    ctx.guide_configure(**params)
    got = ctx.guide_params()
    for k, v in params.items():
        assert got[k] == pytest.approx(v)
    for bad in (dict(region_records=255), dict(refine_fraction=0.0), dict(clamp_median=-1.0),
                dict(uniform_share=1.0), dict(compensate=-0.5), dict(glossy_alpha=-1.0)):
        with pytest.raises(RuntimeError):
            ctx.guide_configure(**dict(params, **bad))
    assert ctx.guide_params() == got
    n = 20000
    recs = _records(n, 7)
    ctx.cache_build(recs)
    nodes, out = ctx.cache_export()
    regions, qnodes, _ = ctx.guide_export()
    g = go.Guide(nodes, out, region_max=params["region_records"], clamp_median=params["clamp_median"],
                 rho=params["refine_fraction"], compensate=params.get("compensate", 0.0))
    assert len(g.regions) > 1
    _compare_trees(regions, qnodes, g, atol_rel=1e-6 if params.get("compensate") else 0.0)
    rng = np.random.default_rng(8)
    m = 1000
    pos = out["position"][rng.integers(0, n, m)].astype(np.float32)
    dirs = rng.normal(size=(m, 3))
    dirs = (dirs / np.linalg.norm(dirs, axis=1, keepdims=True)).astype(np.float32)
    # compensated leaves carry the rounding of a difference of nearly equal
    # fluxes: an absolute tolerance of 1e-7 (pdf ~ 1 / 4 pi on average)
    np.testing.assert_allclose(ctx.guide_pdf(pos, dirs), [g.pdf(p, d) for p, d in zip(pos, dirs)],
                               rtol=1e-5, atol=1e-7 if params.get("compensate") else 1e-12)
