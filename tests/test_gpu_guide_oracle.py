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


def _compare_trees(regions, qnodes, oracle_guide):
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
        for i, (flux, child) in enumerate(tree):
            q = qnodes[base + i]
            want = [c + base if c >= 0 else -1 for c in child]
            assert list(q["child"]) == want, (first, i)
            np.testing.assert_allclose(q["flux"], flux, rtol=1e-5, atol=1e-30)
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
    _compare_trees(regions, qnodes, go.Guide(nodes, out, pss=True))
