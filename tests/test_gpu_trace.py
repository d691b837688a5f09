"""GPU traversal and BVH build against the oracle (bit-exact)."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from pathguidingdissertation_gb300 import scenes

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def _canonical(nodes, idx):
    """Tree as a sorted list of (triangle set, child sets): independent of
    node numbering and of triangle order inside leaves."""
    out = []

    def walk(i):
        n = nodes[i]
        if n["used"] > 0:
            s = tuple(sorted(idx[n["left_first"]:n["left_first"] + n["used"]].tolist()))
            out.append(("L", s))
            return s
        a = walk(n["left_first"])
        b = walk(n["left_first"] + 1)
        s = tuple(sorted(a + b))
        out.append(("I", s))
        return s

    walk(0)
    return sorted(out)


@pytest.mark.parametrize("path", sorted(GOLDEN.glob("traversal_*.npz")), ids=lambda p: p.stem)
def test_gpu_golden_traversal(ctx, path):
    g = np.load(path)
    desc = scenes.SceneDesc(g["triangles"], np.array([scenes.material()]), dict(
        from_=(0, 0, 5), to=(0, 0, 0), up=(0, 1, 0), fov=45.0, width=8, height=8))
    desc.triangles = g["triangles"].copy()
    desc.triangles["material"] = 0
    ctx.upload(desc)
    ctx.bvh_import(g["nodes"], g["idx"])
    hits = ctx.trace_closest(g["rays"])
    assert hits.tobytes() == g["hits"].tobytes()
    vis = ctx.trace_any(g["any_rays"])
    assert np.array_equal(vis, g["visible"])


@pytest.mark.parametrize("n,seed", [(36, 1), (5000, 2), (60000, 3)])
def test_gpu_build_matches_oracle_tree(ctx, oracle, n, seed):
    desc = scenes.cornell_box(seed=seed) if n == 36 else scenes.triangle_soup(n, seed=seed)
    ctx.upload(desc)
    ctx.bvh_build()
    nodes, idx = ctx.bvh_export()
    o_nodes, o_idx = oracle.bvh_build(desc.triangles)
    assert len(nodes) == len(o_nodes)
    assert _canonical(nodes, idx) == _canonical(o_nodes, o_idx)
    st = ctx.bvh_stats()
    assert st.sah_cost == pytest.approx(oracle.sah_cost(o_nodes), rel=1e-9)


def test_gpu_build_interior_sah(ctx, oracle):
    desc = scenes.interior(seed=4, target_tris=200_000, env_width=16, env_height=8)
    ctx.upload(desc)
    ctx.bvh_build()
    nodes, idx = ctx.bvh_export()
    o_nodes, o_idx = oracle.bvh_build(desc.triangles)
    st = ctx.bvh_stats()
    ref_cost = oracle.sah_cost(o_nodes)
    # Identical node sets give identical cost; the requirement is 3 %.
    assert abs(st.sah_cost - ref_cost) <= 0.03 * ref_cost
    assert st.sah_cost == pytest.approx(ref_cost, rel=1e-9)
    assert len(nodes) == len(o_nodes)
    assert sorted(idx.tolist()) == list(range(desc.ntris))


def test_gpu_trace_reference_tree_bit_exact(ctx, oracle):
    desc = scenes.interior(seed=6, target_tris=200_000, env_width=16, env_height=8)
    nodes, idx = oracle.bvh_build(desc.triangles)
    ctx.upload(desc)
    ctx.bvh_import(nodes, idx)
    rays = scenes.random_rays(*desc.bounds(), 10_000_000, seed=7)
    hits = ctx.trace_closest(rays)
    ref = oracle.trace_closest_mt(desc.triangles, nodes, idx, rays, 16)
    assert np.array_equal(hits["id"], ref["id"])
    assert hits.tobytes() == ref.tobytes()


def test_gpu_any_hit_bit_exact(ctx, oracle):
    desc = scenes.triangle_soup(20000, seed=12)
    nodes, idx = oracle.bvh_build(desc.triangles)
    ctx.upload(desc)
    ctx.bvh_import(nodes, idx)
    rays = scenes.random_rays(*desc.bounds(), 200_000, seed=9)
    h, _, _ = oracle.trace_closest(desc.triangles, nodes, idx, rays)
    for scale in (0.5, 1.0, 2.0):
        r = rays.copy()
        r["tmax"] = (np.where(h["id"] >= 0, h["t"], np.float32(4.0)) * np.float32(scale)).astype(np.float32)
        vis = ctx.trace_any(r)
        ref, _, _ = oracle.trace_any(desc.triangles, nodes, idx, r)
        assert np.array_equal(vis, ref)


def test_gpu_built_tree_hits_same_t(ctx, oracle):
    desc = scenes.triangle_soup(30000, seed=21)
    ctx.upload(desc)
    ctx.bvh_build()
    rays = scenes.random_rays(*desc.bounds(), 300_000, seed=4)
    hits = ctx.trace_closest(rays)
    nodes, idx = oracle.bvh_build(desc.triangles)
    ref, _, _ = oracle.trace_closest(desc.triangles, nodes, idx, rays)
    # Same node sets: only the order inside leaves differs, so t is identical
    # and ids differ only on exact ties.
    assert np.array_equal(hits["t"], ref["t"])
    assert np.mean(hits["id"] != ref["id"]) < 1e-4


def test_gpu_counters_match_oracle(ctx, oracle):
    desc = scenes.triangle_soup(5000, seed=30)
    nodes, idx = oracle.bvh_build(desc.triangles)
    ctx.upload(desc)
    ctx.bvh_import(nodes, idx)
    rays = scenes.random_rays(*desc.bounds(), 50_000, seed=1)
    ctx.trace_closest(rays)
    iv, tt = ctx.trace_counters()
    _, oiv, ott = oracle.trace_closest(desc.triangles, nodes, idx, rays)
    assert (iv, tt) == (oiv, ott)


def test_gpu_empty_and_errors(ctx):
    from pathguidingdissertation_gb300.abi import PgxError
    desc = scenes.triangle_soup(10, seed=1)
    ctx.upload(desc)
    with pytest.raises(PgxError):
        ctx.trace_closest(scenes.random_rays(*desc.bounds(), 4))  # no BVH yet
    ctx.bvh_build()
    assert len(ctx.trace_closest(scenes.random_rays(*desc.bounds(), 0))) == 0
    bad = desc.triangles.copy()
    bad["material"][3] = 7
    with pytest.raises(PgxError):
        ctx.upload(scenes.SceneDesc(bad, desc.materials, desc.camera))


def _camera_scenes():
    from oracle import build as ob
    from pathguidingdissertation_gb300 import loader
    out = [("cornell", lambda: scenes.cornell_box(seed=1, width=64, height=48)),
           ("interior", lambda: scenes.interior(seed=3, target_tris=2000, n_objects=8, width=80, height=45,
                                                env_width=16, env_height=8))]
    for name in ("cornell-box", "veach-mis", "dining-room"):
        out.append((name, lambda name=name: loader.load_scene(ob.scenes_dir() / name)))
    return out


@pytest.mark.parametrize("name,make", _camera_scenes(), ids=lambda x: x if isinstance(x, str) else "")
def test_camera_rays_match_reference(ctx, reference, name, make):
    """pgx_camera_rays against the reference's Camera::generateRay
    (Scene.h:45-57) on the same film positions: origins and directions
    bit-identical (pixel corners, centres, jittered positions, film edges)."""
    try:
        desc = make()
    except FileNotFoundError:
        pytest.skip("reference scene not staged")
    w, h = desc.camera["width"], desc.camera["height"]
    rng = np.random.default_rng(5)
    n = 20000
    px = np.concatenate([rng.random(n) * w, np.arange(w) + 0.5, np.arange(w, dtype=np.float64), [0.0, w - 1e-3]])
    py = np.concatenate([rng.random(n) * h, np.full(w, h * 0.5), np.zeros(w), [h - 1e-3, 0.0]])
    px, py = px.astype(np.float32), py.astype(np.float32)
    ctx.upload(desc)
    rays = ctx.camera_rays(px, py)
    rs = reference.scene(desc)
    o, d = rs.camera_rays(px, py)
    rs.close()
    assert rays["o"].tobytes() == o.tobytes()
    assert rays["d"].tobytes() == d.tobytes(), np.abs(rays["d"] - d).max()
