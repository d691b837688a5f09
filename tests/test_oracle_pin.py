"""Pins the oracle (C restatement) to the reference: against the committed
golden fixtures everywhere, and against the reference compiled headless
where its sources are available."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from pathguidingdissertation_gb300 import scenes

GOLDEN = Path(__file__).resolve().parent / "golden"
FIXTURES = sorted(GOLDEN.glob("traversal_*.npz"))


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: p.stem)
def test_oracle_bvh_matches_golden(oracle, path):
    g = np.load(path)
    nodes, idx = oracle.bvh_build(g["triangles"])
    assert nodes.tobytes() == g["nodes"].tobytes()
    assert np.array_equal(idx, g["idx"])


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: p.stem)
def test_oracle_hits_match_golden(oracle, path):
    g = np.load(path)
    hits, _, _ = oracle.trace_closest(g["triangles"], g["nodes"], g["idx"], g["rays"])
    assert hits.tobytes() == g["hits"].tobytes()
    vis, _, _ = oracle.trace_any(g["triangles"], g["nodes"], g["idx"], g["any_rays"])
    assert np.array_equal(vis, g["visible"])


SCENES = {
    "cornell": lambda: scenes.cornell_box(seed=3),
    "soup": lambda: scenes.triangle_soup(4000, seed=5),
    "interior": lambda: scenes.interior(seed=9, target_tris=12000, n_objects=60, env_width=8, env_height=4),
    "degenerate": lambda: _degenerate(),
}


def _degenerate():
    # Many triangles sharing one centroid plus coplanar slabs: exercises the
    # "all centroids equal" leaf rule and failed splits (Geometry.h:304,395).
    d = scenes.triangle_soup(300, seed=2)
    t = d.triangles.copy()
    t["v"]["p"][:100] = t["v"]["p"][0]
    t["v"]["p"][100:200, :, 2] = 1.0
    d.triangles = t
    return d


@pytest.mark.parametrize("name", sorted(SCENES))
def test_oracle_matches_reference(oracle, reference, name):
    desc = SCENES[name]()
    n_o, i_o = oracle.bvh_build(desc.triangles)
    n_r, i_r = reference.bvh_build(desc.triangles)
    assert n_o.tobytes() == n_r.tobytes()
    assert np.array_equal(i_o, i_r)
    bmin, bmax = desc.bounds()
    rays = scenes.random_rays(bmin, bmax, 20000, seed=17)
    h_o, _, _ = oracle.trace_closest(desc.triangles, n_o, i_o, rays)
    world = reference.world(desc.triangles)
    h_r, _ = world.trace_closest(rays)
    assert h_o.tobytes() == h_r.tobytes()
    rays["tmax"] = (np.where(h_o["id"] >= 0, h_o["t"], np.float32(3.0)) * np.float32(1.01)).astype(np.float32)
    v_o, _, _ = oracle.trace_any(desc.triangles, n_o, i_o, rays)
    v_r, _ = world.trace_any(rays)
    assert np.array_equal(v_o, v_r)


def test_oracle_empty_and_tiny(oracle):
    d = scenes.triangle_soup(3, seed=1)
    nodes, idx = oracle.bvh_build(d.triangles)
    assert len(nodes) == 1 and nodes[0]["used"] == 3
    assert sorted(idx.tolist()) == [0, 1, 2]
    nodes0, _ = oracle.bvh_build(d.triangles[:0])
    assert len(nodes0) == 0


def test_oracle_multithreaded_matches_single(oracle):
    d = scenes.triangle_soup(3000, seed=8)
    nodes, idx = oracle.bvh_build(d.triangles)
    rays = scenes.random_rays(*d.bounds(), 10000, seed=3)
    h1, _, _ = oracle.trace_closest(d.triangles, nodes, idx, rays)
    h2 = oracle.trace_closest_mt(d.triangles, nodes, idx, rays, 4)
    assert h1.tobytes() == h2.tobytes()


RENDERS = sorted(GOLDEN.glob("render_*.npz"))


@pytest.mark.parametrize("path", RENDERS, ids=lambda p: p.stem)
def test_reference_reproduces_render_fixture(reference, path):
    """The harness is deterministic: re-rendering gives the fixture bits."""
    g = np.load(path)
    env = g["env"]
    cam = dict(from_=tuple(g["cam_from"]), to=tuple(g["cam_to"]), up=tuple(g["cam_up"]), fov=float(g["cam_fov"]),
               width=int(g["size"][0]), height=int(g["size"][1]))
    desc = scenes.SceneDesc(g["triangles"], g["materials"], cam, env=env if env.size else None)
    rs = reference.scene(desc)
    plain, _, _ = rs.render_pcg(False, int(g["seed"]), 0, int(g["spp"]), threads=4)
    guided, _, _ = rs.render_pcg(True, int(g["seed"]), 0, int(g["spp"]), threads=4)
    assert np.array_equal(plain, g["plain"])
    assert np.array_equal(guided, g["guided"])


def test_reference_runtest_passes(reference):
    """The reference's own inversion test (main.cpp:13-72) through the harness."""
    n = 100000
    rng = np.random.default_rng(1)
    uv = rng.random((n, 2)).astype(np.float32)
    normal = np.tile(np.array([0, 1, 0], np.float32), (n, 1))
    mat = scenes.material(kind=2, albedo=(1, 1, 1), eta=(1.0, 0.6, 1.5), k=(0.65, 0.85, 1.0), roughness=0.5)
    _, _, _, uv_out = reference.bsdf_roundtrip(mat, normal, normal, uv)
    d = np.abs(uv.astype(np.float64) - uv_out)
    d[:, 1] = np.minimum(d[:, 1], np.abs(d[:, 1] - 1.0))
    assert np.all(d < 1e-4)


def test_reference_reproduces_bsdf_fixture(reference):
    g = np.load(GOLDEN / "bsdf_roundtrip.npz")
    for case in sorted({k.split("__")[0] for k in g.files}):
        wi, f, pdf, uv_out = reference.bsdf_roundtrip(g[f"{case}__material"], g[f"{case}__n"], g[f"{case}__wo"],
                                                      g[f"{case}__uv"])
        assert np.array_equal(wi, g[f"{case}__wi"]) and np.array_equal(uv_out, g[f"{case}__uv_out"]), case


def test_metrics_match_reference(reference):
    """pathguidingdissertation_gb300.metrics against Metrics.h."""
    from pathguidingdissertation_gb300 import metrics
    rng = np.random.default_rng(4)
    gt = rng.random((24, 32, 3)).astype(np.float32)
    test = (gt + rng.normal(0, 0.05, gt.shape)).astype(np.float32)
    m, r, rr = reference.metrics(test, gt)
    assert metrics.mse(test, gt) == pytest.approx(m, rel=1e-4)
    assert metrics.rmse(test, gt) == pytest.approx(r, rel=1e-4)
    assert metrics.rrmse(test, gt) == pytest.approx(rr, rel=1e-4)
