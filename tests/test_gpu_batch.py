"""Batched rendering (pgx_batch_*): many scenes in one persistent,
graph-captured launch give the same images as rendering each scene alone."""
from __future__ import annotations

import numpy as np
import pytest

from pathguidingdissertation_gb300 import abi, scenes
from pathguidingdissertation_gb300.api import Batch, Context

pytestmark = pytest.mark.gpu

SPECS = [dict(seed=1, width=32, height=24, target_tris=None), dict(seed=2, width=48, height=48, target_tris=3000),
         dict(seed=3, width=16, height=40, target_tris=20000), dict(seed=4, width=64, height=32, target_tris=800)]


def _ctx(spec):
    c = Context(0)
    c.upload(scenes.cornell_box(**spec))
    c.bvh_build()
    c.clear()
    return c


def _close(a, b):
    rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-3)
    return float(np.max(rel))


def test_batch_equals_single_scene_renders(pgx_lib):
    batch_ctx = [_ctx(s) for s in SPECS]
    solo = [_ctx(s) for s in SPECS]
    b = Batch(batch_ctx)
    b.render(8, seed=5, max_depth=8)
    st = b.stats()
    assert st.paths == sum(s["width"] * s["height"] * 8 for s in SPECS) and st.graph_replayed == 0
    b.render(8, seed=5, max_depth=8)          # same launch shape: the graph is replayed
    assert b.stats().graph_replayed == 1
    for bc, sc in zip(batch_ctx, solo):
        sc.render(16, mode=abi.MODE_PLAIN, seed=5, max_depth=8)
        a, _, na = bc.film()
        r, _, nr = sc.film()
        assert na == nr == 16
        # same seeds and decisions; only the order of the film's float atomics differs
        assert _close(a.astype(np.float64), r.astype(np.float64)) < 1e-4
    b.close()
    for c in batch_ctx + solo:
        c.close()


def test_autotune_keeps_films_and_tuning_applies(pgx_lib):
    ctxs = [_ctx(s) for s in SPECS]
    b = Batch(ctxs)
    t = b.autotune(spp=1, max_depth=8)
    assert t.wave_paths >= 1 << 20 and 1 <= t.trace_blocks_per_sm <= 8 and t.shade_blocks_per_sm >= 1
    assert t.stack_shared in (4, 8, 16)
    for c in ctxs:
        rgb, _, n = c.film()
        assert n == 0 and not rgb.any()
    b.set_tuning(1 << 16, 4, 8)       # many small waves
    b.render(2, seed=9)
    with pytest.raises(abi.PgxError):
        b.set_tuning(1 << 16, 100, 8)
    with pytest.raises(abi.PgxError):
        b.set_tuning(1 << 20, 8, 16, stack_shared=5)
    # the stack's shared-memory depth changes where entries live, not the
    # traversal: the same images
    films = []
    for sh in (4, 8, 16):
        for c in ctxs:
            c.clear()
        b.set_tuning(1 << 20, 8, 16, stack_shared=sh)
        b.render(2, seed=9)
        films.append([c.film()[0].astype(np.float64) for c in ctxs])
    for other in films[1:]:
        for a, r in zip(other, films[0]):
            assert _close(a, r) < 1e-5
    b.close()
    for c in ctxs:
        c.close()


def test_batch_with_environment_scenes_equals_single_renders(pgx_lib):
    """Scenes lit by environment maps (each read from its own context) batched
    with area-lit ones: the same images as rendering each scene alone."""
    def interior(seed, w, h, ew, eh):
        c = Context(0)
        c.upload(scenes.interior(seed=seed, target_tris=3000, n_objects=10, width=w, height=h, env_width=ew,
                                 env_height=eh))
        c.bvh_build()
        c.clear()
        return c

    def make():
        return [interior(3, 24, 16, 64, 32), _ctx(SPECS[1]), interior(5, 16, 20, 32, 16)]

    batch_ctx, solo = make(), make()
    b = Batch(batch_ctx)
    b.render(8, seed=7, max_depth=8)
    for bc, sc in zip(batch_ctx, solo):
        sc.render(8, mode=abi.MODE_PLAIN, seed=7, max_depth=8)
        a, _, na = bc.film()
        r, _, nr = sc.film()
        assert na == nr == 8 and r.any()
        assert _close(a.astype(np.float64), r.astype(np.float64)) < 1e-4
    b.close()
    for c in batch_ctx + solo:
        c.close()
