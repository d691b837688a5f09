"""The allocation-free batch query against the allocating one.

pgx_trace_closest_noalloc serves callers that cannot let the library
allocate device memory during the call (their device memory belongs to their
own pool allocator, or a frame loop must not wait on cudaMalloc): it stages
rays and hits in a fixed file-scope device array instead.  Its hits must be
identical to pgx_trace_closest's — traversal is bit-exact, so the tolerance
is zero — on consecutive calls that share that array.

This file is collected last so a failure here leaves every other test run.
"""
from __future__ import annotations

import numpy as np
import pytest

from pathguidingdissertation_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def test_noalloc_matches_allocating_query_twice(ctx):
    desc = scenes.triangle_soup(20000, seed=41)
    ctx.upload(desc)
    ctx.bvh_build()
    bmin, bmax = desc.bounds()
    rays = scenes.random_rays(bmin, bmax, abi.NOALLOC_MAX_RAYS, seed=5)
    expected = ctx.trace_closest(rays)
    expected_counts = ctx.trace_counters()
    for _ in range(2):
        got = ctx.trace_closest_noalloc(rays)
        assert got.tobytes() == expected.tobytes()
        assert ctx.trace_counters() == expected_counts
    # A smaller batch right after: the shared array still holds the previous
    # call's rays and hits, which must not leak into this result.
    small = scenes.random_rays(bmin, bmax, 777, seed=6)
    assert ctx.trace_closest_noalloc(small).tobytes() == ctx.trace_closest(small).tobytes()


def test_noalloc_rejects_batches_over_the_limit(ctx):
    desc = scenes.triangle_soup(100, seed=2)
    ctx.upload(desc)
    ctx.bvh_build()
    rays = scenes.random_rays(*desc.bounds(), abi.NOALLOC_MAX_RAYS + 1, seed=1)
    with pytest.raises(abi.PgxError) as err:
        ctx.trace_closest_noalloc(rays)
    assert err.value.code == abi.PGX_ERR_INVALID_ARG
    assert str(abi.NOALLOC_MAX_RAYS) in str(err.value)
    assert len(ctx.trace_closest_noalloc(rays[:0])) == 0
