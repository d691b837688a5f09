"""Differentiable rendering on the GPU (pgx_diff_*): the detached primal
against the wavefront renderer, adjoint gradients against central finite
differences of the same primal, and against finite differences of the
reference's own CPU renderer."""
from __future__ import annotations

import numpy as np
import pytest

from pathguidingdissertation_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def _small_terrain(**kw):
    a = dict(grid=64, seed=4, width=40, height=32, env_width=64, env_height=32, sun_peak=20.0)
    a.update(kw)
    return scenes.terrain(**a)


def _setup(ctx, desc):
    ctx.upload(desc)
    ctx.bvh_build()
    ctx.clear()


def test_primal_matches_wavefront_renderer(ctx):
    desc = _small_terrain()
    _setup(ctx, desc)
    spp = 16
    img = ctx.diff_render(spp, seed=5, max_depth=8)
    ctx.render(spp, mode=abi.MODE_PLAIN, seed=5, max_depth=8)
    rgb, _, n = ctx.film()
    ref = rgb.astype(np.float64) / n
    # same seeds, same decisions: only the float32 atomics of the film differ
    rel = np.abs(img - ref) / np.maximum(np.abs(ref), 1e-3)
    assert np.max(rel) < 1e-4, np.max(rel)
    assert np.array_equal(ctx.diff_render(spp, seed=5, max_depth=8), img)   # deterministic


def _loss(img, target):
    d = img - target
    return float(np.sum(d * d))


def test_adjoint_matches_finite_differences(ctx):
    desc = _small_terrain()
    _setup(ctx, desc)
    nm = len(desc.materials)
    rng = np.random.default_rng(1)
    spp, seed, depth = 32, 11, 6
    # target: the scene with perturbed albedos, roughness and environment
    rough0 = desc.materials["roughness"].astype(np.float32)
    env0 = desc.env.astype(np.float32)
    ctx.diff_set_params(env=env0 * np.exp(rng.normal(0, 0.05, env0.shape)).astype(np.float32),
                        albedo_offset=rng.normal(0, 0.05, (nm, 3)).astype(np.float32),
                        roughness=np.clip(rough0 + rng.normal(0, 0.05, nm), 0.02, 1.0).astype(np.float32))
    target = ctx.diff_render(64, seed=99, max_depth=depth)
    ctx.diff_set_params()
    img = ctx.diff_render(spp, seed, depth)
    dimg = (2.0 * (img - target)).astype(np.float32)
    g_env, g_alb, g_rough = ctx.diff_adjoint(dimg, spp, seed, depth)

    h = 1e-3
    checks = []

    def fd(env=None, alb=None, rough=None):
        ctx.diff_set_params(env=env, albedo_offset=alb, roughness=rough)
        return _loss(ctx.diff_render(spp, seed, depth), target)

    used = np.unique(desc.triangles["material"])
    for m in rng.choice(used, 6, replace=False):
        c = int(rng.integers(3))
        a = np.zeros((nm, 3), np.float32)
        a[m, c] = h
        checks.append(("albedo", (fd(alb=a) - fd(alb=-a)) / (2 * h), g_alb[m, c]))
        r = rough0.copy()
        r[m] += h
        rm = rough0.copy()
        rm[m] -= h
        checks.append(("roughness", (fd(rough=r) - fd(rough=rm)) / (2 * h), g_rough[m]))
    flat = np.abs(g_env).ravel()
    for idx in list(np.argsort(flat)[-6:]) + list(rng.choice(np.flatnonzero(flat > 0), 4, replace=False)):
        e = env0.copy().ravel()
        e[idx] += h
        em = env0.copy().ravel()
        em[idx] -= h
        checks.append(("env", (fd(env=e.reshape(env0.shape)) - fd(env=em.reshape(env0.shape))) / (2 * h),
                       g_env.ravel()[idx]))
    ctx.diff_set_params()
    scale = max(abs(c[1]) for c in checks)
    for name, g_fd, g_adj in checks:
        assert abs(g_adj - g_fd) <= 1e-3 * abs(g_fd) + 1e-5 * scale, (name, g_fd, g_adj)


def test_adjoint_matches_reference_renderer_differences(ctx, reference):
    """d(mean luminance)/d(albedo of one wall) of the Cornell box: the adjoint
    on the GPU against central differences of the reference's own CPU path
    tracer (pathTrace driven by the same PCG streams, so both renders of a
    difference share their random numbers)."""
    desc = scenes.cornell_box(seed=1, width=24, height=24)
    _setup(ctx, desc)
    npix = 24 * 24
    w = np.array([0.2126, 0.7152, 0.0722], np.float32)
    dimg = np.tile(w / npix, (24, 24, 1)).astype(np.float32)
    spp = 4096
    _, g_alb, _ = ctx.diff_adjoint(dimg, spp, seed=3, max_depth=8)
    mat = int(desc.triangles["material"][8])   # a side wall
    h = 0.05
    vals = []
    for sgn in (1.0, -1.0):
        d = scenes.SceneDesc(desc.triangles, desc.materials.copy(), desc.camera)
        d.materials["albedo"][mat] = d.materials["albedo"][mat] + sgn * h
        rs = reference.scene(d, threads=16)
        film, _, _ = rs.render_pcg(False, 21, 0, 1024, threads=16)
        rs.close()
        vals.append(float((film.astype(np.float64) / 1024 * w).sum(axis=2).mean()))
    g_ref = (vals[0] - vals[1]) / (2 * h)
    g_gpu = float(g_alb[mat].sum())   # the same offset on all three channels
    assert g_ref > 0 and abs(g_gpu - g_ref) < 0.06 * abs(g_ref), (g_gpu, g_ref)


def test_diff_api_errors(ctx):
    from pathguidingdissertation_gb300.abi import PgxError
    desc = _small_terrain()
    _setup(ctx, desc)
    with pytest.raises(PgxError):
        ctx.diff_render(0)
    with pytest.raises(PgxError):
        ctx.diff_set_params(roughness=-np.ones(len(desc.materials), np.float32))
