"""The learned guide on the GPU: tensor-core forward and backward against
the CPU restatement (oracle/mlp_oracle.py), the mixture's pdf and sampler,
and training on radiance samples."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import mlp_oracle as mo
from pathguidingdissertation_gb300 import abi

pytestmark = pytest.mark.gpu

BMIN, BMAX = np.array([-1.0, 0.0, -2.0], np.float32), np.array([3.0, 2.0, 1.0], np.float32)


def _unit(rng, n):
    v = rng.standard_normal((n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def _queries(rng, n):
    return np.concatenate([rng.uniform(BMIN, BMAX, (n, 3)).astype(np.float32), _unit(rng, n), _unit(rng, n)], 1)


def _samples(rng, n):
    s = np.zeros(n, abi.RADIANCE_SAMPLE)
    q = _queries(rng, n)
    s["position"], s["normal"], s["wo"] = q[:, 0:3], q[:, 3:6], q[:, 6:9]
    s["wi"] = _unit(rng, n)
    s["weight"] = rng.uniform(0.1, 2.0, n)
    return s


@pytest.fixture()
def net(ctx):
    ctx.mlp_init(1, BMIN, BMAX)
    params = mo.init_params(2)
    ctx.mlp_set_params(params)
    return ctx, params


def test_params_round_trip(net):
    ctx, params = net
    assert np.array_equal(ctx.mlp_params(), params)


def test_forward_matches_oracle(net):
    ctx, params = net
    rng = np.random.default_rng(3)
    q = _queries(rng, 1000)          # 7 full tiles and a partial one
    gpu = ctx.mlp_forward(q).astype(np.float64)
    cpu, _ = mo.forward(params, q, BMIN, BMAX)
    # FP32 tensor-core sums vs float64 sums: the bf16 rounding of a hidden
    # activation can land on different sides, so compare in norm
    err = np.linalg.norm(gpu - cpu) / np.linalg.norm(cpu)
    assert err < 5e-3, err
    assert np.max(np.abs(gpu - cpu)) < 0.05 * np.abs(cpu).max()


def test_gradient_matches_oracle(net):
    ctx, params = net
    rng = np.random.default_rng(4)
    s = _samples(rng, 3000)
    g_gpu, loss_gpu = ctx.mlp_gradient(s)
    loss_cpu, g_cpu = mo.loss_and_grad(params, s, BMIN, BMAX)
    assert abs(loss_gpu - loss_cpu) < 5e-3 * abs(loss_cpu)
    err = np.linalg.norm(g_gpu - g_cpu) / np.linalg.norm(g_cpu)
    assert err < 2e-2, err
    # per layer, weights and biases separately
    for (k, n), (ow, ob) in zip(mo.DIMS, mo.OFFSETS):
        for a, b in ((ow, ob), (ob, ob + n)):
            e = np.linalg.norm(g_gpu[a:b] - g_cpu[a:b]) / max(np.linalg.norm(g_cpu[a:b]), 1e-12)
            assert e < 5e-2, (a, b, e)


def _sphere_grid(n):
    c = (np.arange(n) + 0.5) / n * 2.0 - 1.0
    phi = (np.arange(n) + 0.5) / n * 2.0 * np.pi
    cc, pp = np.meshgrid(c, phi, indexing="ij")
    s = np.sqrt(1.0 - cc ** 2)
    return np.stack([s * np.cos(pp), s * np.sin(pp), cc], -1).reshape(-1, 3).astype(np.float32), 4 * np.pi / n ** 2


def test_pdf_is_normalised_and_matches_oracle(net):
    ctx, params = net
    rng = np.random.default_rng(5)
    d, da = _sphere_grid(500)
    for q in _queries(rng, 3):
        qq = np.repeat(q[None], len(d), 0)
        p = ctx.mlp_pdf(qq, d).astype(np.float64)
        assert abs(p.sum() * da - 1.0) < 5e-3
        raw = ctx.mlp_forward(q[None]).astype(np.float64)
        ref = mo.mixture_pdf(np.repeat(raw, len(d), 0), d)
        np.testing.assert_allclose(p, ref, rtol=2e-3, atol=1e-6)


def test_sample_matches_pdf_and_oracle(net):
    ctx, params = net
    rng = np.random.default_rng(6)
    n = 20000
    q = np.repeat(_queries(rng, 1), n, 0)
    u = rng.random((n, 3)).astype(np.float32)
    d, pdf = ctx.mlp_sample(q, u)
    np.testing.assert_allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-5)
    np.testing.assert_allclose(pdf, ctx.mlp_pdf(q, d), rtol=1e-5)
    raw = ctx.mlp_forward(q[:1]).astype(np.float64)
    ref = mo.sample(np.repeat(raw, n, 0), u)
    close = np.sum(d * ref, axis=1) > 1.0 - 1e-4
    assert close.mean() > 0.999     # lobe picks at cdf boundaries may differ


def test_training_learns_a_directional_field(ctx):
    """Samples whose directions follow vMF(mu(x), 20) with mu pointing from a
    light position: after training, the guide's log-likelihood of fresh
    samples is far above that of the uniform density it starts near."""
    ctx.mlp_init(7, BMIN, BMAX)
    rng = np.random.default_rng(8)
    light = np.array([1.0, 3.0, -0.5])

    def batch(n):
        s = _samples(rng, n)
        mu = light - s["position"]
        mu /= np.linalg.norm(mu, axis=1, keepdims=True)
        raw = np.zeros((n, 40))
        raw[:, 8:11] = mu
        raw[:, 11:32] = np.tile(mu, 7)
        raw[:, 32:40] = np.log(np.expm1(20.0))
        s["wi"] = mo.sample(raw, rng.random((n, 3)))
        s["weight"] = 1.0
        return s

    test = batch(20000)
    q = np.concatenate([test["position"], test["normal"], test["wo"]], 1)
    ll0 = np.mean(np.log(ctx.mlp_pdf(q, test["wi"])))
    losses = [ctx.mlp_train_step(batch(1 << 14), lr=1e-2) for _ in range(300)]
    ll1 = np.mean(np.log(ctx.mlp_pdf(q, test["wi"])))
    assert np.all(np.isfinite(losses))
    assert losses[-1] < losses[0] - 1.0
    # uniform: log(1/4pi) = -2.53; the target's own mean log-density is
    # log(20 / 2pi) - 20 (1 - coth 20 + 1/20) = +0.16
    assert ll0 < -1.5 and ll1 > -1.0, (ll0, ll1)


def test_api_errors(ctx, pgx_lib):
    from pathguidingdissertation_gb300.abi import PgxError
    with pytest.raises(PgxError):
        ctx.mlp_forward(np.zeros((4, 9), np.float32))      # not initialised
    ctx.mlp_init(1, BMIN, BMAX)
    assert ctx.mlp_forward(np.zeros((0, 9), np.float32)).shape == (0, 40)
    with pytest.raises(PgxError):
        ctx.mlp_init(1, BMIN, BMIN)                        # empty bounds
    with pytest.raises(PgxError):
        ctx.mlp_configure(lr=-1.0)


# ---- the learned guide inside the renderer ---------------------------------------------
from pathguidingdissertation_gb300 import scenes  # noqa: E402


def _tile_z(a, a2, b, b2, spp, t=8):
    H, W = a.shape[:2]

    def tiles(x):
        return x[: H // t * t, : W // t * t].reshape(H // t, t, W // t, t, 3).sum(axis=(1, 3))

    n = spp * t * t
    ma, mb = tiles(a) / n, tiles(b) / n
    va = np.maximum(tiles(a2) / n - ma * ma, 0) / n
    vb = np.maximum(tiles(b2) / n - mb * mb, 0) / n
    z = np.abs(ma - mb) / np.sqrt(va + vb + 1e-12)
    z_total = abs(ma.sum() - mb.sum()) / np.sqrt(va.sum() + vb.sum())
    return z, z_total


@pytest.mark.parametrize("scene,trained", [("cornell", False), ("cornell", True), ("interior", True)])
def test_mlp_guided_estimator_unbiased(ctx, scene, trained):
    if scene == "cornell":
        desc = scenes.cornell_box(seed=1, width=48, height=48)
    else:
        desc = scenes.interior(seed=3, target_tris=20000, n_objects=40, width=48, height=27, env_width=256,
                               env_height=128)
    ctx.upload(desc)
    ctx.bvh_build()
    ctx.mlp_init(3)
    if trained:
        ctx.mlp_configure(lr=1e-2, decay=0.99, batch=1 << 14)
        ctx.render(32, mode=abi.MODE_GUIDED_MLP, seed=99, max_depth=8, train_guide=True)
        ctx.clear()
    spp = 1024
    ctx.render(spp, mode=abi.MODE_PLAIN, seed=5, max_depth=8)
    a, a2, _ = ctx.film(squares=True)
    ctx.clear()
    ctx.render(spp, mode=abi.MODE_GUIDED_MLP, seed=6, max_depth=8, guide_fraction=0.5)
    b, b2, _ = ctx.film(squares=True)
    z, z_total = _tile_z(a, a2, b, b2, spp)
    assert np.mean(z < 4.0) > 0.97, np.sort(z.ravel())[-5:]
    assert z_total < 4.0, z_total


def test_online_training_updates_the_guide(ctx):
    desc = scenes.cornell_box(seed=2, width=64, height=64)
    ctx.upload(desc)
    ctx.bvh_build()
    ctx.mlp_init(5)
    p0 = ctx.mlp_params()
    ctx.mlp_configure(lr=5e-3, decay=0.999, batch=1 << 15)
    ctx.render(8, mode=abi.MODE_GUIDED_MLP, seed=1, max_depth=8, train_guide=True)
    p1 = ctx.mlp_params()
    assert np.all(np.isfinite(p1)) and not np.array_equal(p0, p1)
    rgb, _, spp = ctx.film()
    assert spp == 8 and np.all(np.isfinite(rgb)) and rgb.mean() > 0
    # training needs the learned-guide mode
    from pathguidingdissertation_gb300.abi import PgxError
    with pytest.raises(PgxError):
        ctx.render(1, mode=abi.MODE_PLAIN, train_guide=True)


def test_trained_guide_lowers_the_error(ctx):
    """What the trained network gains: on the small interior (320 x 180, the
    sky-and-sun environment seen through the window), at equal spp, the
    image rendered with the online-trained learned guide has a lower relMSE
    against a 4,096-spp plain render than (a) plain path tracing, (b) the
    same estimator with the untrained network, by the stated margins, and
    stays within 40 % of (c) the QuadTree guide trained on as many samples
    (the yardstick).  Measured: plain 0.196, untrained 0.546, QuadTree
    0.118-0.120, learned 0.110-0.130 over runs (the gradient sums use float
    atomics, so the trained network differs in its last bits from run to
    run).  relMSE = mean((x - r)^2 / (r^2 + 0.01)) over pixels, without the
    0.1 % largest per-pixel errors (sun fireflies)."""
    from pathguidingdissertation_gb300.metrics import relmse_robust
    desc = scenes.interior(seed=2, target_tris=40000, n_objects=80, width=320, height=180, env_width=512,
                           env_height=256)
    ctx.upload(desc)
    ctx.bvh_build()
    depth, spp, train = 10, 64, 64

    def image(mode, seed, **kw):
        ctx.clear()
        ctx.render(spp, mode=mode, seed=seed, max_depth=depth, **kw)
        rgb, _, n = ctx.film()
        return rgb.astype(np.float64) / n

    ctx.clear()
    ctx.render(4096, mode=abi.MODE_PLAIN, seed=1000, max_depth=depth)
    ref_rgb, _, n = ctx.film()
    ref = ref_rgb.astype(np.float64) / n
    e_plain = relmse_robust(image(abi.MODE_PLAIN, 7), ref)

    ctx.mlp_init(3)
    e_untrained = relmse_robust(image(abi.MODE_GUIDED_MLP, 7, guide_fraction=0.75), ref)
    ctx.mlp_configure(lr=5e-3, decay=0.998, batch=1 << 16, steps=2)
    ctx.clear()
    ctx.render(train, mode=abi.MODE_GUIDED_MLP, seed=11, max_depth=depth, train_guide=True, guide_fraction=0.75)
    e_learned = relmse_robust(image(abi.MODE_GUIDED_MLP, 7, guide_fraction=0.75), ref)

    for it in range(6):  # cache iterations of 1, 2, ..., 32 frames (the first unguided)
        ctx.clear()
        m = abi.MODE_PLAIN if it == 0 else abi.MODE_GUIDED_QUADTREE
        ctx.render(1 << it, mode=m, seed=21 + it, max_depth=depth, record_paths=1 << it, guide_fraction=0.5)
    e_quadtree = relmse_robust(image(abi.MODE_GUIDED_QUADTREE, 7, guide_fraction=0.5), ref)

    summary = dict(plain=e_plain, untrained=e_untrained, learned=e_learned, quadtree=e_quadtree)
    assert e_learned < 0.85 * e_plain, summary
    assert e_learned < 0.8 * e_untrained, summary
    assert e_learned < 1.4 * e_quadtree, summary


def test_quadtree_fallback_for_untrained_regions(ctx):
    """The QuadTree guide stands in for the learned guide in radiance-cache
    regions where the network has seen fewer than pgx_mlp_set_fallback's
    count of training samples.  With an untrained network every guided
    vertex falls back, and the image equals the QuadTree mode's (same
    random numbers, same estimator); after online training the network
    takes over most vertices; with the fallback off it takes all."""
    desc = scenes.interior(seed=3, target_tris=20000, n_objects=40, width=64, height=36, env_width=256,
                           env_height=128)
    ctx.upload(desc)
    ctx.bvh_build()
    ctx.clear()
    ctx.render(2, mode=abi.MODE_PLAIN, seed=1, max_depth=8, record_paths=2)  # the radiance cache
    ctx.clear()
    ctx.render(4, mode=abi.MODE_GUIDED_QUADTREE, seed=7, max_depth=8, guide_fraction=0.5)
    q, _, _ = ctx.film()
    ctx.mlp_init(3)
    ctx.clear()
    ctx.render(4, mode=abi.MODE_GUIDED_MLP, seed=7, max_depth=8, guide_fraction=0.5)
    untrained = ctx.render_stats().guide_fallbacks
    m, _, _ = ctx.film()
    assert untrained > 0
    rel = np.abs(m.astype(np.float64) - q) / np.maximum(np.abs(q.astype(np.float64)), 1e-3)
    assert rel.max() < 1e-4, rel.max()

    ctx.mlp_configure(lr=5e-3, decay=0.998, batch=1 << 14, steps=4)
    ctx.clear()
    ctx.render(24, mode=abi.MODE_GUIDED_MLP, seed=11, max_depth=8, train_guide=True)
    ctx.clear()
    ctx.render(4, mode=abi.MODE_GUIDED_MLP, seed=7, max_depth=8, guide_fraction=0.5)
    trained = ctx.render_stats().guide_fallbacks
    assert trained < 0.5 * untrained, (trained, untrained)
    ctx.mlp_set_fallback(0)
    ctx.clear()
    ctx.render(4, mode=abi.MODE_GUIDED_MLP, seed=7, max_depth=8, guide_fraction=0.5)
    assert ctx.render_stats().guide_fallbacks == 0
    with pytest.raises(abi.PgxError):
        ctx.mlp_set_fallback(-1)
