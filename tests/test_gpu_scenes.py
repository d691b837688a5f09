"""The reference's own scenes rendered on the GPU against the reference.

Each complete scene of the reference (every mesh present) is read with
pgx's loader (the reader of SceneLoader.h:104-269's format), its albedo
textures replaced by the texels the reference's own Texture::load decodes
(Imaging.h:44-79, stb_image), so the GPU's bilinear texture fetch
(Texture::sample, Imaging.h:82-108) is compared on identical texels.  The
film is reduced to 96 pixels wide at the scene's aspect ratio, the
reference's own BVH is installed (identical traversal order), and pgx's
wavefront integrators are compared per pixel with the reference's
pathTrace / guidedPath driven by the same PCG32 streams."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import build as ob
from pathguidingdissertation_gb300 import abi, loader

pytestmark = pytest.mark.gpu

SCENES = ob.COMPLETE_SCENES


def _reduced(desc, width=96):
    w, h = desc.camera["width"], desc.camera["height"]
    desc.camera = dict(desc.camera, width=width, height=max(8, int(round(width * h / w))))
    return desc


def _with_reference_texels(desc, ref_export):
    assert len(desc.textures) == len(ref_export["textures"])
    texs = []
    for mine, theirs in zip(desc.textures, ref_export["textures"]):
        assert mine.shape == theirs.shape
        texs.append(np.ascontiguousarray(theirs, np.float32))
    desc.textures = texs
    if ref_export["env"] is not None:
        assert np.array_equal(desc.env, ref_export["env"])
    return desc


def _compare(gpu, ref, tol=1e-3, max_bad=0.02, sum_tol=0.01):
    g = gpu.reshape(-1, 3).astype(np.float64)
    r = ref.reshape(-1, 3).astype(np.float64)
    err = np.abs(g - r).max(axis=1) / np.maximum(np.abs(r).max(axis=1), 1e-3)
    bad = float(np.mean(err > tol))
    assert bad <= max_bad, f"{bad:.4f} of pixels differ by more than {tol}"
    rel = abs(g.sum() - r.sum()) / max(abs(r.sum()), 1e-9)
    assert rel < sum_tol, f"image sums differ by {rel:.4f}"
    return bad


@pytest.fixture(scope="module")
def loaded(reference):
    cache = {}

    def get(name):
        if name not in cache:
            d = ob.scenes_dir() / name
            if not (d / "scene.json").exists():
                pytest.skip(f"reference scene {name} not staged")
            desc = loader.load_scene(d)
            desc = _with_reference_texels(desc, reference.load_scene(str(d)))
            nodes, idx = reference.bvh_build(desc.triangles)
            cache[name] = (_reduced(desc), nodes, idx)
        return cache[name]
    return get


@pytest.mark.parametrize("mode", [abi.MODE_PLAIN, abi.MODE_GUIDED_LI], ids=["plain", "guided_li"])
@pytest.mark.parametrize("name", SCENES)
def test_reference_scene_per_pixel(ctx, reference, loaded, name, mode):
    desc, nodes, idx = loaded(name)
    spp = 4
    ctx.upload(desc)
    ctx.bvh_import(nodes, idx)
    ctx.clear()
    ctx.render(spp, mode=mode, seed=17, max_depth=8)
    film, _, got = ctx.film()
    assert got == spp
    rs = reference.scene(desc)
    ref_film, _, _ = rs.render_pcg(mode == abi.MODE_GUIDED_LI, 17, 0, spp, threads=8)
    rs.close()
    assert np.isfinite(film).all()
    assert ref_film.sum() > 0
    _compare(film, ref_film)


def test_textured_scene_uses_textures(ctx, reference, loaded):
    """The textured dining room: a render with every albedo texture replaced
    by its mean colour differs from the textured render in most lit pixels
    (the texture fetch is live; the per-pixel match with the reference is
    test_reference_scene_per_pixel)."""
    desc, nodes, idx = loaded("dining-room")
    big = [t for t in desc.textures if t.shape[0] * t.shape[1] > 1]
    assert big, "the dining room has image textures"
    ctx.upload(desc)
    ctx.bvh_import(nodes, idx)
    ctx.clear()
    ctx.render(4, mode=abi.MODE_PLAIN, seed=23, max_depth=8)
    textured, _, _ = ctx.film()
    flat = type(desc)(desc.triangles, desc.materials, desc.camera, env=desc.env,
                      textures=[np.broadcast_to(t.reshape(-1, 3).mean(0), (1, 1, 3)).astype(np.float32).copy()
                                for t in desc.textures], name=desc.name)
    ctx.upload(flat)
    ctx.bvh_import(nodes, idx)
    ctx.clear()
    ctx.render(4, mode=abi.MODE_PLAIN, seed=23, max_depth=8)
    untextured, _, _ = ctx.film()
    d = np.abs(textured - untextured).max(axis=-1)
    s = np.maximum(np.abs(textured), np.abs(untextured)).max(axis=-1)
    lit = s > 0
    assert np.mean(d[lit] > 1e-3 * s[lit]) > 0.15
