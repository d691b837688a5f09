"""Scene ingestion: the host reader of the reference's scene format
(scene.json + .gem + textures) against the reference's own loadScene
(SceneLoader.h:104-269) and Texture::load (Imaging.h:44-79), compiled
headless; plus the writer's round trip.  CPU only."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from pathguidingdissertation_gb300 import loader, scenes
from pathguidingdissertation_gb300.abi import BSDF_CONDUCTOR, BSDF_DIFFUSE, BSDF_GLASS, BSDF_PLASTIC

from oracle import build as _oracle_build

# The checkout's scene folder (every scene, for the image-format tests).
REF_SCENES = _oracle_build.reference_root() / "Scenes"
# The reference scenes whose meshes are all present and whose textures are
# PNG or HDR (the others lack mesh files, on which loadScene exits).
COMPLETE = ["cornell-box", "veach-mis", "veach-bidir", "MaterialsScene"]
# Complete reference scenes with JPEG albedo maps: pgx decodes JPEG itself
# (pgx_image_decode_jpeg), in floating point where stb_image uses fixed
# point, so those texels may differ from the reference's by a few levels.
COMPLETE_JPEG = ["dining-room", "living-room", "staircase2"]


def _assert_jpeg_close(a, b, what=""):
    """Texels within 3/255 of stb_image's, 95 % equal, 99 % within 1/255."""
    assert a.shape == b.shape, what
    d = np.rint(np.abs(a.astype(np.float64) - b.astype(np.float64)) * 255.0)
    assert d.max() <= 3, (what, d.max())
    assert np.mean(d == 0) >= 0.95, (what, np.mean(d == 0))
    assert np.mean(d <= 1) >= 0.99, (what, np.mean(d <= 1))


def _assert_same(mine_desc, ref_export, reference, jpeg=False):
    m = reference.loaded_from_desc(mine_desc)
    r = ref_export
    assert len(m["triangles"]) == len(r["triangles"])
    assert m["triangles"].tobytes() == r["triangles"].tobytes()
    # columns 16..19 are the coating's sigmaA and thickness, which LayeredBSDF
    # stores but never reads (Materials.h:855-897); pgx keeps only the flag
    assert np.array_equal(m["materials"][:, :16], r["materials"][:, :16])
    assert np.array_equal(m["projection"], r["projection"])
    assert np.array_equal(m["camera"], r["camera"])
    assert (m["width"], m["height"]) == (r["width"], r["height"])
    assert len(m["textures"]) == len(r["textures"])
    for i, (a, b) in enumerate(zip(m["textures"], r["textures"])):
        assert a.shape == b.shape
        if not (jpeg and not np.array_equal(a, b)):
            assert np.array_equal(a, b), i
        else:
            _assert_jpeg_close(a, b, f"texture {i}")
    assert (m["env"] is None) == (r["env"] is None)
    if r["env"] is not None:
        assert np.array_equal(m["env"], r["env"])


@pytest.mark.parametrize("name", COMPLETE)
def test_load_reference_scene(reference, name):
    d = REF_SCENES / name
    if not d.is_dir():
        pytest.skip("reference scenes not available")
    _assert_same(loader.load_scene(d), reference.load_scene(str(d)), reference)


@pytest.mark.parametrize("name", COMPLETE_JPEG)
def test_load_reference_scene_with_jpeg(reference, name):
    d = REF_SCENES / name
    if not d.is_dir():
        pytest.skip("reference scenes not available")
    _assert_same(loader.load_scene(d), reference.load_scene(str(d)), reference, jpeg=True)


def test_jpeg_textures_match_stb(reference):
    """Every JPEG of the reference's scenes (baseline 4:4:4 and 4:2:0,
    progressive) against Texture::load through the reference's stb_image."""
    files = sorted(REF_SCENES.glob("*/*.jpg"))
    if not files:
        pytest.skip("reference scenes not available")
    for f in files:
        _assert_jpeg_close(loader.load_texture(str(f)), reference.load_texture(str(f)), f.name)


def test_jpeg_rejects_bad_data(tmp_path):
    bad = tmp_path / "bad.jpg"
    bad.write_bytes(b"\xff\xd8\xff\xdb\x00\x02garbage")
    with pytest.raises(ValueError):
        loader.read_jpeg(bad)
    # Texture::load falls back to the 1x1 white texture when stbi_load fails
    w = loader.load_texture(str(bad))
    assert w.shape == (1, 1, 3) and np.all(w == 1.0)
    (tmp_path / "not.jpg").write_bytes(b"PNG\x00\x01")
    with pytest.raises(ValueError):
        loader.read_jpeg(tmp_path / "not.jpg")


def test_jpeg_truncated_files_do_not_crash(tmp_path):
    """Cut-off entropy-coded data decodes with zeros fed after the end (or is
    rejected); never out of bounds."""
    files = sorted(REF_SCENES.glob("staircase2/*.jpg"))[:2]
    if not files:
        pytest.skip("reference scenes not available")
    for f in files:
        data = f.read_bytes()
        for frac in (0.02, 0.3, 0.7, 0.99):
            cut = tmp_path / f"cut_{frac}.jpg"
            cut.write_bytes(data[:int(len(data) * frac)])
            try:
                img, ch = loader.read_jpeg(cut)
                assert img.ndim == 3 and ch in (1, 3)
            except ValueError:
                pass


def test_texture_formats_match_stb(reference):
    files = sorted(REF_SCENES.glob("*/*.hdr"))[:3] + sorted(REF_SCENES.glob("*/*.bmp")) + \
        sorted(REF_SCENES.glob("*/*.tga")) + sorted(REF_SCENES.glob("living-room/leaf.png"))
    if not files:
        pytest.skip("reference scenes not available")
    for f in files:
        a = reference.load_texture(str(f))
        b = loader.load_texture(str(f))
        assert a.shape == b.shape and np.array_equal(a, b), f.name


def _gem_quad(offset=(0.0, 0.0, 0.0)):
    v = np.zeros((4, 11), np.float32)
    v[:, 0:3] = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32) + np.float32(offset)
    v[:, 5] = 1.0
    v[:, 9:11] = [[0, 0], [1, 0], [1, 1], [0, 1]]
    return v


def _write_png(path, rgb8):
    from pathguidingdissertation_gb300.api import write_png
    write_png(str(path), np.asarray(rgb8, np.uint8))


def js_world():
    return [1.5, 0.2, 0.0, 0.1, 0.0, 0.75, 0.3, -0.2, 0.1, 0.0, 2.0, 0.5, 0.0, 0.0, 0.0, 1.0]


def _edge_scene(root: Path) -> Path:
    """A scene exercising the loader's corner rules."""
    d = root / "edge"
    d.mkdir()
    # Mesh with two parts: the reference offsets the second part's indices by
    # the number of indices read so far (SceneLoader.h:209-212), not vertices.
    a = _gem_quad()
    b = _gem_quad((2.0, 0.0, 0.0))[:3]
    loader.write_gem(d / "two.gem", [(a, np.array([0, 1, 2], np.uint32)), (b, np.array([0, 1, 2], np.uint32))])
    quad = _gem_quad()
    # A degenerate (zero-area) triangle after a valid one: dropped.
    deg = quad.copy()
    deg[2, 0:3] = deg[1, 0:3]
    loader.write_gem(d / "quad.gem", [(quad, np.array([0, 1, 2, 0, 2, 3], np.uint32))])
    loader.write_gem(d / "deg.gem", [(deg, np.array([0, 1, 2, 0, 2, 3], np.uint32))])
    _write_png(d / "red.png", [[[200, 10, 10], [10, 200, 10]], [[10, 10, 200], [255, 255, 255]]])
    _write_png(d / "grey.png", [[[128, 128, 128]]])
    world = js_world()
    ident = [1.0, 0, 0, 0, 0, 1.0, 0, 0, 0, 0, 1.0, 0, 0, 0, 0, 1.0]
    js = {
        "width": 96, "height": "64.7", "fov": "33.3333", "flipX": "1",
        "from": "0.1 0.2  3.0", "to": "0 0.5 0 ", "up": "0 1",
        "zzz": [{"filename": "quad.gem", "world": ident, "bsdf": "diffuse", "reflectance": "grey.png"}],
        "instances": [
            {"filename": "two.gem", "world": world, "bsdf": "diffuse", "reflectance": "red.png",
             "emission": "1.5 2 2.5"},
            {"filename": "quad.gem", "world": world, "bsdf": "conductor", "reflectance": "red.png",
             "eta": "0.2 0.9", "k": "3.1 2.9 2.5x", "roughness": 0.25},
            {"filename": "quad.gem", "world": ident, "bsdf": "dielectric", "reflectance": "missing.png",
             "intIOR": "1.5", "roughness": "0.0005"},
            {"filename": "quad.gem", "world": ident, "bsdf": "dielectric", "reflectance": "grey.png",
             "intIOR": "1.45", "extIOR": "1.01", "roughness": "0.3"},
            {"filename": "quad.gem", "world": ident, "bsdf": "velvet", "reflectance": "grey.png"},
            {"filename": "deg.gem", "world": ident, "bsdf": "plastic", "reflectance": "grey.png",
             "roughness": "0.1", "coatingThickness": "0.5", "emission": "3 3 3"},
            {"filename": "quad.gem", "world": ident, "bsdf": "plastic", "reflectance": "grey.png",
             "roughness": "0.1", "coatingThickness": "2", "coatingSigmaA": "0.5 0.5 0.5", "emission": "3 3 3"},
            {"filename": "quad.gem", "world": ident, "bsdf": "orennayar", "alpha": "0.35"},
            {"filename": "quad.gem", "world": ident, "bsdf": "mirror", "reflectance": "grey.png"},
            {"filename": "quad.gem", "world": ident, "bsdf": "glass", "reflectance": "red.png"},
        ],
    }
    (d / "scene.json").write_text(json.dumps(js))
    return d


def test_loader_corner_rules_match_reference(reference, tmp_path):
    d = _edge_scene(tmp_path)
    mine = loader.load_scene(d)
    ref = reference.load_scene(str(d))
    _assert_same(mine, ref, reference)
    # the rules themselves, as the reference applies them
    kinds = list(mine.materials["kind"])
    assert len(mine.materials) == 10            # "velvet" is skipped
    assert kinds[2] == BSDF_GLASS               # dielectric, roughness < 0.001
    assert mine.materials["layered"].tolist() == [0, 0, 0, 0, 0, 1, 0, 0, 0, 0]  # stoi("0.5") == 0
    assert float(mine.materials["emission"][5].max()) == 0.0   # the coating drops the emission
    assert mine.camera["height"] == 64 and mine.camera["flip_x"] == 1
    assert mine.camera["up"] == (0.0, 1.0, 0.0)
    assert kinds[0] == BSDF_DIFFUSE and kinds[1] == BSDF_CONDUCTOR and kinds[4] == BSDF_PLASTIC
    # the index-offset rule: the second part's triangle starts at vertex 3 of
    # the first part (offset 3 = indices read), not at its own vertex 0
    two = mine.triangles[mine.triangles["material"] == 0]
    assert len(two) == 2
    first = loader._mul_point(np.array(js_world(), np.float32), _gem_quad()[3:4, 0:3])[0]
    assert np.array_equal(two["v"]["p"][1, 0], first)
    # missing texture -> 1x1 white default
    assert any(t.shape == (1, 1, 3) and np.all(t == 1.0) for t in mine.textures)


def test_write_scene_round_trip(reference, tmp_path):
    desc = scenes.cornell_box(seed=4, width=64, height=48)
    d = loader.write_scene(desc, tmp_path / "box")
    mine = loader.load_scene(d)
    _assert_same(mine, reference.load_scene(str(d)), reference)
    # geometry is written exactly; constant albedos become 8-bit 1x1 textures
    order = np.argsort(mine.triangles["material"], kind="stable")
    src = desc.triangles[np.argsort(desc.triangles["material"], kind="stable")]
    assert np.array_equal(mine.triangles["v"]["p"][order], src["v"]["p"])
    albedo = np.array([mine.textures[int(m["albedo_texture"])][0, 0] for m in mine.materials])
    assert np.max(np.abs(albedo - desc.materials["albedo"])) <= 0.5 / 255 + 1e-7
    assert np.array_equal(mine.materials["emission"], desc.materials["emission"])


def test_write_scene_with_environment(reference, tmp_path):
    desc = scenes.interior(seed=2, target_tris=3000, n_objects=12, env_width=32, env_height=16, width=40,
                           height=30)
    d = loader.write_scene(desc, tmp_path / "room")
    mine = loader.load_scene(d)
    assert mine.env is not None and mine.env.shape == (16, 32, 3)
    # RGBE keeps 8 mantissa bits of the largest channel, truncated
    err = np.abs(mine.env - desc.env)
    assert np.all(err <= desc.env.max(axis=2, keepdims=True) / 128 + 1e-30)
    _assert_same(mine, reference.load_scene(str(d)), reference)


def test_gem_round_trip(tmp_path):
    v = np.random.default_rng(1).standard_normal((7, 11)).astype(np.float32)
    idx = np.array([0, 1, 2, 4, 5, 6], np.uint32)
    loader.write_gem(tmp_path / "m.gem", [(v, idx), (v[:3], idx[:3])])
    meshes = loader.read_gem(tmp_path / "m.gem")
    assert len(meshes) == 2
    assert np.array_equal(meshes[0][1], v) and np.array_equal(meshes[0][2], idx)
    assert np.array_equal(meshes[1][1], v[:3])
    (tmp_path / "bad.gem").write_bytes(b"\0" * 16)
    with pytest.raises(ValueError):
        loader.read_gem(tmp_path / "bad.gem")


def test_property_parsing_rules():
    assert loader._as_vec3("1 2 ") == (1.0, 2.0, 0.0)
    assert loader._as_vec3(" 1 2 3") == (0.0, 1.0, 2.0)
    assert loader._as_vec3("1  2") == (1.0, 0.0, 2.0)
    assert loader._as_vec3("1.5abc x 2") == (1.5, 0.0, 2.0)
    assert loader._as_float("", 45.0) == 45.0
    assert loader._as_float("zz", 45.0) == 45.0
    assert loader._as_float("1e99", 7.0) == 7.0             # std::stof throws out_of_range
    assert loader._as_float("0.1", 0.0) == float(np.float32(0.1))
    assert loader._as_int("0.5", 3) == 0 and loader._as_int("x", 3) == 3 and loader._as_int("12.000000", 0) == 12
    assert loader._prop_str(1280.0) == "1280.000000"


@pytest.mark.parametrize("name", COMPLETE + COMPLETE_JPEG)
def test_native_reader_matches_python_loader(pgx_lib, name):
    """pgx_scene_read (C++, csrc/scene_load.cu) gives byte-identical upload
    arrays to the Python reader on every complete reference scene (both
    decode JPEG with the same pgx_image_decode_jpeg)."""
    from pathguidingdissertation_gb300.api import read_scene
    d = _oracle_build.scenes_dir() / name
    if not d.is_dir():
        pytest.skip("reference scenes not available")
    a = loader.load_scene(d)
    b = read_scene(str(d))
    assert a.triangles.tobytes() == b.triangles.tobytes()
    assert a.materials.tobytes() == b.materials.tobytes()
    assert len(a.textures) == len(b.textures)
    for x, y in zip(a.textures, b.textures):
        assert x.shape == y.shape and x.tobytes() == y.tobytes()
    assert (a.env is None) == (b.env is None)
    if a.env is not None:
        assert a.env.tobytes() == b.env.tobytes()
    for k in ("from_", "to", "up"):
        assert np.float32(a.camera[k]).tobytes() == np.float32(b.camera[k]).tobytes()
    assert np.float32(a.camera["fov"]) == np.float32(b.camera["fov"])
    assert (a.camera["width"], a.camera["height"], a.camera["flip_x"]) == \
        (b.camera["width"], b.camera["height"], b.camera["flip_x"])


def test_native_reader_corner_rules(pgx_lib, tmp_path):
    """The loader's corner rules through the native reader: sorted keys,
    last duplicate wins, stof/stoi prefixes and defaults, vector words,
    unknown BSDFs skipped, dielectric below roughness 1e-3 becoming glass,
    a coating dropping the emission, unreadable textures as white, and the
    same arrays as the Python reader."""
    from pathguidingdissertation_gb300.api import read_scene
    d = tmp_path / "s"
    d.mkdir()
    verts = np.zeros((4, 11), np.float32)
    verts[:, :3] = [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]]
    verts[:, 3:6] = [0, 0, 1]
    verts[:, 9:] = [[0, 0], [1, 0], [1, 1], [0, 1]]
    loader.write_gem(d / "quad.gem", [(verts, np.array([0, 1, 2, 0, 2, 3, 0, 0, 0], np.uint32))])
    loader._write_png(d / "a.png", np.array([[[10, 200, 30], [0, 0, 255]]], np.uint8))
    (d / "bad.png").write_bytes(b"not a png")
    js = """{"width": "64x", "height": "  48", "fov": "55.5deg", "from": "0 0  3", "to": "0 0", "up": "0 1 0 9",
      "flipX": true, "width": "32",
      "instances": [
        {"filename": "quad.gem", "bsdf": "diffuse", "reflectance": "a.png",
         "world": [2, 0, 0, 1, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1]},
        {"filename": "quad.gem", "bsdf": "dielectric", "roughness": "0.0005", "intIOR": 1.7,
         "reflectance": "bad.png"},
        {"filename": "quad.gem", "bsdf": "velvet"},
        {"filename": "quad.gem", "bsdf": "conductor", "eta": "0.2 0.9", "k": "3 x 1", "roughness": "",
         "emission": "5 5 5", "coatingThickness": "2", "reflectance": "a.png"}
      ]}"""
    (d / "scene.json").write_text(js)
    a = loader.load_scene(d)
    b = read_scene(str(d))
    assert a.triangles.tobytes() == b.triangles.tobytes()
    assert a.materials.tobytes() == b.materials.tobytes()
    assert [t.tobytes() for t in a.textures] == [t.tobytes() for t in b.textures]
    assert b.camera["width"] == 32 and b.camera["height"] == 48 and b.camera["flip_x"] == 1
    assert len(b.materials) == 3 and b.materials["kind"][1] == BSDF_GLASS
    assert b.materials["layered"][2] == 1 and np.all(b.materials["emission"][2] == 0)
    assert b.textures[1].shape == (1, 1, 3) and np.all(b.textures[1] == 1)
    with pytest.raises(Exception):
        read_scene(str(tmp_path / "missing"))
