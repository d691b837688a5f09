"""ctypes access to the oracle libraries — TEST INFRASTRUCTURE ONLY.

Used by tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline
leg as the checker / CPU baseline; the product (libpgx) never loads it.

* ``Oracle`` — oracle/_build/liboracle.so, the C restatement.
* ``Reference`` — oracle/_ref/liborcref*.so, the reference itself compiled
  headless (available where the reference sources were staged).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_P = C.c_void_p
_I64 = C.c_int64
_I32 = C.c_int32
_U64 = C.c_uint64

# numpy layouts of include/pgx.h structs (duplicated to keep the oracle
# independent of the product package).
VERTEX = np.dtype([("p", "<f4", 3), ("n", "<f4", 3), ("u", "<f4"), ("v", "<f4")])
TRIANGLE = np.dtype([("v", VERTEX, 3), ("material", "<u4")])
RAY = np.dtype([("o", "<f4", 3), ("tmax", "<f4"), ("d", "<f4", 3), ("pad", "<f4")])
HIT = np.dtype([("id", "<i4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4")])
BVH_NODE = np.dtype([("bmin", "<f4", 3), ("bmax", "<f4", 3), ("left_first", "<i4"), ("used", "<i4")])
MATERIAL = np.dtype([
    ("kind", "<i4"), ("albedo_texture", "<i4"), ("albedo", "<f4", 3), ("eta", "<f4", 3), ("k", "<f4", 3),
    ("int_ior", "<f4"), ("ext_ior", "<f4"), ("roughness", "<f4"), ("sigma", "<f4"), ("emission", "<f4", 3),
    ("layered", "<i4"),
])
PATH_VERTEX = np.dtype([("position", "<f4", 3), ("normal", "<f4", 3), ("wi", "<f4", 3), ("Li", "<f4", 3)])
CACHE_NODE = np.dtype([("bmin", "<f4", 3), ("bmax", "<f4", 3), ("left", "<i4"), ("right", "<i4"),
                       ("offset", "<i4"), ("used", "<i4")])


class Texture(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("rgb", C.c_void_p)]


class Camera(C.Structure):
    _fields_ = [("from_", C.c_float * 3), ("to", C.c_float * 3), ("up", C.c_float * 3),
                ("fov_degrees", C.c_float), ("width", C.c_int32), ("height", C.c_int32), ("flip_x", C.c_int32)]


class SceneArgs:
    """Keeps the ctypes views of a scene description alive for one call."""

    def __init__(self, desc):
        self.tris = np.ascontiguousarray(desc.triangles, TRIANGLE)
        self.mats = np.ascontiguousarray(desc.materials, MATERIAL)
        self.texs = [np.ascontiguousarray(t, np.float32) for t in desc.textures]
        self.tex_arr = (Texture * max(1, len(self.texs)))()
        for i, t in enumerate(self.texs):
            self.tex_arr[i] = Texture(t.shape[1], t.shape[0], t.ctypes.data)
        self.env = None
        self.env_arr = None
        if desc.env is not None:
            self.env_arr = np.ascontiguousarray(desc.env, np.float32)
            self.env = Texture(self.env_arr.shape[1], self.env_arr.shape[0], self.env_arr.ctypes.data)
        c = desc.camera
        self.cam = Camera((C.c_float * 3)(*c["from_"]), (C.c_float * 3)(*c["to"]), (C.c_float * 3)(*c["up"]),
                          float(c["fov"]), int(c["width"]), int(c["height"]), int(c.get("flip_x", 0)))
        self.width = int(c["width"])
        self.height = int(c["height"])

    def args(self):
        return (_p(self.tris), len(self.tris), _p(self.mats), len(self.mats),
                C.cast(self.tex_arr, C.c_void_p) if self.texs else None, len(self.texs),
                C.byref(self.env) if self.env is not None else None, C.byref(self.cam))


def _p(a):
    return None if a is None else a.ctypes.data


class Oracle:
    def __init__(self, path: str | Path | None = None):
        if path is None:
            from . import build as _b  # noqa: PLC0415
            path = _b.build_oracle()
        self.lib = C.CDLL(str(path))
        L = self.lib
        L.orc_bvh_build.restype = _I64
        L.orc_bvh_build.argtypes = [_P, _I64, _P, _P]
        L.orc_sah_cost.restype = C.c_double
        L.orc_sah_cost.argtypes = [_P, _I64]
        for name in ("orc_trace_closest", "orc_trace_any"):
            fn = getattr(L, name)
            fn.restype = None
            fn.argtypes = [_P, _P, _P, _P, _I64, _P, C.POINTER(_I64), C.POINTER(_I64)]
        L.orc_trace_closest_mt.restype = None
        L.orc_trace_closest_mt.argtypes = [_P, _P, _P, _P, _I64, _P, _I32]
        L.orc_rng_floats.restype = None
        L.orc_rng_floats.argtypes = [_U64, _U64, _U64, _I32, _P]

    def bvh_build(self, tris: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        tris = np.ascontiguousarray(tris, TRIANGLE)
        n = len(tris)
        nodes = np.zeros(max(1, 2 * n - 1), BVH_NODE)
        idx = np.zeros(max(1, n), np.int32)
        cnt = self.lib.orc_bvh_build(_p(tris), n, _p(nodes), _p(idx))
        return nodes[:cnt].copy(), idx[:n].copy()

    def sah_cost(self, nodes: np.ndarray) -> float:
        nodes = np.ascontiguousarray(nodes, BVH_NODE)
        return float(self.lib.orc_sah_cost(_p(nodes), len(nodes)))

    def trace_closest(self, tris, nodes, idx, rays) -> tuple[np.ndarray, int, int]:
        tris = np.ascontiguousarray(tris, TRIANGLE)
        nodes = np.ascontiguousarray(nodes, BVH_NODE)
        idx = np.ascontiguousarray(idx, np.int32)
        rays = np.ascontiguousarray(rays, RAY)
        hits = np.zeros(len(rays), HIT)
        a, b = _I64(0), _I64(0)
        self.lib.orc_trace_closest(_p(tris), _p(nodes), _p(idx), _p(rays), len(rays), _p(hits), C.byref(a),
                                   C.byref(b))
        return hits, a.value, b.value

    def trace_any(self, tris, nodes, idx, rays) -> tuple[np.ndarray, int, int]:
        tris = np.ascontiguousarray(tris, TRIANGLE)
        nodes = np.ascontiguousarray(nodes, BVH_NODE)
        idx = np.ascontiguousarray(idx, np.int32)
        rays = np.ascontiguousarray(rays, RAY)
        vis = np.zeros(len(rays), np.uint8)
        a, b = _I64(0), _I64(0)
        self.lib.orc_trace_any(_p(tris), _p(nodes), _p(idx), _p(rays), len(rays), _p(vis), C.byref(a), C.byref(b))
        return vis, a.value, b.value

    def trace_closest_mt(self, tris, nodes, idx, rays, threads: int) -> np.ndarray:
        tris = np.ascontiguousarray(tris, TRIANGLE)
        nodes = np.ascontiguousarray(nodes, BVH_NODE)
        idx = np.ascontiguousarray(idx, np.int32)
        rays = np.ascontiguousarray(rays, RAY)
        hits = np.zeros(len(rays), HIT)
        self.lib.orc_trace_closest_mt(_p(tris), _p(nodes), _p(idx), _p(rays), len(rays), _p(hits), threads)
        return hits

    def rng_floats(self, seed: int, pixel: int, sample: int, count: int) -> np.ndarray:
        out = np.zeros(count, np.float32)
        self.lib.orc_rng_floats(seed, pixel, sample, count, _p(out))
        return out


def reference_available() -> bool:
    from . import build as _b  # noqa: PLC0415
    return (HERE / "_ref" / "liborcref.so").exists() or (HERE / "_ref" / "src" / "Renderer.h").exists() or \
        (_b.reference_sources() / "Renderer.h").exists()


class Reference:
    """The reference renderer compiled headless (oracle/ref_harness.cpp).

    variant: "parity" (-O2 -ffp-contract=off, GUIDED_PATH as shipped),
    "fast" (-O3, as shipped) or "plain_fast" (-O3, GUIDED_PATH false)."""

    def __init__(self, fast: bool = False, variant: str | None = None):
        from . import build as _b  # noqa: PLC0415
        p = _b.build_reference()
        if p is None:
            raise RuntimeError("reference sources unavailable")
        variant = variant or ("fast" if fast else "parity")
        names = {"parity": "liborcref.so", "fast": "liborcref_fast.so", "plain_fast": "liborcref_plain_fast.so"}
        p = p.parent / names[variant]
        self.lib = C.CDLL(str(p))
        L = self.lib
        L.orcref_bvh_build.restype = _I64
        L.orcref_bvh_build.argtypes = [_P, _I64, _P, _P]
        L.orcref_world_create.restype = _P
        L.orcref_world_create.argtypes = [_P, _I64]
        L.orcref_world_destroy.restype = None
        L.orcref_world_destroy.argtypes = [_P]
        L.orcref_trace_closest.restype = C.c_double
        L.orcref_trace_closest.argtypes = [_P, _P, _I64, _P, _I32]
        L.orcref_trace_any.restype = C.c_double
        L.orcref_trace_any.argtypes = [_P, _P, _I64, _P, _I32]
        L.orcref_rng_floats.restype = None
        L.orcref_rng_floats.argtypes = [_U64, _U64, _U64, _I32, _P]
        L.orcref_scene_create.restype = _P
        L.orcref_scene_create.argtypes = [_P, _I64, _P, _I32, _P, _I32, _P, _P, _I32]
        L.orcref_scene_destroy.restype = None
        L.orcref_scene_destroy.argtypes = [_P]
        L.orcref_render_pcg.restype = _I64
        L.orcref_render_pcg.argtypes = [_P, _I32, _U64, _I32, _I32, _P, _I32, _I32, _P, _I64, C.POINTER(_I64)]
        L.orcref_render_native.restype = C.c_double
        L.orcref_render_native.argtypes = [_P, _I32, _P, C.POINTER(_I32), C.POINTER(_I64)]
        L.orcref_clear.restype = None
        L.orcref_clear.argtypes = [_P]
        L.orcref_camera_rays.restype = None
        L.orcref_camera_rays.argtypes = [_P, _P, _P, _I64, _P, _P]
        L.orcref_pointbvh.restype = _I64
        L.orcref_pointbvh.argtypes = [_P, _I64, _P, _P]
        L.orcref_set_filter.restype = None
        L.orcref_set_filter.argtypes = [_I32]
        L.orcref_tonemap.restype = None
        L.orcref_tonemap.argtypes = [_P, _I32, _I32, _I32, C.c_float, C.c_float, _P]
        L.orcref_metrics.restype = None
        L.orcref_metrics.argtypes = [_P, _P, _I32, _I32, _P]
        L.orcref_bsdf_roundtrip.restype = None
        L.orcref_bsdf_roundtrip.argtypes = [_P, _P, _P, _P, _I64, _P, _P, _P, _P]
        L.orcref_load_scene.restype = _P
        L.orcref_load_scene.argtypes = [C.c_char_p, _P]
        L.orcref_loaded_from_arrays.restype = _P
        L.orcref_loaded_from_arrays.argtypes = [_P, _I64, _P, _I32, _P, _I32, _P, _P, _P]
        L.orcref_loaded_destroy.restype = None
        L.orcref_loaded_destroy.argtypes = [_P]
        for f in (L.orcref_loaded_triangles, L.orcref_loaded_materials, L.orcref_loaded_camera):
            f.restype = None
            f.argtypes = [_P, _P]
        L.orcref_texture_load.restype = _P
        L.orcref_texture_load.argtypes = [C.c_char_p, _P]
        L.orcref_texture_read.restype = None
        L.orcref_texture_read.argtypes = [_P, _P]
        for f in (L.orcref_loaded_texture_size, L.orcref_loaded_texture):
            f.restype = None
            f.argtypes = [_P, _I32, _P]

    def bvh_build(self, tris: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        tris = np.ascontiguousarray(tris, TRIANGLE)
        n = len(tris)
        nodes = np.zeros(max(1, 2 * n - 1), BVH_NODE)
        idx = np.zeros(max(1, n), np.int32)
        cnt = self.lib.orcref_bvh_build(_p(tris), n, _p(nodes), _p(idx))
        return nodes[:cnt].copy(), idx[:n].copy()

    def set_filter(self, mitchell: bool) -> None:
        self.lib.orcref_set_filter(int(mitchell))

    def tonemap(self, film: np.ndarray, spp: int, exposure: float = 1.0, lmax_white: float = 10.0) -> np.ndarray:
        f = np.ascontiguousarray(film, np.float32).copy()
        h, w = f.shape[:2]
        out = np.zeros((h, w, 3), np.uint8)
        self.lib.orcref_tonemap(_p(f), w, h, spp, exposure, lmax_white, _p(out))
        return out

    def metrics(self, test: np.ndarray, gt: np.ndarray) -> tuple[float, float, float]:
        t = np.ascontiguousarray(test, np.float32)
        g = np.ascontiguousarray(gt, np.float32)
        h, w = t.shape[:2]
        out = np.zeros(3, np.float32)
        self.lib.orcref_metrics(_p(t), _p(g), w, h, _p(out))
        return float(out[0]), float(out[1]), float(out[2])

    def bsdf_roundtrip(self, material, normals, wo, uv):
        """Reference BSDF::sample (TestSampler) and BSDF::invert per row."""
        mat = np.ascontiguousarray(material, MATERIAL).reshape(())
        n = np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
        o = np.ascontiguousarray(wo, np.float32).reshape(-1, 3)
        u = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
        cnt = len(u)
        wi = np.zeros((cnt, 3), np.float32)
        f = np.zeros((cnt, 3), np.float32)
        pdf = np.zeros(cnt, np.float32)
        uv_out = np.zeros((cnt, 2), np.float32)
        self.lib.orcref_bsdf_roundtrip(mat.ctypes.data, _p(n), _p(o), _p(u), cnt, _p(wi), _p(f), _p(pdf),
                                       _p(uv_out))
        return wi, f, pdf, uv_out

    def _export_loaded(self, h, counts: np.ndarray) -> dict:
        L = self.lib
        try:
            tris = np.zeros(int(counts[0]), TRIANGLE)
            L.orcref_loaded_triangles(h, _p(tris))
            mats = np.zeros((int(counts[1]), 20), np.float32)
            L.orcref_loaded_materials(h, _p(mats))
            texs = []
            for i in list(range(int(counts[2]))) + [-1]:
                wh = np.zeros(2, np.int32)
                L.orcref_loaded_texture_size(h, i, _p(wh))
                if wh[0] == 0:
                    texs.append(None)
                    continue
                img = np.zeros((int(wh[1]), int(wh[0]), 3), np.float32)
                L.orcref_loaded_texture(h, i, _p(img))
                texs.append(img)
            cam = np.zeros(32, np.float32)
            L.orcref_loaded_camera(h, _p(cam))
        finally:
            L.orcref_loaded_destroy(h)
        return dict(triangles=tris, materials=mats, textures=texs[:-1], env=texs[-1],
                    projection=cam[:16].reshape(4, 4), camera=cam[16:].reshape(4, 4),
                    width=int(counts[3]), height=int(counts[4]))

    def load_texture(self, filename: str) -> np.ndarray:
        """Texture::load of one image file: (H, W, 3) float32 texels."""
        wh = np.zeros(2, np.int32)
        h = self.lib.orcref_texture_load(str(filename).encode(), _p(wh))
        img = np.zeros((int(wh[1]), int(wh[0]), 3), np.float32)
        self.lib.orcref_texture_read(h, _p(img))
        return img

    def load_scene(self, scene_dir: str) -> dict:
        """The reference's loadScene on a scene directory, exported: triangles,
        per-material parameters (20 floats, see orcref_loaded_materials),
        distinct albedo textures, environment texels and camera matrices."""
        counts = np.zeros(5, np.int64)
        h = self.lib.orcref_load_scene(str(scene_dir).encode(), _p(counts))
        return self._export_loaded(h, counts)

    def loaded_from_desc(self, desc) -> dict:
        """The same export for a scene assembled from pgx upload arrays."""
        sa = SceneArgs(desc)
        counts = np.zeros(5, np.int64)
        h = self.lib.orcref_loaded_from_arrays(*sa.args(), _p(counts))
        return self._export_loaded(h, counts)

    def world(self, tris: np.ndarray) -> "RefWorld":
        return RefWorld(self, tris)

    def scene(self, desc, threads: int = 0) -> "RefScene":
        return RefScene(self, desc, threads)

    def pointbvh(self, records: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        records = np.ascontiguousarray(records, PATH_VERTEX)
        n = len(records)
        nodes = np.zeros(max(1, 2 * n), CACHE_NODE)
        out = np.zeros(max(1, n), PATH_VERTEX)
        cnt = self.lib.orcref_pointbvh(_p(records), n, _p(nodes), _p(out))
        return nodes[:cnt].copy(), out[:n].copy()


class RefScene:
    """A reference `Scene` + `RayTracer` (SceneLoader.h:222-269)."""

    def __init__(self, ref: "Reference", desc, threads: int = 0):
        self.ref = ref
        self.sa = SceneArgs(desc)
        self.h = ref.lib.orcref_scene_create(*self.sa.args(), threads)

    def close(self):
        if self.h:
            self.ref.lib.orcref_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def render_pcg(self, guided: bool, seed: int, spp0: int, nspp: int, threads: int = 8, collect: int = -1,
                   vcap: int = 0):
        film = np.zeros((self.sa.height, self.sa.width, 3), np.float32)
        verts = np.zeros(max(1, vcap), PATH_VERTEX)
        rays = _I64(0)
        nv = self.ref.lib.orcref_render_pcg(self.h, int(guided), seed, spp0, nspp, _p(film), threads, collect,
                                            _p(verts), vcap, C.byref(rays))
        return film, verts[:min(nv, vcap)].copy(), rays.value

    def render_native(self, frames: int):
        film = np.zeros((self.sa.height, self.sa.width, 3), np.float32)
        spp = _I32(0)
        rays = _I64(0)
        secs = self.ref.lib.orcref_render_native(self.h, frames, _p(film), C.byref(spp), C.byref(rays))
        return film, spp.value, rays.value, secs

    def clear(self):
        self.ref.lib.orcref_clear(self.h)

    def camera_rays(self, px: np.ndarray, py: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """Camera::generateRay at film positions (px, py): origins, directions."""
        px = np.ascontiguousarray(px, np.float32)
        py = np.ascontiguousarray(py, np.float32)
        o = np.zeros((len(px), 3), np.float32)
        d = np.zeros((len(px), 3), np.float32)
        self.ref.lib.orcref_camera_rays(self.h, _p(px), _p(py), len(px), _p(o), _p(d))
        return o, d


class RefWorld:
    def __init__(self, ref: Reference, tris: np.ndarray):
        self.ref = ref
        self.tris = np.ascontiguousarray(tris, TRIANGLE)
        self.h = ref.lib.orcref_world_create(_p(self.tris), len(self.tris))

    def close(self):
        if self.h:
            self.ref.lib.orcref_world_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def trace_closest(self, rays: np.ndarray, threads: int = 1) -> tuple[np.ndarray, float]:
        rays = np.ascontiguousarray(rays, RAY)
        hits = np.zeros(len(rays), HIT)
        secs = self.ref.lib.orcref_trace_closest(self.h, _p(rays), len(rays), _p(hits), threads)
        return hits, secs

    def trace_any(self, rays: np.ndarray, threads: int = 1) -> tuple[np.ndarray, float]:
        rays = np.ascontiguousarray(rays, RAY)
        vis = np.zeros(len(rays), np.uint8)
        secs = self.ref.lib.orcref_trace_any(self.h, _p(rays), len(rays), _p(vis), threads)
        return vis, secs
