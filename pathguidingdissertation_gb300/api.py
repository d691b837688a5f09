"""Python mirror of the reference's renderer interface over the C ABI.

``Context`` wraps one ``pgx_ctx``.  ``Scene`` and ``RayTracer`` keep the
reference's names and semantics (Scene.h:76-176, Renderer.h:236-752):
``Scene.init``/``build``/``traverse``/``visible``, ``RayTracer.init``/
``render`` (one sample per pixel per call, accumulated)/``clear``/``getSPP``/
``saveHDR``.  All work happens in libpgx; nothing here computes on the CPU.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import abi
from .abi import PgxError, ptr
from .scenes import SceneDesc


class Context:
    def __init__(self, device: int = 0, lib_path=None):
        self.lib = abi.load(lib_path)
        h = C.c_void_p()
        rc = self.lib.pgx_create(device, C.byref(h))
        if rc != abi.PGX_OK:
            raise PgxError(rc, self.lib.pgx_last_error(None).decode())
        self.h = h
        self.scene: SceneDesc | None = None

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.pgx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def check(self, rc: int) -> None:
        if rc != abi.PGX_OK:
            raise PgxError(rc, self.lib.pgx_last_error(self.h).decode())

    # ---- scene ---------------------------------------------------------------
    def upload(self, scene: SceneDesc) -> None:
        tris = np.ascontiguousarray(scene.triangles)
        mats = np.ascontiguousarray(scene.materials)
        texs = [np.ascontiguousarray(t, dtype=np.float32) for t in scene.textures]
        tex_arr = (abi.Texture * max(1, len(texs)))()
        for i, t in enumerate(texs):
            tex_arr[i] = abi.Texture(t.shape[1], t.shape[0], t.ctypes.data)
        env = None
        env_keep = None
        if scene.env is not None:
            env_keep = np.ascontiguousarray(scene.env, dtype=np.float32)
            env = abi.Texture(env_keep.shape[1], env_keep.shape[0], env_keep.ctypes.data)
        cam = camera_struct(scene.camera)
        self.check(self.lib.pgx_scene_upload(self.h, ptr(tris), len(tris), ptr(mats), len(mats),
                                             C.cast(tex_arr, C.c_void_p) if texs else None, len(texs),
                                             C.byref(env) if env is not None else None, C.byref(cam)))
        self.scene = scene
        del env_keep, texs

    def load_scene(self, scene_dir: str) -> SceneDesc:
        """pgx_scene_load: the reference's scene directory read by the native
        loader and uploaded; returns the same arrays as a SceneDesc."""
        desc = read_scene(scene_dir)
        self.check(self.lib.pgx_scene_load(self.h, str(scene_dir).encode()))
        self.scene = desc
        return desc

    def bvh_build(self) -> None:
        self.check(self.lib.pgx_bvh_build(self.h))

    def bvh_import(self, nodes: np.ndarray, idx: np.ndarray) -> None:
        nodes = np.ascontiguousarray(nodes, abi.BVH_NODE)
        idx = np.ascontiguousarray(idx, np.int32)
        self.check(self.lib.pgx_bvh_import(self.h, ptr(nodes), len(nodes), ptr(idx)))

    def bvh_export(self) -> tuple[np.ndarray, np.ndarray]:
        nn, ni = C.c_int64(), C.c_int64()
        self.check(self.lib.pgx_bvh_export(self.h, None, C.byref(nn), None, C.byref(ni)))
        nodes = np.zeros(nn.value, abi.BVH_NODE)
        idx = np.zeros(ni.value, np.int32)
        self.check(self.lib.pgx_bvh_export(self.h, ptr(nodes), C.byref(nn), ptr(idx), C.byref(ni)))
        return nodes, idx

    def bvh_stats(self) -> abi.BvhStats:
        s = abi.BvhStats()
        self.check(self.lib.pgx_bvh_get_stats(self.h, C.byref(s)))
        return s

    # ---- rays ------------------------------------------------------------------
    def trace_closest(self, rays: np.ndarray) -> np.ndarray:
        rays = np.ascontiguousarray(rays, abi.RAY)
        hits = np.zeros(len(rays), abi.HIT)
        self.check(self.lib.pgx_trace_closest(self.h, ptr(rays), len(rays), ptr(hits)))
        return hits

    def trace_closest_noalloc(self, rays: np.ndarray) -> np.ndarray:
        """pgx_trace_closest_noalloc: same hits, no device allocation, at
        most abi.NOALLOC_MAX_RAYS rays per call."""
        rays = np.ascontiguousarray(rays, abi.RAY)
        hits = np.zeros(len(rays), abi.HIT)
        self.check(self.lib.pgx_trace_closest_noalloc(self.h, ptr(rays), len(rays), ptr(hits)))
        return hits

    def trace_any(self, rays: np.ndarray) -> np.ndarray:
        rays = np.ascontiguousarray(rays, abi.RAY)
        vis = np.zeros(len(rays), np.uint8)
        self.check(self.lib.pgx_trace_any(self.h, ptr(rays), len(rays), ptr(vis)))
        return vis

    def trace_counters(self) -> tuple[int, int]:
        a, b = C.c_int64(), C.c_int64()
        self.check(self.lib.pgx_trace_counters(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def camera_rays(self, px: np.ndarray, py: np.ndarray) -> np.ndarray:
        px = np.ascontiguousarray(px, np.float32)
        py = np.ascontiguousarray(py, np.float32)
        out = np.zeros(len(px), abi.RAY)
        self.check(self.lib.pgx_camera_rays(self.h, ptr(px), ptr(py), len(px), ptr(out)))
        return out

    # ---- rendering -------------------------------------------------------------
    def set_camera(self, camera: dict) -> None:
        self.check(self.lib.pgx_set_camera(self.h, C.byref(camera_struct(camera))))

    def render(self, frames: int = 1, mode: int = abi.MODE_PLAIN, seed: int = 1, max_depth: int = 8,
               guide_fraction: float = 0.5, record_paths: int | bool = 0, profile: bool = False,
               mitchell: bool = False, train_guide: bool = False, guide_depth: int = 0, timing: bool = False) -> None:
        """profile: per-stage times and traversal counters (counting kernels);
        timing: per-stage times only (the kernels of an unflagged render)."""
        flags = (abi.RENDER_PROFILE if profile else 0) | (abi.RENDER_FILTER_MITCHELL if mitchell else 0) | \
            (abi.RENDER_TRAIN_GUIDE if train_guide else 0) | (abi.RENDER_TIMING if timing else 0)
        cfg = abi.RenderConfig(mode, max_depth, seed, guide_fraction, int(record_paths), flags, guide_depth)
        self.check(self.lib.pgx_render(self.h, C.byref(cfg), frames))

    def clear(self) -> None:
        self.check(self.lib.pgx_clear(self.h))

    def spp(self) -> int:
        s = C.c_int32()
        self.check(self.lib.pgx_get_spp(self.h, C.byref(s)))
        return s.value

    def film(self, squares: bool = False) -> tuple[np.ndarray, np.ndarray | None, int]:
        w, h = self.scene.camera["width"], self.scene.camera["height"]
        rgb = np.zeros((h, w, 3), np.float32)
        rgb2 = np.zeros((h, w, 3), np.float32) if squares else None
        s = C.c_int32()
        self.check(self.lib.pgx_film_read(self.h, ptr(rgb), ptr(rgb2), C.byref(s)))
        return rgb, rgb2, s.value

    def tonemap(self, exposure: float = 1.0, lmax_white: float = 10.0) -> np.ndarray:
        """Film::tonemap of every pixel: (H, W, 3) uint8."""
        w, h = self.scene.camera["width"], self.scene.camera["height"]
        out = np.zeros((h, w, 3), np.uint8)
        self.check(self.lib.pgx_film_tonemap(self.h, exposure, lmax_white, ptr(out)))
        return out

    def render_stats(self) -> abi.RenderStats:
        s = abi.RenderStats()
        self.check(self.lib.pgx_render_get_stats(self.h, C.byref(s)))
        return s

    # ---- BSDF queries ---------------------------------------------------------
    def bsdf_sample(self, material: np.ndarray, normals: np.ndarray, wo: np.ndarray, uv: np.ndarray):
        """BSDF::sample with TestSampler semantics: (wi, f, pdf) per row."""
        mat = np.ascontiguousarray(material, abi.MATERIAL).reshape(())
        n = np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
        o = np.ascontiguousarray(wo, np.float32).reshape(-1, 3)
        u = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
        wi = np.zeros((len(u), 3), np.float32)
        f = np.zeros((len(u), 3), np.float32)
        pdf = np.zeros(len(u), np.float32)
        self.check(self.lib.pgx_bsdf_sample_batch(self.h, mat.ctypes.data, ptr(n), ptr(o), ptr(u), len(u), ptr(wi),
                                                  ptr(f), ptr(pdf)))
        return wi, f, pdf

    def bsdf_invert(self, material: np.ndarray, normals: np.ndarray, wo: np.ndarray, wi: np.ndarray) -> np.ndarray:
        mat = np.ascontiguousarray(material, abi.MATERIAL).reshape(())
        n = np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
        o = np.ascontiguousarray(wo, np.float32).reshape(-1, 3)
        w = np.ascontiguousarray(wi, np.float32).reshape(-1, 3)
        uv = np.zeros((len(w), 2), np.float32)
        self.check(self.lib.pgx_bsdf_invert_batch(self.h, mat.ctypes.data, ptr(n), ptr(o), ptr(w), len(w), ptr(uv)))
        return uv

    # ---- radiance cache -------------------------------------------------------
    def cache_build(self, records: np.ndarray) -> None:
        records = np.ascontiguousarray(records, abi.PATH_VERTEX)
        self.check(self.lib.pgx_cache_build(self.h, ptr(records), len(records)))

    def cache_build_from_render(self) -> None:
        self.check(self.lib.pgx_cache_build_from_render(self.h))

    def cache_stats(self) -> abi.CacheStats:
        s = abi.CacheStats()
        self.check(self.lib.pgx_cache_get_stats(self.h, C.byref(s)))
        return s

    def cache_export(self) -> tuple[np.ndarray, np.ndarray]:
        nn, nr = C.c_int64(), C.c_int64()
        self.check(self.lib.pgx_cache_export(self.h, None, C.byref(nn), None, C.byref(nr)))
        nodes = np.zeros(nn.value, abi.CACHE_NODE)
        recs = np.zeros(nr.value, abi.PATH_VERTEX)
        self.check(self.lib.pgx_cache_export(self.h, ptr(nodes), C.byref(nn), ptr(recs), C.byref(nr)))
        return nodes, recs

    def cache_weights(self) -> np.ndarray:
        """The QuadTree guide's flux weight of each exported record
        (pgx_cache_export_weights)."""
        nr = C.c_int64()
        self.check(self.lib.pgx_cache_export_weights(self.h, None, C.byref(nr)))
        w = np.zeros(nr.value, np.float32)
        self.check(self.lib.pgx_cache_export_weights(self.h, ptr(w), C.byref(nr)))
        return w

    def guide_pdf(self, positions: np.ndarray, dirs: np.ndarray) -> np.ndarray:
        p = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
        out = np.zeros(len(p), np.float32)
        self.check(self.lib.pgx_guide_pdf(self.h, ptr(p), ptr(d), len(p), ptr(out)))
        return out

    def guide_sample(self, positions: np.ndarray, u2: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        p = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
        u = np.ascontiguousarray(u2, np.float32).reshape(-1, 2)
        dirs = np.zeros((len(p), 3), np.float32)
        pdf = np.zeros(len(p), np.float32)
        self.check(self.lib.pgx_guide_sample(self.h, ptr(p), ptr(u), len(p), ptr(dirs), ptr(pdf)))
        return dirs, pdf

    def guide_export(self) -> tuple[np.ndarray, np.ndarray, bool]:
        """The QuadTree guide's regions and quad nodes (pgx_guide_export)."""
        nreg, pss = C.c_int32(), C.c_int32()
        self.check(self.lib.pgx_guide_export(self.h, None, C.byref(nreg), None, C.byref(pss)))
        regions = np.zeros(nreg.value, abi.GUIDE_REGION)
        qnodes = np.zeros(nreg.value * abi.GUIDE_MAX_QUAD_NODES, abi.QUAD_NODE)
        if nreg.value:
            self.check(self.lib.pgx_guide_export(self.h, ptr(regions), C.byref(nreg), ptr(qnodes), C.byref(pss)))
        return regions, qnodes, bool(pss.value)

    def guide_configure(self, region_records: int = 1024, refine_fraction: float = 0.01,
                        clamp_median: float = 10.0, uniform_share: float = 0.2, compensate: float = 0.0,
                        glossy_alpha: float = 0.0) -> None:
        """QuadTree guide parameters (pgx_guide_configure): region size,
        refinement share, flux clamp and MIS compensation shape the next
        cache build; the uniform share and the glossy threshold apply to
        later renders (the share also to queries)."""
        gp = abi.GuideParams(region_records, refine_fraction, clamp_median, uniform_share, compensate, glossy_alpha)
        self.check(self.lib.pgx_guide_configure(self.h, C.byref(gp)))

    def guide_params(self) -> dict:
        gp = abi.GuideParams()
        self.check(self.lib.pgx_guide_get_params(self.h, C.byref(gp)))
        return {f: getattr(gp, f) for f, _ in gp._fields_}

    # ---- learned guide ----
    def mlp_init(self, seed: int = 1, bmin=None, bmax=None) -> None:
        lo = None if bmin is None else np.ascontiguousarray(bmin, np.float32)
        hi = None if bmax is None else np.ascontiguousarray(bmax, np.float32)
        self.check(self.lib.pgx_mlp_init(self.h, seed, ptr(lo), ptr(hi)))

    def mlp_params(self) -> np.ndarray:
        out = np.zeros(abi.MLP_PARAMS, np.float32)
        self.check(self.lib.pgx_mlp_get_params(self.h, ptr(out)))
        return out

    def mlp_set_params(self, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, np.float32)
        assert p.size == abi.MLP_PARAMS
        self.check(self.lib.pgx_mlp_set_params(self.h, ptr(p)))

    @staticmethod
    def _queries(queries) -> np.ndarray:
        return np.ascontiguousarray(queries, np.float32).reshape(-1, 9)

    def mlp_forward(self, queries: np.ndarray) -> np.ndarray:
        q = self._queries(queries)
        out = np.zeros((len(q), abi.MLP_OUTPUTS), np.float32)
        self.check(self.lib.pgx_mlp_forward(self.h, ptr(q), len(q), ptr(out)))
        return out

    def mlp_pdf(self, queries: np.ndarray, dirs: np.ndarray) -> np.ndarray:
        q = self._queries(queries)
        d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
        out = np.zeros(len(q), np.float32)
        self.check(self.lib.pgx_mlp_pdf(self.h, ptr(q), ptr(d), len(q), ptr(out)))
        return out

    def mlp_sample(self, queries: np.ndarray, u3: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        q = self._queries(queries)
        u = np.ascontiguousarray(u3, np.float32).reshape(-1, 3)
        dirs = np.zeros((len(q), 3), np.float32)
        pdf = np.zeros(len(q), np.float32)
        self.check(self.lib.pgx_mlp_sample(self.h, ptr(q), ptr(u), len(q), ptr(dirs), ptr(pdf)))
        return dirs, pdf

    def mlp_gradient(self, samples: np.ndarray) -> tuple[np.ndarray, float]:
        s = np.ascontiguousarray(samples, abi.RADIANCE_SAMPLE)
        g = np.zeros(abi.MLP_PARAMS, np.float32)
        loss = C.c_double(0.0)
        self.check(self.lib.pgx_mlp_gradient(self.h, ptr(s), len(s), ptr(g), C.byref(loss)))
        return g, loss.value

    def mlp_train_step(self, samples: np.ndarray, lr: float = 1e-2) -> float:
        s = np.ascontiguousarray(samples, abi.RADIANCE_SAMPLE)
        loss = C.c_double(0.0)
        self.check(self.lib.pgx_mlp_train_step(self.h, ptr(s), len(s), lr, C.byref(loss)))
        return loss.value

    def mlp_set_fallback(self, min_samples: int) -> None:
        """pgx_mlp_set_fallback: regions whose training samples number fewer
        than min_samples are guided by the QuadTree guide (0: never)."""
        self.check(self.lib.pgx_mlp_set_fallback(self.h, int(min_samples)))

    def mlp_configure(self, lr: float = 5e-3, decay: float = 0.998, batch: int = 262144, steps: int = 4,
                      direct: bool = True) -> None:
        self.check(self.lib.pgx_mlp_configure(self.h, lr, decay, batch, steps, int(direct)))

    # ---- differentiable rendering ----
    def diff_set_params(self, env: np.ndarray | None = None, albedo_offset: np.ndarray | None = None,
                        roughness: np.ndarray | None = None) -> None:
        e = None if env is None else np.ascontiguousarray(env, np.float32)
        a = None if albedo_offset is None else np.ascontiguousarray(albedo_offset, np.float32)
        r = None if roughness is None else np.ascontiguousarray(roughness, np.float32)
        self.check(self.lib.pgx_diff_set_params(self.h, ptr(e), ptr(a), ptr(r)))

    def diff_render(self, spp: int, seed: int = 1, max_depth: int = 8) -> np.ndarray:
        w, h = self.scene.camera["width"], self.scene.camera["height"]
        img = np.zeros((h, w, 3), np.float64)
        self.check(self.lib.pgx_diff_render(self.h, spp, seed, max_depth, ptr(img)))
        return img

    def diff_adjoint(self, dloss_dimage: np.ndarray, spp: int, seed: int = 1, max_depth: int = 8):
        """(grad_env (H_env, W_env, 3) or None, grad_albedo (nmats, 3), grad_roughness (nmats,))."""
        d = np.ascontiguousarray(dloss_dimage, np.float32)
        nm = len(self.scene.materials)
        env = self.scene.env
        ge = None if env is None else np.zeros(env.shape, np.float32)
        ga = np.zeros((nm, 3), np.float32)
        gr = np.zeros(nm, np.float32)
        self.check(self.lib.pgx_diff_adjoint(self.h, spp, seed, max_depth, ptr(d), ptr(ge), ptr(ga), ptr(gr)))
        return ge, ga, gr

    def cache_knn(self, queries: np.ndarray, k: int) -> tuple[np.ndarray, np.ndarray]:
        q = np.ascontiguousarray(queries, np.float32).reshape(-1, 3)
        idx = np.zeros((len(q), k), np.int32)
        d2 = np.zeros((len(q), k), np.float32)
        self.check(self.lib.pgx_cache_knn(self.h, ptr(q), len(q), k, ptr(idx), ptr(d2)))
        return idx, d2


class Batch:
    """Many scenes (one Context each, same device) rendered by one persistent,
    graph-captured launch (pgx_batch_*)."""

    def __init__(self, contexts: list[Context]):
        self.contexts = list(contexts)
        self.lib = abi.load()
        arr = (C.c_void_p * len(self.contexts))(*[c.h for c in self.contexts])
        h = C.c_void_p()
        rc = self.lib.pgx_batch_create(arr, len(self.contexts), C.byref(h))
        if rc != 0:
            raise PgxError(rc, "pgx_batch_create failed (scenes need an uploaded scene and a BVH on one device)")
        self.h = h

    def check(self, rc: int) -> None:
        if rc != 0:
            raise PgxError(rc, self.lib.pgx_batch_last_error(self.h).decode())

    def render(self, spp: int, seed: int = 1, max_depth: int = 8) -> None:
        self.check(self.lib.pgx_batch_render(self.h, spp, seed, max_depth))

    def autotune(self, spp: int = 1, max_depth: int = 8) -> abi.BatchTuning:
        t = abi.BatchTuning()
        self.check(self.lib.pgx_batch_autotune(self.h, spp, max_depth, C.byref(t)))
        return t

    def set_tuning(self, wave_paths: int, trace_blocks_per_sm: int, shade_blocks_per_sm: int,
                   stack_shared: int = 8) -> None:
        t = abi.BatchTuning(wave_paths, trace_blocks_per_sm, shade_blocks_per_sm, stack_shared)
        self.check(self.lib.pgx_batch_set_tuning(self.h, C.byref(t)))

    def stats(self) -> abi.BatchStats:
        s = abi.BatchStats()
        self.check(self.lib.pgx_batch_get_stats(self.h, C.byref(s)))
        return s

    def close(self) -> None:
        if self.h:
            self.lib.pgx_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_scene(scene_dir: str) -> SceneDesc:
    """`loadScene` by the native reader (pgx_scene_read), copied into a
    SceneDesc.  Raises PgxError for a missing or malformed scene."""
    lib = abi.load()
    out = C.POINTER(abi.SceneData)()
    msg = C.create_string_buffer(512)
    rc = lib.pgx_scene_read(str(scene_dir).encode(), C.byref(out), msg, 512)
    if rc != abi.PGX_OK:
        raise PgxError(rc, msg.value.decode(errors="replace"))
    try:
        d = out.contents

        def arr(p, n, dtype):
            if n == 0:
                return np.zeros(0, dtype)
            buf = (C.c_uint8 * (n * dtype.itemsize)).from_address(p)
            return np.frombuffer(buf, dtype, n).copy()

        def tex(t):
            return arr(t.rgb, t.width * t.height * 3, np.dtype(np.float32)).reshape(t.height, t.width, 3)

        tris = arr(d.triangles, d.ntris, abi.TRIANGLE)
        mats = arr(d.materials, d.nmats, abi.MATERIAL)
        texs = [tex(abi.Texture.from_address(d.textures + i * C.sizeof(abi.Texture))) for i in range(d.ntextures)]
        env = tex(d.env) if d.has_env else None
        c = d.camera
        cam = dict(from_=tuple(c.from_), to=tuple(c.to), up=tuple(c.up), fov=c.fov_degrees, width=c.width,
                   height=c.height, flip_x=c.flip_x)
    finally:
        lib.pgx_scene_data_free(out)
    return SceneDesc(tris, mats, cam, env=env, textures=texs, name=Path(str(scene_dir).rstrip("/")).name)


def camera_struct(c: dict) -> abi.Camera:
    return abi.Camera((C.c_float * 3)(*c["from_"]), (C.c_float * 3)(*c["to"]), (C.c_float * 3)(*c["up"]),
                      float(c["fov"]), int(c["width"]), int(c["height"]), int(c.get("flip_x", 0)))


class Scene:
    """Reference `Scene` (Scene.h:76-176) backed by a device context."""

    def __init__(self, ctx: Context | None = None):
        self.ctx = ctx or Context()
        self.desc: SceneDesc | None = None

    def init(self, desc: SceneDesc) -> None:
        """Scene::init: triangles, materials, background (env or black)."""
        self.desc = desc
        self.ctx.upload(desc)

    def build(self) -> None:
        """Scene::build: BVH (on the GPU) and the light list."""
        self.ctx.bvh_build()

    def traverse(self, rays: np.ndarray) -> np.ndarray:
        return self.ctx.trace_closest(rays)

    def visible(self, p1: np.ndarray, p2: np.ndarray) -> np.ndarray:
        """Scene::visible (Scene.h:139-146) for arrays of point pairs."""
        p1 = np.asarray(p1, np.float32).reshape(-1, 3)
        p2 = np.asarray(p2, np.float32).reshape(-1, 3)
        d = p2 - p1
        length = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]).astype(np.float32)
        maxt = (length - np.float32(2e-4)).astype(np.float32)
        dn = d * (np.float32(1.0) / length)[:, None]
        rays = np.zeros(len(p1), abi.RAY)
        rays["o"] = p1 + dn * np.float32(1e-4)
        rays["d"] = dn
        rays["tmax"] = maxt
        return self.ctx.trace_any(rays).astype(bool)


class RayTracer:
    """Reference `RayTracer` (Renderer.h:236-752): progressive film, one
    sample per pixel per `render()` call."""

    def __init__(self, mode: int = abi.MODE_PLAIN, seed: int = 1, max_depth: int = 8):
        self.mode = mode
        self.seed = seed
        self.max_depth = max_depth
        self.scene: Scene | None = None

    def init(self, scene: Scene) -> None:
        self.scene = scene
        self.clear()

    def clear(self) -> None:
        self.scene.ctx.clear()

    def render(self) -> None:
        self.scene.ctx.render(1, self.mode, self.seed, self.max_depth, record_paths=self.mode == abi.MODE_GUIDED_LI)

    def getSPP(self) -> int:  # noqa: N802 - reference name
        return self.scene.ctx.spp()

    def savePNG(self, filename: str) -> None:  # noqa: N802 - reference name
        """RayTracer::savePNG (Renderer.h:751): the tonemapped film as PNG."""
        write_png(filename, self.scene.ctx.tonemap())

    def saveHDR(self, filename: str) -> None:  # noqa: N802 - reference name
        """Film::save (Imaging.h:263-272): film / SPP as Radiance HDR."""
        rgb, _, spp = self.scene.ctx.film()
        img = rgb * (np.float32(1.0) / np.float32(spp) if spp > 0 else np.float32(1.0))
        write_hdr(filename, img)


def write_hdr(filename: str, img: np.ndarray) -> None:
    """Radiance RGBE writer.  Scanlines 8..32767 pixels wide are written in
    the run-length layout (one literal run per 128 bytes of each channel),
    which no reader can mistake for a flat scanline; other widths flat."""
    h, w, _ = img.shape
    rgb = np.asarray(img, np.float64)
    mx = rgb.max(axis=2)
    e = np.zeros_like(mx, dtype=np.int32)
    m = np.zeros_like(mx)
    nz = mx > 1e-32
    m[nz], e[nz] = np.frexp(mx[nz])
    scale = np.where(nz, m * 256.0 / np.where(nz, mx, 1.0), 0.0)
    out = np.zeros((h, w, 4), np.uint8)
    out[..., :3] = np.clip(rgb * scale[..., None], 0, 255).astype(np.uint8)
    out[..., 3] = np.where(nz, e + 128, 0).astype(np.uint8)
    with open(filename, "wb") as f:
        f.write(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n")
        f.write(f"-Y {h} +X {w}\n".encode())
        if not 8 <= w < 32768:
            f.write(out.tobytes())
            return
        head = bytes([2, 2, w >> 8, w & 255])
        runs = [(x, min(128, w - x)) for x in range(0, w, 128)]
        for y in range(h):
            parts = [head]
            for c in range(4):
                row = out[y, :, c].tobytes()
                for x, n in runs:
                    parts.append(bytes([n]) + row[x:x + n])
            f.write(b"".join(parts))


def write_png(filename: str, rgb8: np.ndarray) -> None:
    """8-bit RGB PNG (filter 0 on every row, zlib stream)."""
    import struct
    import zlib
    h, w, _ = rgb8.shape
    raw = b"".join(b"\x00" + np.ascontiguousarray(rgb8[y]).tobytes() for y in range(h))

    def chunk(tag: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    with open(filename, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))
