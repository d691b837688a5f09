"""Seeded procedural scenes for the workloads the renderer is measured on.

* ``cornell_box`` — the plain-path-tracing box: a 2x2x2 five-wall box open at
  the front (10 triangles), two yawed inner boxes (12 triangles each, size
  U[0.4, 0.9], yaw U[0, 90 deg]), a 0.5x0.5 ceiling light (2 triangles,
  radiance 17), Lambert albedos U[0.1, 0.8]^3, 40 deg pinhole camera.
* ``interior`` — the guided-rendering interior: an 8x4x6 room with a 1.5x1
  window portal, boxes and UV-spheres with log-normal sizes (mu=-1,
  sigma=0.5) tessellated to a triangle budget (200k by default), 40 % Lambert,
  40 % GGX conductor (roughness U[0.05, 0.5], F0 U[0.5, 1]), 20 % smooth
  dielectric (IOR 1.5), and an HDR sky (gradient + Gaussian sun lobe,
  sigma = 1 deg, peak 5e4) that reaches the room through the window.
* ``triangle_soup`` / ``random_rays`` — inputs for traversal checks.

Conductors are specified by F0; the reference's conductor takes (eta, k)
(Materials.h:245-250), so F0 maps to k = 0 and eta = (1 + sqrt(F0)) /
(1 - sqrt(F0)), for which the reference's Fresnel term (Materials.h:63-90)
gives reflectance F0 at normal incidence.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .abi import (BSDF_CONDUCTOR, BSDF_DIELECTRIC, BSDF_DIFFUSE, BSDF_GLASS, BSDF_MIRROR, BSDF_ORENNAYAR,
                  BSDF_PLASTIC, MATERIAL, RAY, TRIANGLE)


@dataclass
class SceneDesc:
    triangles: np.ndarray                 # TRIANGLE
    materials: np.ndarray                 # MATERIAL
    camera: dict                          # from, to, up, fov, width, height
    env: np.ndarray | None = None         # (H, W, 3) float32, row 0 = top (theta = 0)
    textures: list = field(default_factory=list)  # list of (H, W, 3) float32
    name: str = "scene"

    @property
    def ntris(self) -> int:
        return int(self.triangles.shape[0])

    def bounds(self) -> tuple[np.ndarray, np.ndarray]:
        p = self.triangles["v"]["p"].reshape(-1, 3)
        return p.min(axis=0), p.max(axis=0)


def material(kind=BSDF_DIFFUSE, albedo=(0.8, 0.8, 0.8), emission=(0, 0, 0), roughness=0.0, eta=(1.5, 1.5, 1.5),
             k=(0, 0, 0), int_ior=1.5, ext_ior=1.0, sigma=0.0, texture=-1, layered=0) -> np.ndarray:
    m = np.zeros((), MATERIAL)
    m["kind"] = kind
    m["albedo_texture"] = texture
    m["albedo"] = albedo
    m["eta"] = eta
    m["k"] = k
    m["int_ior"] = int_ior
    m["ext_ior"] = ext_ior
    m["roughness"] = roughness
    m["sigma"] = sigma
    m["emission"] = emission
    m["layered"] = layered
    return m


def conductor_from_f0(f0: float, roughness: float) -> np.ndarray:
    s = math.sqrt(min(f0, 0.999))
    eta = (1.0 + s) / (1.0 - s)
    return material(BSDF_CONDUCTOR, albedo=(1, 1, 1), roughness=roughness, eta=(eta, eta, eta), k=(0, 0, 0))


class MeshBuilder:
    """Accumulates triangles with per-vertex normals and uvs."""

    def __init__(self):
        self.p: list[np.ndarray] = []
        self.n: list[np.ndarray] = []
        self.uv: list[np.ndarray] = []
        self.mat: list[np.ndarray] = []

    def add(self, p: np.ndarray, n: np.ndarray, uv: np.ndarray, mat: int) -> None:
        """p, n: (T, 3, 3); uv: (T, 3, 2)."""
        self.p.append(np.asarray(p, np.float32))
        self.n.append(np.asarray(n, np.float32))
        self.uv.append(np.asarray(uv, np.float32))
        self.mat.append(np.full(len(p), mat, np.uint32))

    def quad_grid(self, origin, du, dv, normal, res: int, mat: int) -> None:
        """Planar quad origin + s*du + t*dv, split into res x res cells."""
        origin, du, dv = (np.asarray(x, np.float64) for x in (origin, du, dv))
        s = np.linspace(0.0, 1.0, res + 1)
        i, j = np.meshgrid(np.arange(res), np.arange(res), indexing="ij")
        i = i.ravel()
        j = j.ravel()
        s0, s1, t0, t1 = s[i], s[i + 1], s[j], s[j + 1]

        def pt(a, b):
            return origin + a[:, None] * du + b[:, None] * dv

        c00, c10, c01, c11 = pt(s0, t0), pt(s1, t0), pt(s0, t1), pt(s1, t1)
        tris = np.stack([np.stack([c00, c10, c11], 1), np.stack([c00, c11, c01], 1)], 1).reshape(-1, 3, 3)
        uv = np.stack([np.stack([np.stack([s0, t0], -1), np.stack([s1, t0], -1), np.stack([s1, t1], -1)], 1),
                       np.stack([np.stack([s0, t0], -1), np.stack([s1, t1], -1), np.stack([s0, t1], -1)], 1)],
                      1).reshape(-1, 3, 2)
        # Orient the winding so the face normal agrees with `normal`.
        fn = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0])
        flip = (fn @ np.asarray(normal, np.float64)) < 0
        tris[flip] = tris[flip][:, [0, 2, 1]]
        uv[flip] = uv[flip][:, [0, 2, 1]]
        nrm = np.broadcast_to(np.asarray(normal, np.float64), tris.shape)
        self.add(tris, nrm, uv, mat)

    def box(self, centre, size, yaw: float, mat: int, res: int = 1, inward: bool = False) -> None:
        """Box rotated by `yaw` about +y; faces split into res x res cells."""
        c = np.asarray(centre, np.float64)
        h = np.asarray(size, np.float64) * 0.5
        cy, sy = math.cos(yaw), math.sin(yaw)
        R = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
        sgn = -1.0 if inward else 1.0
        for axis in range(3):
            for side in (-1.0, 1.0):
                n = np.zeros(3)
                n[axis] = side
                u_ax, v_ax = [a for a in range(3) if a != axis]
                du = np.zeros(3)
                dv = np.zeros(3)
                du[u_ax] = 2 * h[u_ax]
                dv[v_ax] = 2 * h[v_ax]
                o = -h.copy()
                o[axis] = side * h[axis]
                self.quad_grid(c + R @ o, R @ du, R @ dv, sgn * (R @ n), res, mat)

    def sphere(self, centre, radius: float, slices: int, stacks: int, mat: int) -> None:
        """UV sphere: 2 * slices * (stacks - 1) triangles, smooth normals."""
        c = np.asarray(centre, np.float64)
        th = np.linspace(0, math.pi, stacks + 1)
        ph = np.linspace(0, 2 * math.pi, slices + 1)
        T, P = np.meshgrid(th, ph, indexing="ij")
        dirs = np.stack([np.sin(T) * np.cos(P), np.cos(T), np.sin(T) * np.sin(P)], -1)
        pts = c + radius * dirs
        uvg = np.stack([P / (2 * math.pi), T / math.pi], -1)
        i, j = np.meshgrid(np.arange(stacks), np.arange(slices), indexing="ij")
        i = i.ravel()
        j = j.ravel()
        upper = i != 0            # triangle (a, d, c) exists below the north cap row
        lower = i != stacks - 1   # triangle (a, c, b) exists above the south cap row
        quads = [((i, j), (i, j + 1), (i + 1, j + 1), upper), ((i, j), (i + 1, j + 1), (i + 1, j), lower)]
        tris, nrms, uvs = [], [], []
        for a, b, cc, keep in quads:
            idx = [(x[0][keep], x[1][keep]) for x in (a, b, cc)]
            tris.append(np.stack([pts[x] for x in idx], 1))
            nrms.append(np.stack([dirs[x] for x in idx], 1))
            uvs.append(np.stack([uvg[x] for x in idx], 1))
        tris = np.concatenate(tris)
        nrms = np.concatenate(nrms)
        uvs = np.concatenate(uvs)
        fn = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0])
        flip = np.einsum("ij,ij->i", fn, nrms[:, 0]) < 0
        tris[flip] = tris[flip][:, [0, 2, 1]]
        nrms[flip] = nrms[flip][:, [0, 2, 1]]
        uvs[flip] = uvs[flip][:, [0, 2, 1]]
        self.add(tris, nrms, uvs, mat)

    def triangles(self) -> np.ndarray:
        p = np.concatenate(self.p)
        n = np.concatenate(self.n)
        uv = np.concatenate(self.uv)
        out = np.zeros(len(p), TRIANGLE)
        out["v"]["p"] = p
        out["v"]["n"] = n
        out["v"]["u"] = uv[..., 0]
        out["v"]["v"] = uv[..., 1]
        out["material"] = np.concatenate(self.mat)
        return out


def cornell_box(seed: int = 1, width: int = 256, height: int = 256, target_tris: int | None = None) -> SceneDesc:
    """The plain path-tracing configuration (36 triangles).  With
    `target_tris`, walls and boxes are tessellated into res x res cells
    (34 res^2 + 2 triangles, res = round(sqrt((target - 2) / 34))); the
    geometry and the light stay the same."""
    rng = np.random.default_rng(seed)
    mb = MeshBuilder()
    mats = []
    res = 1 if target_tris is None else max(1, int(round(math.sqrt(max(target_tris - 2, 34) / 34.0))))

    def lambert():
        mats.append(material(BSDF_DIFFUSE, albedo=tuple(rng.uniform(0.1, 0.8, 3))))
        return len(mats) - 1

    # Five walls of the box [-1,1] x [0,2] x [-1,1], open towards +z, normals inward.
    mb.quad_grid((-1, 0, -1), (2, 0, 0), (0, 0, 2), (0, 1, 0), res, lambert())       # floor
    mb.quad_grid((-1, 2, -1), (2, 0, 0), (0, 0, 2), (0, -1, 0), res, lambert())      # ceiling
    mb.quad_grid((-1, 0, -1), (2, 0, 0), (0, 2, 0), (0, 0, 1), res, lambert())       # back
    mb.quad_grid((-1, 0, -1), (0, 0, 2), (0, 2, 0), (1, 0, 0), res, lambert())       # left
    mb.quad_grid((1, 0, -1), (0, 0, 2), (0, 2, 0), (-1, 0, 0), res, lambert())       # right
    for cx, cz in ((-0.4, -0.3), (0.4, 0.35)):
        s = rng.uniform(0.4, 0.9)
        yaw = math.radians(rng.uniform(0.0, 90.0))
        mb.box((cx, s * 0.5, cz), (s, s, s), yaw, lambert(), res=res)
    mats.append(material(BSDF_DIFFUSE, albedo=(0.0, 0.0, 0.0), emission=(17.0, 17.0, 17.0)))
    mb.quad_grid((-0.25, 1.999, -0.25), (0.5, 0, 0), (0, 0, 0.5), (0, -1, 0), 1, len(mats) - 1)
    cam = dict(from_=(0.0, 1.0, 3.8), to=(0.0, 1.0, 0.0), up=(0.0, 1.0, 0.0), fov=40.0, width=width, height=height)
    return SceneDesc(mb.triangles(), np.array(mats, MATERIAL), cam, name="cornell_box")


def material_zoo(seed: int = 1, width: int = 64, height: int = 64, env: bool = False) -> SceneDesc:
    """The Cornell box with a box of every further BSDF kind on its floor:
    mirror, rough plastic, rough dielectric, Oren-Nayar, smooth and rough
    conductor, layered diffuse (LayeredBSDF) and glass; with `env`, a sky and
    sun environment map lights it as well."""
    base = cornell_box(seed=seed, width=width, height=height)
    rng = np.random.default_rng(seed + 100)
    mb = MeshBuilder()
    mats = list(base.materials)
    kinds = [material(BSDF_MIRROR, albedo=(0.9, 0.9, 0.9)),
             material(BSDF_PLASTIC, albedo=(0.2, 0.5, 0.8), roughness=0.3, int_ior=1.5, ext_ior=1.0),
             material(BSDF_DIELECTRIC, albedo=(1, 1, 1), roughness=0.2, int_ior=1.45, ext_ior=1.0),
             material(BSDF_ORENNAYAR, albedo=(0.7, 0.4, 0.3), sigma=0.6),
             conductor_from_f0(0.9, 0.0),
             conductor_from_f0(0.7, 0.35),
             material(BSDF_DIFFUSE, albedo=(0.5, 0.7, 0.3), layered=1),
             material(BSDF_GLASS, albedo=(1, 1, 1), int_ior=1.5, ext_ior=1.0)]
    for i, m in enumerate(kinds):
        mats.append(m)
        cx, cz = -0.7 + 0.2 * i, 0.55 - 0.12 * (i % 3)
        s = rng.uniform(0.12, 0.18)
        mb.box((cx, s * 0.5 + 0.001, cz), (s, s, s), math.radians(rng.uniform(0.0, 90.0)), len(mats) - 1)
    tris = np.concatenate([base.triangles, mb.triangles()])
    envmap = sky_envmap(64, 32) if env else None
    return SceneDesc(tris, np.array(mats, MATERIAL), base.camera, env=envmap, name="material_zoo")


def sky_envmap(width: int = 2048, height: int = 1024, sun_dir=(0.8, 0.45, 0.25), sun_sigma_deg: float = 1.0,
               sun_peak: float = 5e4) -> np.ndarray:
    """Lat-long HDR sky in the reference's convention (Lights.h:148-178):
    u = atan2(z, x) / 2pi, v = acos(y) / pi, texel (u, v) at column u*W, row v*H."""
    v = (np.arange(height) + 0.5) / height
    u = (np.arange(width) + 0.5) / width
    theta = math.pi * v[:, None]
    phi = 2 * math.pi * u[None, :]
    d = np.stack([np.cos(phi) * np.sin(theta), np.cos(theta) * np.ones_like(phi), np.sin(phi) * np.sin(theta)], -1)
    y = d[..., 1]
    zen = np.array([0.35, 0.55, 1.0])
    hor = np.array([0.95, 0.9, 0.85])
    t = np.clip(y, 0.0, 1.0)[..., None]
    sky = (1 - t) * hor + t * zen
    ground = np.array([0.18, 0.16, 0.14])
    rgb = np.where((y >= 0)[..., None], sky * 2.0, ground * (1.0 + y[..., None]))
    s = np.asarray(sun_dir, np.float64)
    s = s / np.linalg.norm(s)
    ang = np.arccos(np.clip(d @ s, -1.0, 1.0))
    sig = math.radians(sun_sigma_deg)
    sun = sun_peak * np.exp(-0.5 * (ang / sig) ** 2)
    rgb = rgb + sun[..., None] * np.array([1.0, 0.95, 0.85])
    return rgb.astype(np.float32)


def interior(seed: int = 2, target_tris: int = 200_000, n_objects: int = 400, width: int = 1280, height: int = 720,
             env_width: int = 2048, env_height: int = 1024) -> SceneDesc:
    """The guided-rendering interior (room 8x4x6, window 1.5x1, furniture)."""
    rng = np.random.default_rng(seed)
    mb = MeshBuilder()
    mats = []

    def add_mat(m):
        mats.append(m)
        return len(mats) - 1

    wall = add_mat(material(BSDF_DIFFUSE, albedo=(0.7, 0.68, 0.65)))
    floor = add_mat(material(BSDF_DIFFUSE, albedo=(0.45, 0.35, 0.25)))
    ceil = add_mat(material(BSDF_DIFFUSE, albedo=(0.8, 0.8, 0.8)))
    X, Y, Z = 4.0, 4.0, 3.0
    mb.quad_grid((-X, 0, -Z), (2 * X, 0, 0), (0, 0, 2 * Z), (0, 1, 0), 4, floor)
    mb.quad_grid((-X, Y, -Z), (2 * X, 0, 0), (0, 0, 2 * Z), (0, -1, 0), 4, ceil)
    mb.quad_grid((-X, 0, -Z), (2 * X, 0, 0), (0, Y, 0), (0, 0, 1), 4, wall)
    mb.quad_grid((-X, 0, Z), (2 * X, 0, 0), (0, Y, 0), (0, 0, -1), 4, wall)
    mb.quad_grid((-X, 0, -Z), (0, 0, 2 * Z), (0, Y, 0), (1, 0, 0), 4, wall)
    # +x wall with a 1.5 (z) x 1 (y) window centred at z = 0, y = 2.4.
    wz0, wz1, wy0, wy1 = -0.75, 0.75, 1.9, 2.9
    for (z0, z1, y0, y1) in ((-Z, wz0, 0, Y), (wz1, Z, 0, Y), (wz0, wz1, 0, wy0), (wz0, wz1, wy1, Y)):
        mb.quad_grid((X, y0, z0), (0, 0, z1 - z0), (0, y1 - y0, 0), (-1, 0, 0), 2, wall)
    base_tris = sum(len(p) for p in mb.p)

    # Furniture: half boxes, half spheres, tessellated to the triangle budget
    # (a box has 12 res^2 triangles, a sphere 2 slices (stacks - 1)).
    n_box = (n_objects + 1) // 2
    n_sph = n_objects // 2
    per_obj = max(12.0, (target_tris - base_tris) / max(n_objects, 1))
    box_res = max(1, int(round(math.sqrt(per_obj / 12.0))))
    rest = max(4.0, (target_tris - base_tris - n_box * 12 * box_res * box_res) / max(n_sph, 1))
    sphere_slices = max(4, int(round(math.sqrt(rest))))
    sphere_stacks = max(3, int(round(rest / (2.0 * sphere_slices))) + 1)
    kinds = rng.choice(3, size=n_objects, p=[0.4, 0.4, 0.2])
    sizes = np.exp(rng.normal(-1.0, 0.5, n_objects))
    for i in range(n_objects):
        if kinds[i] == 0:
            m = add_mat(material(BSDF_DIFFUSE, albedo=tuple(rng.uniform(0.1, 0.8, 3))))
        elif kinds[i] == 1:
            m = add_mat(conductor_from_f0(rng.uniform(0.5, 1.0), rng.uniform(0.05, 0.5)))
        else:
            m = add_mat(material(BSDF_GLASS, albedo=(1, 1, 1), int_ior=1.5, ext_ior=1.0))
        s = float(min(sizes[i], 1.5))
        x = rng.uniform(-X + s, X - s)
        z = rng.uniform(-Z + s, Z - s)
        y = s * 0.5 + rng.uniform(0.0, 0.3) * (rng.uniform() < 0.3) * (Y - s)
        if i % 2 == 0:
            dims = s * rng.uniform(0.5, 1.0, 3)
            mb.box((x, dims[1] * 0.5 + y - s * 0.5, z), dims, rng.uniform(0, math.pi / 2), m, res=box_res)
        else:
            mb.sphere((x, y, z), s * 0.5, sphere_slices, sphere_stacks, m)
    env = sky_envmap(env_width, env_height)
    cam = dict(from_=(-3.6, 1.7, 2.6), to=(1.5, 1.3, -1.2), up=(0.0, 1.0, 0.0), fov=60.0, width=width, height=height)
    return SceneDesc(mb.triangles(), np.array(mats, MATERIAL), cam, env=env, name="interior")


def fbm(n: int, seed: int, octaves: int = 6, lacunarity: float = 2.0, gain: float = 0.5, base: int = 4) -> np.ndarray:
    """Fractional Brownian motion of value noise on an n x n grid over [0,1]^2:
    sum over octaves o of gain^o * noise(base * lacunarity^o * x), each noise a
    random lattice smoothly (smoothstep) interpolated.  Values ~ [-1, 1]."""
    rng = np.random.default_rng(seed)
    x = np.linspace(0.0, 1.0, n)
    h = np.zeros((n, n))
    amp, freq, norm = 1.0, float(base), 0.0
    for _ in range(octaves):
        m = int(math.ceil(freq)) + 2
        lat = rng.uniform(-1.0, 1.0, (m, m))
        t = x * freq
        i = np.floor(t).astype(np.int64)
        f = t - i
        f = f * f * (3.0 - 2.0 * f)
        a = lat[i[:, None], i[None, :]]
        b = lat[i[:, None], i[None, :] + 1]
        c = lat[i[:, None] + 1, i[None, :]]
        d = lat[i[:, None] + 1, i[None, :] + 1]
        fy, fx = f[:, None], f[None, :]
        h += amp * ((a * (1 - fx) + b * fx) * (1 - fy) + (c * (1 - fx) + d * fx) * fy)
        norm += amp
        amp *= gain
        freq *= lacunarity
    return h / norm


def terrain(grid: int = 1024, seed: int = 4, n_materials: int = 32, width: int = 512, height: int = 512,
            env_width: int = 512, env_height: int = 256, height_scale: float = 0.35, sun_peak: float = 60.0) -> SceneDesc:
    """The differentiable-rendering heightfield: a grid x grid vertex
    heightfield over [-1,1]^2 (2 (grid-1)^2 triangles) with fBm heights (6
    octaves, lacunarity 2, gain 0.5), `n_materials` GGX conductor materials
    (albedo U[0.1,0.8]^3, roughness U[0.05,0.5], F0 U[0.5,1]) assigned by
    height band, lit only by a sky environment map."""
    rng = np.random.default_rng(seed)
    hgt = fbm(grid, seed + 1) * height_scale
    xs = np.linspace(-1.0, 1.0, grid)
    X, Z = np.meshgrid(xs, xs, indexing="xy")
    P = np.stack([X, hgt, Z], -1)
    # vertex normals from central differences of the height
    gx = np.gradient(hgt, xs, axis=1)
    gz = np.gradient(hgt, xs, axis=0)
    Nrm = np.stack([-gx, np.ones_like(hgt), -gz], -1)
    Nrm /= np.linalg.norm(Nrm, axis=-1, keepdims=True)
    UV = np.stack([(X + 1) * 0.5, (Z + 1) * 0.5], -1)
    i, j = np.meshgrid(np.arange(grid - 1), np.arange(grid - 1), indexing="ij")
    v00 = (i * grid + j).ravel()
    v01 = v00 + 1
    v10 = v00 + grid
    v11 = v10 + 1
    tri_idx = np.concatenate([np.stack([v00, v10, v11], 1), np.stack([v00, v11, v01], 1)])
    Pf, Nf, UVf = P.reshape(-1, 3), Nrm.reshape(-1, 3), UV.reshape(-1, 2)
    t = np.zeros(len(tri_idx), TRIANGLE)
    t["v"]["p"] = Pf[tri_idx]
    t["v"]["n"] = Nf[tri_idx]
    t["v"]["u"] = UVf[tri_idx, 0]
    t["v"]["v"] = UVf[tri_idx, 1]
    centre_h = Pf[tri_idx][:, :, 1].mean(axis=1)
    lo, hi = hgt.min(), hgt.max()
    band = np.clip(((centre_h - lo) / max(hi - lo, 1e-9) * n_materials).astype(np.int64), 0, n_materials - 1)
    t["material"] = band
    mats = []
    for _ in range(n_materials):
        m = conductor_from_f0(rng.uniform(0.5, 1.0), rng.uniform(0.05, 0.5))
        m["albedo"] = rng.uniform(0.1, 0.8, 3)
        mats.append(m)
    cam = dict(from_=(0.0, 1.25, 2.1), to=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), fov=45.0, width=width, height=height)
    env = sky_envmap(env_width, env_height, sun_dir=(0.5, 0.6, -0.4), sun_sigma_deg=4.0, sun_peak=sun_peak)
    return SceneDesc(t, np.array(mats, MATERIAL), cam, env=env, name="terrain")


def triangle_soup(n: int, seed: int = 0, extent: float = 10.0, size: float = 0.5) -> SceneDesc:
    """n random triangles in a cube, for traversal checks."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-extent, extent, (n, 1, 3))
    p = c + rng.normal(0.0, size, (n, 3, 3))
    out = np.zeros(n, TRIANGLE)
    out["v"]["p"] = p.astype(np.float32)
    nrm = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-20)
    out["v"]["n"] = np.repeat(nrm[:, None, :], 3, axis=1).astype(np.float32)
    mats = np.array([material()], MATERIAL)
    cam = dict(from_=(0.0, 0.0, 3 * extent), to=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), fov=45.0, width=64, height=64)
    return SceneDesc(out, mats, cam, name=f"soup{n}")


def random_rays(bmin, bmax, n: int, seed: int = 7, inset: float = 0.9) -> np.ndarray:
    """Rays with origins uniform in the central `inset` fraction of the box
    and uniformly distributed unit directions; tmax = FLT_MAX."""
    rng = np.random.default_rng(seed)
    bmin = np.asarray(bmin, np.float64)
    bmax = np.asarray(bmax, np.float64)
    c = 0.5 * (bmin + bmax)
    h = 0.5 * (bmax - bmin) * inset
    o = rng.uniform(c - h, c + h, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros(n, RAY)
    r["o"] = o.astype(np.float32)
    r["d"] = d.astype(np.float32)
    r["tmax"] = np.finfo(np.float32).max
    return r
