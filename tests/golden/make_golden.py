"""Regenerates the golden fixtures in this directory from the reference
itself (compiled headless by oracle/build.py).  Run here, where the reference
checkout exists:

    python tests/golden/make_golden.py

Each fixture stores its inputs (triangles, rays) next to the reference's
outputs, so the tests never regenerate inputs with a possibly different
numpy on another machine.

* render_<scene>.npz — scene inputs and the films of the reference's own
  integrators (`pathTrace`, `guidedPath`) driven by the PCG32 stream of
  (seed, pixel, sample) through oracle/ref_harness.cpp.
* bsdf_roundtrip.npz — per material: `BSDF::sample` driven by TestSampler and
  `BSDF::invert` (Materials.h:121-897) on random normals / outgoing
  directions.
* traversal_<scene>.npz — triangles; the reference's BVH (`BVHNode::build`,
  Geometry.h:419-446) as nodes + triangle indexes; rays; closest hits from
  `BVHNode::traverse` (Geometry.h:455-512); any-hit visibility from
  `BVHNode::traverseVisible` (Geometry.h:514-567) for rays clipped to
  0.5x and 1.5x the closest hit distance.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle.ffi import Reference  # noqa: E402
from pathguidingdissertation_gb300 import scenes  # noqa: E402


def traversal_fixture(ref: Reference, name: str, desc, nrays: int, seed: int) -> None:
    tris = desc.triangles
    nodes, idx = ref.bvh_build(tris)
    bmin, bmax = desc.bounds()
    rays = scenes.random_rays(bmin, bmax, nrays, seed=seed)
    world = ref.world(tris)
    hits, _ = world.trace_closest(rays)
    short = rays.copy()
    far = np.where(hits["id"] >= 0, hits["t"], np.float32(1.0))
    short["tmax"] = (far * np.float32(0.5)).astype(np.float32)
    longer = rays.copy()
    longer["tmax"] = (far * np.float32(1.5)).astype(np.float32)
    any_rays = np.concatenate([short, longer])
    vis, _ = world.trace_any(any_rays)
    world.close()
    np.savez_compressed(HERE / f"traversal_{name}.npz", triangles=tris, nodes=nodes, idx=idx, rays=rays, hits=hits,
                        any_rays=any_rays, visible=vis)
    print(f"traversal_{name}: {len(tris)} tris, {len(nodes)} nodes, {nrays} rays, "
          f"hit {np.mean(hits['id'] >= 0):.3f}, visible {vis.mean():.3f}")


def render_fixture(ref: Reference, name: str, desc, spp: int, seed: int) -> None:
    """Reference integrators (pathTrace and guidedPath, Renderer.h:368-613)
    driven by the PCG32 stream, `spp` samples per pixel."""
    rs = ref.scene(desc)
    plain, _, rays_p = rs.render_pcg(False, seed, 0, spp, threads=8)
    guided, _, rays_g = rs.render_pcg(True, seed, 0, spp, threads=8)
    rs.close()
    c = desc.camera
    env = desc.env if desc.env is not None else np.zeros((0, 0, 3), np.float32)
    np.savez_compressed(HERE / f"render_{name}.npz", triangles=desc.triangles, materials=desc.materials, env=env,
                        cam_from=np.array(c["from_"], np.float32), cam_to=np.array(c["to"], np.float32),
                        cam_up=np.array(c["up"], np.float32), cam_fov=np.float32(c["fov"]),
                        size=np.array([c["width"], c["height"]], np.int32), spp=np.int32(spp), seed=np.int64(seed),
                        plain=plain, guided=guided)
    print(f"render_{name}: {desc.ntris} tris, {c['width']}x{c['height']} x {spp} spp, "
          f"plain mean {plain.mean() / spp:.4f}, guided mean {guided.mean() / spp:.4f}")


BSDF_CASES = {
    # name: material keyword arguments (scenes.material)
    "conductor_runtest": dict(kind=2, albedo=(1, 1, 1), eta=(1.0, 0.6, 1.5), k=(0.65, 0.85, 1.0), roughness=0.5),
    "conductor_smooth": dict(kind=2, albedo=(0.9, 0.8, 0.7), eta=(0.2, 0.9, 1.1), k=(3.9, 2.4, 2.2), roughness=0.0),
    "diffuse": dict(kind=0, albedo=(0.6, 0.5, 0.4)),
    "mirror": dict(kind=1, albedo=(0.9, 0.9, 0.9)),
    "glass": dict(kind=3, albedo=(1, 1, 1), int_ior=1.5, ext_ior=1.0),
    "dielectric_rough": dict(kind=4, albedo=(1, 1, 1), int_ior=1.5, ext_ior=1.0, roughness=0.3),
    "orennayar": dict(kind=5, albedo=(0.7, 0.6, 0.5), sigma=0.5),
    "plastic": dict(kind=6, albedo=(0.3, 0.5, 0.7), int_ior=1.5, ext_ior=1.0, roughness=0.2),
}


def bsdf_fixture(ref: Reference, count: int = 800, seed: int = 21) -> None:
    """BSDF::sample with TestSampler and BSDF::invert (Materials.h) per
    material, for random normals and outgoing directions (some below the
    surface, to exercise the two-sided and transmission branches)."""
    rng = np.random.default_rng(seed)
    out = {}
    for name, kw in BSDF_CASES.items():
        n = rng.normal(size=(count, 3))
        n /= np.linalg.norm(n, axis=1, keepdims=True)
        wo = rng.normal(size=(count, 3))
        wo /= np.linalg.norm(wo, axis=1, keepdims=True)
        flip = np.einsum("ij,ij->i", n, wo) < 0
        flip[: count // 5] = False  # keep a fifth below the surface
        wo[flip] = -wo[flip]
        uv = rng.random((count, 2))
        n, wo, uv = n.astype(np.float32), wo.astype(np.float32), uv.astype(np.float32)
        mat = scenes.material(**kw)
        wi, f, pdf, uv_out = ref.bsdf_roundtrip(mat, n, wo, uv)
        for k, v in dict(material=mat, n=n, wo=wo, uv=uv, wi=wi, f=f, pdf=pdf, uv_out=uv_out).items():
            out[f"{name}__{k}"] = v
    np.savez_compressed(HERE / "bsdf_roundtrip.npz", **out)
    print(f"bsdf_roundtrip: {len(BSDF_CASES)} materials x {count} samples")


def main() -> None:
    ref = Reference()
    bsdf_fixture(ref)
    render_fixture(ref, "cornell", scenes.cornell_box(seed=1, width=32, height=32), 4, seed=11)
    render_fixture(ref, "interior", scenes.interior(seed=5, target_tris=3000, n_objects=24, width=48, height=27,
                                                    env_width=64, env_height=32), 4, seed=12)
    traversal_fixture(ref, "cornell", scenes.cornell_box(seed=1), 2000, seed=101)
    traversal_fixture(ref, "soup", scenes.triangle_soup(1500, seed=11), 2000, seed=102)
    traversal_fixture(ref, "interior", scenes.interior(seed=5, target_tris=3000, n_objects=24, env_width=8,
                                                       env_height=4), 2000, seed=103)


if __name__ == "__main__":
    main()
