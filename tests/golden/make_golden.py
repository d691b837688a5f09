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


def main() -> None:
    ref = Reference()
    render_fixture(ref, "cornell", scenes.cornell_box(seed=1, width=32, height=32), 4, seed=11)
    render_fixture(ref, "interior", scenes.interior(seed=5, target_tris=3000, n_objects=24, width=48, height=27,
                                                    env_width=64, env_height=32), 4, seed=12)
    traversal_fixture(ref, "cornell", scenes.cornell_box(seed=1), 2000, seed=101)
    traversal_fixture(ref, "soup", scenes.triangle_soup(1500, seed=11), 2000, seed=102)
    traversal_fixture(ref, "interior", scenes.interior(seed=5, target_tris=3000, n_objects=24, env_width=8,
                                                       env_height=4), 2000, seed=103)


if __name__ == "__main__":
    main()
