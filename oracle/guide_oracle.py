"""CPU restatement of the QuadTree directional guide — TEST INFRASTRUCTURE.

Used only by tests/ as the checker of pgx's QuadTree guide (libpgx's
k_quadtree / quad_pdf / quad_sample / guide_region_root).  The reference
has no working guide: its QuadTree.h:24-174 stores points over (u, v) with
`insert`/`search` only, and its subdivision test (QuadTree.h:79) is always
true, so nothing of it can be pinned by running it.  This module restates
the published method pgx follows instead:

* Müller, Gross, Novák, "Practical Path Guiding for Efficient Light-Transport
  Simulation" (EGSR 2017), §3-4: a directional quadtree per spatial region
  over a cylindrical equal-area map of the sphere, built from radiance
  records whose flux estimates Li |cos| (the renderer's weight Lum(Li) |cos| /
  pdf; the luminance of Li for records without one); a cell is subdivided while it
  holds more than a fraction rho = 1 % of the region's flux; the pdf is the
  product of 4 x (child flux / cell flux) along the descent; sampling picks
  children in proportion to flux and maps the remaining uniforms into the
  leaf.
* With the reference's conventions: luminance weights of Colour::Lum
  (MyMath.h:60-62), the shading frame of Frame::fromVector
  (MyMath.h:412-423) and the cosine sampler's inverse of
  DiffuseBSDF::invert (Materials.h:163-171) for trees over the BSDF's
  primary samples (the reference's intended design, Renderer.h:403-414).
* pgx's own bounds (pgx_guide_params; defaults in brackets): spatial
  regions are the point-BVH subtrees (the reference's PointBVHNode,
  Renderer.h:71-234) whose record count first drops to region_records
  [1,024]; records are clamped at clamp_median [10] x the region's median
  positive luminance (the median found by 24 bisection steps on the value;
  0 = no clamp); cells are refined at refine_fraction [rho = 1 %]; at most
  256 cells per region and depth 10; a child is only refined when it holds
  at least 2 records; optionally MIS compensation of the leaves (Karlík et
  al. 2019) [off]; the guide mixes the tree with a uniform share [20 %].

Decisions (median, membership of a record in a cell) use float32 arithmetic
in the kernel's operation order so that the trees come out node for node the
same; flux sums, pdfs and sampled positions are float64.
"""
from __future__ import annotations

import numpy as np

REGION_MAX = 1024
CLAMP_MEDIAN = np.float32(10.0)
MAX_NODES = 256
MAX_DEPTH = 10
RHO = 0.01
UNIFORM = 0.2
ONE_MINUS = np.float32(0.99999994)
F = np.float32
PI_F = F(3.14159265)


def luminance(li: np.ndarray) -> np.ndarray:
    """Colour::Lum (MyMath.h:60-62) in float32, non-finite or non-positive -> 0."""
    li = np.asarray(li, F)
    w = (F(0.2126) * li[:, 0] + F(0.7152) * li[:, 1]) + F(0.0722) * li[:, 2]
    with np.errstate(invalid="ignore"):
        ok = np.isfinite(w) & (w > 0)
    return np.where(ok, w, F(0.0)).astype(F)


def dir_to_uv(w: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(u, v) = ((cos theta + 1) / 2, (phi + pi) / 2 pi), theta from +z, in
    the half-open unit square."""
    w = np.asarray(w, F).reshape(-1, 3)
    c = np.clip(w[:, 2], F(-1), F(1))
    u = (c + F(1)) * F(0.5)
    phi = np.arctan2(w[:, 1], w[:, 0]).astype(F)
    v = (phi + PI_F) * (F(1) / (F(2) * PI_F))
    return np.clip(u, F(0), ONE_MINUS), np.clip(v, F(0), ONE_MINUS)


def uv_to_dir(u, v) -> np.ndarray:
    u = np.asarray(u, np.float64)
    v = np.asarray(v, np.float64)
    c = 2.0 * u - 1.0
    s = np.sqrt(np.maximum(0.0, 1.0 - c * c))
    phi = 2.0 * np.pi * v - np.pi
    return np.stack([s * np.cos(phi), s * np.sin(phi), c], axis=-1)


def _frame(n: np.ndarray):
    """Frame::fromVector (MyMath.h:412-423) in float32."""
    n = np.asarray(n, F)
    inv = F(1) / np.sqrt((n[:, 0] * n[:, 0] + n[:, 1] * n[:, 1]) + n[:, 2] * n[:, 2])
    w = n * inv[:, None]
    a = np.abs(w[:, 0]) > np.abs(w[:, 1])
    la = F(1) / np.sqrt(w[:, 0] * w[:, 0] + w[:, 2] * w[:, 2])
    lb = F(1) / np.sqrt(w[:, 1] * w[:, 1] + w[:, 2] * w[:, 2])
    z = np.zeros(len(w), F)
    ua = np.stack([w[:, 2] * la, z, -w[:, 0] * la], 1)
    ub = np.stack([z, w[:, 2] * lb, -w[:, 1] * lb], 1)
    u = np.where(a[:, None], ua, ub)
    v = np.stack([w[:, 1] * u[:, 2] - w[:, 2] * u[:, 1], w[:, 2] * u[:, 0] - w[:, 0] * u[:, 2],
                  w[:, 0] * u[:, 1] - w[:, 1] * u[:, 0]], 1)
    return u, v, w


def _dot(a, b):
    return (a[:, 0] * b[:, 0] + a[:, 1] * b[:, 1]) + a[:, 2] * b[:, 2]


def pss_uv(normal: np.ndarray, wi: np.ndarray) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Primary sample of the cosine sampler that maps to wi about the
    shading normal (DiffuseBSDF::invert, Materials.h:163-171): u = cos^2
    theta, v = phi / 2 pi; valid where wi is above the hemisphere."""
    wi = np.asarray(wi, F)
    fu, fv, fw = _frame(normal)
    ok = _dot(wi, fw) > 0
    lx, ly, lz = _dot(wi, fu), _dot(wi, fv), _dot(wi, fw)
    theta = np.arccos(np.clip(lz, F(-1), F(1))).astype(F)
    phi = np.arctan2(ly, lx).astype(F)
    phi = np.where(phi < 0, phi + F(2.0 * np.pi), phi).astype(F)
    c = np.cos(theta).astype(F)
    u = c * c
    v = phi * F(0.159154943091895335769)
    return np.clip(u, F(0), ONE_MINUS), np.clip(v, F(0), ONE_MINUS), ok


def subtree_ranges(nodes: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(first record, record count) of every node's subtree, from the leaves'
    ranges (records are in leaf order, so a subtree's records are contiguous)."""
    n = len(nodes)
    first = np.zeros(n, np.int64)
    count = np.zeros(n, np.int64)
    order, stack = [], [0]
    while stack:
        i = stack.pop()
        order.append(i)
        if nodes[i]["left"] >= 0:
            stack += [int(nodes[i]["left"]), int(nodes[i]["right"])]
    for i in reversed(order):
        nd = nodes[i]
        if nd["left"] < 0:
            first[i], count[i] = int(nd["offset"]), int(nd["used"])
        else:
            a, b = int(nd["left"]), int(nd["right"])
            first[i] = min(first[a], first[b])
            count[i] = count[a] + count[b]
    return first, count


def regions_from_bvh(nodes: np.ndarray, n_records: int,
                     region_max: int = REGION_MAX) -> list[tuple[int, int, int]]:
    """(first, count, node) of every region, in record order: the subtrees
    whose record count first drops to region_max (the root when the cache
    holds at most that many records)."""
    if n_records == 0 or len(nodes) == 0:
        return []
    if n_records <= region_max:
        return [(0, n_records, 0)]
    first, count = subtree_ranges(nodes)
    out = []
    stack = [0]
    while stack:
        i = stack.pop()
        if nodes[i]["left"] < 0:
            continue  # a leaf of a region above the bound cannot exist (leaves hold <= 8)
        for c in (int(nodes[i]["left"]), int(nodes[i]["right"])):
            if count[c] <= region_max:
                out.append((int(first[c]), int(count[c]), c))
            else:
                stack.append(c)
    return sorted(out)


def median_bisection(w: np.ndarray) -> F:
    """Upper end of 24 bisection steps on the value towards the median of
    the positive weights (float32, as the kernel does)."""
    pos = w[w > 0]
    lo, hi = F(pos.min()), F(pos.max())
    half = (len(pos) + 1) // 2
    for _ in range(24):
        mid = F(F(0.5) * F(lo + hi))
        if int(np.count_nonzero(pos <= mid)) >= half:
            hi = mid
        else:
            lo = mid
    return hi


def flux_weights(w) -> np.ndarray:
    """Given per-record flux weights, float32, non-finite or non-positive -> 0."""
    w = np.asarray(w, F)
    with np.errstate(invalid="ignore"):
        ok = np.isfinite(w) & (w > 0)
    return np.where(ok, w, F(0.0)).astype(F)


def compensate_tree(tree, alpha: float):
    """MIS compensation (Karlík, Šik, Vévoda, Skřivan, Křivánek, "MIS
    compensation: optimizing sampling techniques in multiple importance
    sampling", SIGGRAPH Asia 2019) of a quadtree: every leaf loses alpha x
    the tree's mean flux over its area (floored at 0), interior cells are
    the sums of their children; a tree left with under 5 % of its flux is
    returned unchanged."""
    depth = [0] * len(tree)
    for i, (_, child) in enumerate(tree):
        for c in child:
            if c >= 0:
                depth[c] = depth[i] + 1
    tot = sum(tree[0][0])
    comp = [0.0] * len(tree)
    for i in range(len(tree) - 1, -1, -1):
        flux, child = tree[i]
        sub = alpha * tot * 4.0 ** -(depth[i] + 1)
        comp[i] = sum(comp[c] if c >= 0 else max(f - sub, 0.0) for f, c in zip(flux, child))
    if comp[0] < 0.05 * tot:
        return tree
    out = []
    for i, (flux, child) in enumerate(tree):
        sub = alpha * tot * 4.0 ** -(depth[i] + 1)
        out.append(([comp[c] if c >= 0 else max(f - sub, 0.0) for f, c in zip(flux, child)], child))
    return out


def build_quadtree(records: np.ndarray, pss: bool = False, clamp_median: float = float(CLAMP_MEDIAN),
                   rho: float = RHO, weights=None, compensate: float = 0.0):
    """One region's quadtree: list of (flux[4] float64, child[4]) in
    breadth-first order (cell 0 the root), or None when the region has no
    flux.  A record's flux is its weight (the renderer's Lum(Li) |cos| / pdf,
    which estimates Li |cos| whatever distribution sampled wi; Müller et
    al. 2017 divide by the pdf too) or, without weights, Lum(Li)."""
    w = luminance(records["Li"]) if weights is None else flux_weights(weights)
    if not np.any(w > 0):
        return None
    if clamp_median > 0:
        clamp = F(F(clamp_median) * median_bisection(w))
        wc = np.minimum(w, clamp).astype(np.float64)
    else:
        wc = w.astype(np.float64)
    total = float(wc.sum())
    if not (total > 0) or not np.isfinite(total):
        return None
    if pss:
        u, v, ok = pss_uv(records["normal"], records["wi"])
    else:
        u, v = dir_to_uv(records["wi"])
        ok = np.ones(len(u), bool)
    keep = (w > 0) & ok
    u, v, wc = u[keep], v[keep], wc[keep]
    thresh = rho * total
    cells = [(F(0), F(0), F(1), 0)]
    out = []
    head = 0
    while head < len(cells):
        u0, v0, sz, depth = cells[head]
        head += 1
        half = F(sz * F(0.5))
        inside = (u >= u0) & (u < F(u0 + sz)) & (v >= v0) & (v < F(v0 + sz))
        xi = (u >= F(u0 + half)).astype(int)
        yi = (v >= F(v0 + half)).astype(int)
        c_of = 2 * yi + xi
        flux = [0.0] * 4
        child = [-1] * 4
        for c in range(4):
            m = inside & (c_of == c)
            flux[c] = float(wc[m].sum())
            cnt = int(np.count_nonzero(m))
            if flux[c] > thresh and cnt >= 2 and depth + 1 < MAX_DEPTH and len(cells) < MAX_NODES:
                child[c] = len(cells)
                cells.append((F(u0 + F(half * F(c & 1))), F(v0 + F(half * F(c >> 1))), half, depth + 1))
        out.append((flux, child))
    return compensate_tree(out, compensate) if compensate > 0 else out


def quad_pdf(tree, u: float, v: float) -> float:
    """Density of the tree over the unit square at (u, v) (1 = uniform)."""
    pdf, node = 1.0, 0
    for _ in range(MAX_DEPTH + 1):
        flux, child = tree[node]
        total = sum(flux)
        if not total > 0:
            return 0.0
        xi, yi = int(u >= 0.5), int(v >= 0.5)
        c = 2 * yi + xi
        pdf *= 4.0 * flux[c] / total
        if child[c] < 0 or pdf == 0.0:
            return pdf
        u, v = u * 2.0 - xi, v * 2.0 - yi
        node = child[c]
    return pdf


def quad_sample(tree, r1: float, r2: float) -> tuple[float, float]:
    """(u, v) for two uniforms: x half by the flux of the left and right
    columns, then y half within the column, each uniform rescaled to the
    chosen interval; the last pair places the point inside the leaf."""
    u0 = v0 = 0.0
    size = 1.0
    node = 0
    for _ in range(MAX_DEPTH + 1):
        flux, child = tree[node]
        left, right = flux[0] + flux[2], flux[1] + flux[3]
        total = left + right
        pl = left / total if total > 0 else 0.5
        if r1 < pl:
            xi, r1 = 0, (r1 / pl if pl > 0 else 0.0)
        else:
            xi, r1 = 1, ((r1 - pl) / (1.0 - pl) if 1.0 - pl > 0 else 0.0)
        top, bot = flux[xi], flux[2 + xi]
        pt = top / (top + bot) if top + bot > 0 else 0.5
        if r2 < pt:
            yi, r2 = 0, (r2 / pt if pt > 0 else 0.0)
        else:
            yi, r2 = 1, ((r2 - pt) / (1.0 - pt) if 1.0 - pt > 0 else 0.0)
        size *= 0.5
        u0 += size * xi
        v0 += size * yi
        c = 2 * yi + xi
        if child[c] < 0:
            break
        node = child[c]
    return u0 + size * r1, v0 + size * r2


def region_of(nodes: np.ndarray, root_node_to_region: dict, x: np.ndarray) -> int:
    """Region of a position: descend the point BVH from the root into the
    child whose box is nearer (0 inside; ties to the left) until a region
    root (-1 if a leaf comes first)."""
    x = np.asarray(x, F)

    def box_d(n):
        d = np.maximum(np.maximum(n["bmin"] - x, x - n["bmax"]), F(0)).astype(F)
        return F((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2])

    node = 0
    for _ in range(64):
        if node in root_node_to_region:
            return root_node_to_region[node]
        n = nodes[node]
        if n["left"] < 0:
            return -1
        a, b = int(n["left"]), int(n["right"])
        node = b if box_d(nodes[b]) < box_d(nodes[a]) else a
    return -1


class Guide:
    """The whole guide over an exported cache (point-BVH nodes and records
    in leaf order)."""

    def __init__(self, nodes: np.ndarray, records: np.ndarray, pss: bool = False, region_max: int = REGION_MAX,
                 clamp_median: float = float(CLAMP_MEDIAN), rho: float = RHO, weights=None,
                 compensate: float = 0.0):
        self.nodes = nodes
        self.regions = regions_from_bvh(nodes, len(records), region_max)
        self.trees = [build_quadtree(records[f:f + c], pss, clamp_median, rho,
                                     None if weights is None else weights[f:f + c], compensate)
                      for f, c, _ in self.regions]
        self.root_region = {node: i for i, (_, _, node) in enumerate(self.regions)}

    def tree_at(self, x):
        r = region_of(self.nodes, self.root_region, x)
        return None if r < 0 else self.trees[r]

    def pdf(self, x, wi) -> float:
        """Solid-angle pdf of the quadtree alone (no uniform share)."""
        t = self.tree_at(x)
        if t is None:
            return 0.0
        wi = np.asarray(wi, np.float64)
        wi = (wi / np.linalg.norm(wi)).astype(F)
        u, v = dir_to_uv(wi[None])
        return quad_pdf(t, float(u[0]), float(v[0])) / (4.0 * np.pi)

    def sample(self, x, r1: float, r2: float):
        """(direction, solid-angle pdf of the quadtree alone) or None."""
        t = self.tree_at(x)
        if t is None:
            return None
        u, v = quad_sample(t, r1, r2)
        return uv_to_dir(u, v), quad_pdf(t, u, v) / (4.0 * np.pi)
