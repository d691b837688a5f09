"""Reading and writing the reference's scene format on the host.

`load_scene(dir)` mirrors `loadScene` (SceneLoader.h:222-269) and
`loadInstance` (SceneLoader.h:104-220): `scene.json` (GEMScene::load,
GEMLoader.h:853-882) holds the image size, fov, camera (from/to/up, flipX), an
optional `envmap` and a list of instances (mesh file, 4x4 world matrix and
material keys); meshes are `.gem` files (GEMModelLoader::load,
GEMLoader.h:430-457: magic 4058972161, static vertices of position, normal,
tangent, u, v as 11 floats, uint32 indices).  Vertices are transformed in
float32 in the reference's operation order (Matrix::mulPoint, the transposed
MESA inverse for normals), zero-area triangles are dropped, and one material
is created per instance, so the result feeds `pgx_scene_upload` with the
same triangles the reference builds.  Albedo textures are 8-bit PNGs scaled
by 1/255 (Imaging.h:42-78); environment maps are Radiance .hdr files.

`write_scene(desc, dir)` writes a SceneDesc in the same format (identity
world matrices, one mesh per material, 1x1 PNG albedos), so the reference's
own loader reads the procedural scenes.
"""
from __future__ import annotations

import ctypes
import json
import re
import struct
import zlib
from pathlib import Path

import numpy as np

from .abi import (BSDF_CONDUCTOR, BSDF_DIELECTRIC, BSDF_DIFFUSE, BSDF_GLASS, BSDF_MIRROR, BSDF_ORENNAYAR,
                  BSDF_PLASTIC, MATERIAL, TRIANGLE)
from .scenes import SceneDesc

GEM_MAGIC = 4058972161
F32 = np.float32


# ---- images ---------------------------------------------------------------------

def read_png(path: str | Path) -> tuple[np.ndarray, int]:
    """8-bit, non-interlaced PNG -> (H, W, C) uint8 and C."""
    data = Path(path).read_bytes()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError(f"{path}: not a PNG file")
    pos = 8
    idat = b""
    w = h = 0
    ctype = bitd = interlace = 0
    palette = None
    while pos < len(data):
        ln, tag = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + ln]
        pos += 12 + ln
        if tag == b"IHDR":
            w, h, bitd, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif tag == b"PLTE":
            palette = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif tag == b"IDAT":
            idat += body
        elif tag == b"IEND":
            break
    if bitd != 8 or interlace != 0:
        raise ValueError(f"{path}: only 8-bit non-interlaced PNGs are supported")
    channels = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    raw = zlib.decompress(idat)
    stride = w * channels
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    p = 0
    for y in range(h):
        ftype = raw[p]
        line = np.frombuffer(raw, np.uint8, stride, p + 1).astype(np.int32)
        p += 1 + stride
        cur = np.zeros(stride, np.int32)
        if ftype == 0:
            cur = line
        elif ftype == 2:
            cur = (line + prev) & 255
        else:
            for x in range(stride):
                a = cur[x - channels] if x >= channels else 0
                b = prev[x]
                c = prev[x - channels] if x >= channels else 0
                if ftype == 1:
                    pr = a
                elif ftype == 3:
                    pr = (a + b) >> 1
                else:
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    pr = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (line[x] + pr) & 255
        out[y] = cur
        prev = cur
    img = out.reshape(h, w, channels)
    if ctype == 3:
        img = palette[img[..., 0]]
        channels = 3
    return img, channels


def read_hdr(path: str | Path) -> np.ndarray:
    """Radiance RGBE -> (H, W, 3) float32, texel = byte * 2^(e - 136), zero
    when e == 0, with stb_image's scanline rules: widths 8..32767 start each
    scanline with a run-length header (2, 2, width); a scanline without one
    switches to flat pixels, which are then read for the whole image from
    that point of the file."""
    data = Path(path).read_bytes()
    if not (data.startswith(b"#?RADIANCE\n") or data.startswith(b"#?RGBE\n")):
        raise ValueError(f"{path}: not a Radiance file")
    pos = 0
    while True:
        end = data.index(b"\n", pos)
        line = data[pos:end]
        pos = end + 1
        if line == b"":
            break
    end = data.index(b"\n", pos)
    parts = data[pos:end].split()
    pos = end + 1
    if len(parts) != 4 or parts[0] != b"-Y" or parts[2] != b"+X":
        raise ValueError(f"{path}: unsupported Radiance orientation")
    h, w = int(parts[1]), int(parts[3])
    rgbe = np.zeros((h, w, 4), np.uint8)
    flat = not (8 <= w < 32768)
    if not flat:
        for y in range(h):
            if not (data[pos] == 2 and data[pos + 1] == 2 and data[pos + 2] < 128):
                flat = True
                break
            if (data[pos + 2] << 8 | data[pos + 3]) != w:
                raise ValueError(f"{path}: invalid decoded scanline length")
            pos += 4
            for c in range(4):
                x = 0
                while x < w:
                    cnt = data[pos]
                    pos += 1
                    if cnt > 128:
                        cnt -= 128
                        rgbe[y, x:x + cnt, c] = data[pos]
                        pos += 1
                    else:
                        rgbe[y, x:x + cnt, c] = np.frombuffer(data, np.uint8, cnt, pos)
                        pos += cnt
                    x += cnt
    if flat:
        rgbe = np.frombuffer(data, np.uint8, w * h * 4, pos).reshape(h, w, 4).copy()
    e = rgbe[..., 3].astype(np.int32)
    f = np.where(e == 0, 0.0, np.ldexp(1.0, e - 136)).astype(F32)
    return (rgbe[..., :3].astype(F32) * f[..., None]).astype(F32)


def read_bmp(path: str | Path) -> tuple[np.ndarray, int]:
    """Uncompressed 24/32-bit BMP -> (H, W, C) uint8 rows top-down, RGB(A)."""
    data = Path(path).read_bytes()
    if data[:2] != b"BM":
        raise ValueError(f"{path}: not a BMP file")
    off = struct.unpack_from("<I", data, 10)[0]
    hsize, w, h, _, bpp, comp = struct.unpack_from("<IiiHHI", data, 14)
    if comp not in (0, 3) or bpp not in (24, 32):
        raise ValueError(f"{path}: only uncompressed 24/32-bit BMPs are supported")
    ch = bpp // 8
    stride = (w * ch + 3) & ~3
    rows = np.frombuffer(data, np.uint8, stride * abs(h), off).reshape(abs(h), stride)[:, :w * ch]
    img = rows.reshape(abs(h), w, ch)
    if h > 0:
        img = img[::-1]
    out = img[..., [2, 1, 0] + ([3] if ch == 4 else [])]
    return np.ascontiguousarray(out), ch


def read_tga(path: str | Path) -> tuple[np.ndarray, int]:
    """True-colour TGA (types 2 and 10, 24/32-bit) -> (H, W, C) uint8 rows top-down."""
    data = Path(path).read_bytes()
    idlen, cmtype, itype = data[0], data[1], data[2]
    w, h, bpp, desc = struct.unpack_from("<HHBB", data, 12)
    if cmtype != 0 or itype not in (2, 10) or bpp not in (24, 32):
        raise ValueError(f"{path}: only true-colour 24/32-bit TGAs are supported")
    ch = bpp // 8
    pos = 18 + idlen
    n = w * h
    if itype == 2:
        px = np.frombuffer(data, np.uint8, n * ch, pos).reshape(n, ch)
    else:
        px = np.zeros((n, ch), np.uint8)
        i = 0
        while i < n:
            hdr = data[pos]
            pos += 1
            cnt = (hdr & 127) + 1
            if hdr & 128:
                px[i:i + cnt] = np.frombuffer(data, np.uint8, ch, pos)
                pos += ch
            else:
                px[i:i + cnt] = np.frombuffer(data, np.uint8, cnt * ch, pos).reshape(cnt, ch)
                pos += cnt * ch
            i += cnt
    img = px.reshape(h, w, ch)
    if not (desc & 0x20):
        img = img[::-1]
    out = img[..., [2, 1, 0] + ([3] if ch == 4 else [])]
    return np.ascontiguousarray(out), ch


def read_jpeg(path: str | Path) -> tuple[np.ndarray, int]:
    """8-bit samples (H, W, C) and channel count of a JPEG file, decoded by
    libpgx's pgx_image_decode_jpeg (baseline and progressive Huffman JPEG).
    Raises ValueError for malformed or unsupported data."""
    from . import abi
    data = Path(path).read_bytes()
    lib = abi.load()
    buf = (ctypes.c_uint8 * len(data)).from_buffer_copy(data)
    w, h, c = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    msg = ctypes.create_string_buffer(256)
    args = (ctypes.addressof(buf), len(data), ctypes.byref(w), ctypes.byref(h), ctypes.byref(c))
    if lib.pgx_image_decode_jpeg(*args, None, 0, msg, 256) != abi.PGX_OK:
        raise ValueError(f"{path}: {msg.value.decode(errors='replace')}")
    out = np.zeros(w.value * h.value * c.value, np.uint8)
    if lib.pgx_image_decode_jpeg(*args, out.ctypes.data, out.size, msg, 256) != abi.PGX_OK:
        raise ValueError(f"{path}: {msg.value.decode(errors='replace')}")
    return out.reshape(h.value, w.value, c.value), c.value


def _white() -> np.ndarray:
    """Texture::loadDefault (Imaging.h:36-42)."""
    return np.ones((1, 1, 3), F32)


def load_texture(path: str) -> np.ndarray:
    """Texture::load (Imaging.h:44-79): RGB float texels, rows top-down.

    A file that cannot be read gives the 1x1 white default, as stbi_load
    failing does in the reference.  8-bit images are scaled by 1/255; the
    reference reads texel i at bytes [i*C, i*C+3) whatever the channel count C,
    so 1- and 2-channel images take their colour from the next bytes (bytes
    past the end of the image read as 0 here).  JPEG is decoded by libpgx
    (pgx_image_decode_jpeg), whose samples agree with stb_image's to within a
    few levels (it rounds the inverse DCT, chroma upsampling and colour
    conversion in floating point where stb_image uses fixed point)."""
    if ".hdr" in path:
        try:
            return read_hdr(path)
        except (OSError, ValueError):
            return _white()
    low = path.lower()
    try:
        if low.endswith(".png"):
            img, ch = read_png(path)
        elif low.endswith(".bmp"):
            img, ch = read_bmp(path)
        elif low.endswith(".tga"):
            img, ch = read_tga(path)
        elif low.endswith((".jpg", ".jpeg")):
            img, ch = read_jpeg(path)
        else:
            return _white()
    except (OSError, ValueError):
        return _white()
    h, w = img.shape[:2]
    flat = img.reshape(-1)
    idx = np.arange(h * w)[:, None] * ch + np.arange(3)[None, :]
    padded = np.concatenate([flat, np.zeros(3, np.uint8)])
    texels = padded[idx].astype(F32) * (F32(1.0) / F32(255.0))
    return texels.reshape(h, w, 3).astype(F32)


# ---- float32 matrix helpers in the reference's operation order ---------------------

def _invert(m: np.ndarray) -> np.ndarray:
    """Matrix::invert (MyMath.h:286-323), float32, same expression order."""
    m = [F32(x) for x in m]
    inv = [F32(0)] * 16

    def t(a, b, c):
        return m[a] * m[b] * m[c]

    inv[0] = t(5, 10, 15) - t(5, 11, 14) - t(9, 6, 15) + t(9, 7, 14) + t(13, 6, 11) - t(13, 7, 10)
    inv[4] = -m[4] * m[10] * m[15] + t(4, 11, 14) + t(8, 6, 15) - t(8, 7, 14) - t(12, 6, 11) + t(12, 7, 10)
    inv[8] = t(4, 9, 15) - t(4, 11, 13) - t(8, 5, 15) + t(8, 7, 13) + t(12, 5, 11) - t(12, 7, 9)
    inv[12] = -m[4] * m[9] * m[14] + t(4, 10, 13) + t(8, 5, 14) - t(8, 6, 13) - t(12, 5, 10) + t(12, 6, 9)
    inv[1] = -m[1] * m[10] * m[15] + t(1, 11, 14) + t(9, 2, 15) - t(9, 3, 14) - t(13, 2, 11) + t(13, 3, 10)
    inv[5] = t(0, 10, 15) - t(0, 11, 14) - t(8, 2, 15) + t(8, 3, 14) + t(12, 2, 11) - t(12, 3, 10)
    inv[9] = -m[0] * m[9] * m[15] + t(0, 11, 13) + t(8, 1, 15) - t(8, 3, 13) - t(12, 1, 11) + t(12, 3, 9)
    inv[13] = t(0, 9, 14) - t(0, 10, 13) - t(8, 1, 14) + t(8, 2, 13) + t(12, 1, 10) - t(12, 2, 9)
    inv[2] = t(1, 6, 15) - t(1, 7, 14) - t(5, 2, 15) + t(5, 3, 14) + t(13, 2, 7) - t(13, 3, 6)
    inv[6] = -m[0] * m[6] * m[15] + t(0, 7, 14) + t(4, 2, 15) - t(4, 3, 14) - t(12, 2, 7) + t(12, 3, 6)
    inv[10] = t(0, 5, 15) - t(0, 7, 13) - t(4, 1, 15) + t(4, 3, 13) + t(12, 1, 7) - t(12, 3, 5)
    inv[14] = -m[0] * m[5] * m[14] + t(0, 6, 13) + t(4, 1, 14) - t(4, 2, 13) - t(12, 1, 6) + t(12, 2, 5)
    inv[3] = -m[1] * m[6] * m[11] + t(1, 7, 10) + t(5, 2, 11) - t(5, 3, 10) - t(9, 2, 7) + t(9, 3, 6)
    inv[7] = t(0, 6, 11) - t(0, 7, 10) - t(4, 2, 11) + t(4, 3, 10) + t(8, 2, 7) - t(8, 3, 6)
    inv[11] = -m[0] * m[5] * m[11] + t(0, 7, 9) + t(4, 1, 11) - t(4, 3, 9) - t(8, 1, 7) + t(8, 3, 5)
    inv[15] = t(0, 5, 10) - t(0, 6, 9) - t(4, 1, 10) + t(4, 2, 9) + t(8, 1, 6) - t(8, 2, 5)
    det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12]
    if det == 0:
        det = F32(1)
    det = F32(1) / det
    return np.array([x * det for x in inv], F32)


def _mul_point(m: np.ndarray, p: np.ndarray) -> np.ndarray:
    x, y, z = p[:, 0], p[:, 1], p[:, 2]
    return np.stack([((x * m[0] + y * m[1]) + z * m[2]) + m[3], ((x * m[4] + y * m[5]) + z * m[6]) + m[7],
                     ((x * m[8] + y * m[9]) + z * m[10]) + m[11]], 1).astype(F32)


def _mul_vec(m: np.ndarray, v: np.ndarray) -> np.ndarray:
    x, y, z = v[:, 0], v[:, 1], v[:, 2]
    return np.stack([(x * m[0] + y * m[1]) + z * m[2], (x * m[4] + y * m[5]) + z * m[6],
                     (x * m[8] + y * m[9]) + z * m[10]], 1).astype(F32)


def _normalize(v: np.ndarray) -> np.ndarray:
    ln = np.sqrt((v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2]).astype(F32)
    inv = (F32(1) / ln).astype(F32)
    return (v * inv[:, None]).astype(F32)


def _tri_area(p0, p1, p2) -> np.ndarray:
    """Triangle::init's area (Geometry.h:86-92)."""
    e1 = (p2 - p1).astype(F32)
    e2 = (p0 - p2).astype(F32)
    cx = e1[:, 1] * e2[:, 2] - e1[:, 2] * e2[:, 1]
    cy = e1[:, 2] * e2[:, 0] - e1[:, 0] * e2[:, 2]
    cz = e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]
    return np.sqrt((cx * cx + cy * cy) + cz * cz).astype(F32) * F32(0.5)


# ---- GEM meshes --------------------------------------------------------------------

def read_gem(path: str | Path) -> list[tuple[dict, np.ndarray, np.ndarray]]:
    """GEMModelLoader::load: [(material properties, vertices (V, 11) f32, indices u32)]."""
    data = Path(path).read_bytes()
    magic, animated, nmesh = struct.unpack_from("<III", data, 0)
    if magic != GEM_MAGIC:
        raise ValueError(f"{path} is not a GE Model File")
    if animated:
        raise ValueError(f"{path}: animated meshes are not supported")
    pos = 12
    meshes = []

    def string():
        nonlocal pos
        (ln,) = struct.unpack_from("<i", data, pos)
        s = data[pos + 4:pos + 4 + ln].split(b"\0")[0].decode("latin-1")
        pos += 4 + ln
        return s

    for _ in range(nmesh):
        (nprop,) = struct.unpack_from("<I", data, pos)
        pos += 4
        props = {}
        for _ in range(nprop):
            k = string()
            props[k] = string()
        (nv,) = struct.unpack_from("<I", data, pos)
        pos += 4
        verts = np.frombuffer(data, F32, nv * 11, pos).reshape(nv, 11).copy()
        pos += nv * 44
        (ni,) = struct.unpack_from("<I", data, pos)
        pos += 4
        idx = np.frombuffer(data, np.uint32, ni, pos).copy()
        pos += ni * 4
        meshes.append((props, verts, idx))
    return meshes


def write_gem(path: str | Path, meshes: list[tuple[np.ndarray, np.ndarray]]) -> None:
    """Writes static meshes [(vertices (V, 11) f32, indices u32)] without material properties."""
    out = bytearray(struct.pack("<III", GEM_MAGIC, 0, len(meshes)))
    for verts, idx in meshes:
        out += struct.pack("<I", 0)
        v = np.ascontiguousarray(verts, F32)
        out += struct.pack("<I", len(v)) + v.tobytes()
        i = np.ascontiguousarray(idx, np.uint32)
        out += struct.pack("<I", len(i)) + i.tobytes()
    Path(path).write_bytes(bytes(out))


# ---- scene.json ----------------------------------------------------------------------

_libc = ctypes.CDLL(None, use_errno=True)
_libc.strtof.restype = ctypes.c_float
_libc.strtof.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p)]
_INT_PREFIX = re.compile(r"^[ \t\n\v\f\r]*[+-]?[0-9]+")


def _stof(s: str) -> float | None:
    """std::stof: strtof on the longest valid prefix (C library, so decimal
    strings round to float32 exactly as in the reference); None where stof
    throws (no conversion, or out of range)."""
    b = s.encode("latin-1", "replace")
    end = ctypes.c_char_p()
    ctypes.set_errno(0)
    buf = ctypes.create_string_buffer(b)
    v = _libc.strtof(ctypes.cast(buf, ctypes.c_char_p), ctypes.byref(end))
    consumed = ctypes.cast(end, ctypes.c_void_p).value - ctypes.addressof(buf)
    if consumed == 0 or ctypes.get_errno() != 0:
        return None
    return float(np.float32(v))


def _stoi(s: str) -> int | None:
    """std::stoi: leading decimal integer, None where stoi throws."""
    m = _INT_PREFIX.match(s)
    if not m:
        return None
    v = int(m.group(0))
    return v if -2**31 <= v < 2**31 else None


def _json_float(tok: str) -> float:
    """GEMJsonParser::parseNum keeps numbers as std::stof of their text."""
    v = _stof(tok)
    if v is None:
        raise ValueError(f"number out of float range: {tok}")
    return v


def _prop_str(v) -> str:
    """GEMJson::asStr (GEMLoader.h:577-590): booleans and numbers through
    std::to_string (numbers as float, six decimals), other values empty."""
    if isinstance(v, bool):
        return str(int(v))
    if isinstance(v, (int, float)):
        return "%f" % float(v)
    if isinstance(v, str):
        return v
    return ""


def _as_float(s: str, default: float) -> float:
    """GEMProperty::getValue(float) (GEMLoader.h:61-76)."""
    if s == "":
        return default
    v = _stof(s)
    return default if v is None else v


def _as_int(s: str, default: int) -> int:
    """GEMProperty::getValue(int) (GEMLoader.h:78-94)."""
    if s == "":
        return default
    v = _stoi(s)
    return default if v is None else v


def _as_vec3(s: str) -> tuple[float, float, float]:
    """GEMProperty::getValuesAsVector3 (GEMLoader.h:96-144): std::getline
    split on ' ' (no token after a trailing separator), each word through
    stof, empty or unparsable words and missing entries 0."""
    words = s.split(" ")
    if words and words[-1] == "":
        words = words[:-1]
    vals = []
    for w in words:
        v = _stof(w) if w != "" else None
        vals.append(0.0 if v is None else v)
    vals += [0.0] * (3 - len(vals))
    return vals[0], vals[1], vals[2]


def _parse_json(text: str):
    """scene.json as GEMJsonParser reads it: objects become dicts whose
    iteration order is sorted by key (std::map, last duplicate wins) and
    numbers are float32 values."""
    def hook(pairs):
        d = {}
        for k, v in pairs:
            d[k] = v
        return {k: d[k] for k in sorted(d)}
    return json.loads(text, object_pairs_hook=hook, parse_float=_json_float, parse_int=_json_float)


_BSDF_NAMES = {"diffuse": BSDF_DIFFUSE, "orennayar": BSDF_ORENNAYAR, "glass": BSDF_GLASS, "mirror": BSDF_MIRROR,
               "plastic": BSDF_PLASTIC, "dielectric": BSDF_DIELECTRIC, "conductor": BSDF_CONDUCTOR}


def _instance_material(keys: dict, texture) -> np.ndarray | None:
    """The BSDF loadInstance makes for one instance (SceneLoader.h:107-176);
    None when `bsdf` names no known BSDF (the instance is then skipped)."""
    kind = _BSDF_NAMES.get(keys.get("bsdf", ""))
    if kind is None:
        return None
    m = np.zeros((), MATERIAL)
    m["albedo_texture"] = texture(keys.get("reflectance", ""))
    if kind == BSDF_ORENNAYAR:
        m["sigma"] = _as_float(keys.get("alpha", ""), 1.0)
    if kind in (BSDF_GLASS, BSDF_PLASTIC, BSDF_DIELECTRIC):
        m["int_ior"] = _as_float(keys.get("intIOR", ""), 1.33)
        m["ext_ior"] = _as_float(keys.get("extIOR", ""), 1.0)
    if kind in (BSDF_PLASTIC, BSDF_DIELECTRIC, BSDF_CONDUCTOR):
        m["roughness"] = _as_float(keys.get("roughness", ""), 1.0)
    if kind == BSDF_DIELECTRIC and float(m["roughness"]) < float(F32(0.001)):
        kind = BSDF_GLASS  # SceneLoader.h:145-149
        m["roughness"] = 0.0
    if kind == BSDF_CONDUCTOR:
        m["eta"] = _as_vec3(keys.get("eta", ""))
        m["k"] = _as_vec3(keys.get("k", ""))
    m["kind"] = kind
    if keys.get("emission", "") != "":
        m["emission"] = _as_vec3(keys["emission"])
    if _as_int(keys.get("coatingThickness", ""), 0) > 0:
        # LayeredBSDF (Materials.h:855-897) passes every query to its base and
        # is built after addLight, so the wrapped material emits nothing.
        m["layered"] = 1
        m["emission"] = 0.0
    return m


def load_scene(scene_dir: str | Path) -> SceneDesc:
    """loadScene (SceneLoader.h:222-269): scene.json, .gem meshes and textures
    in the renderer's upload layout.

    Instances are read in the order GEMScene::load keeps them (top-level keys
    sorted, then array order); each known instance adds one material, its
    albedo texture (deduplicated by file name, first use first) and its
    non-degenerate triangles with float32 vertices transformed exactly as
    the reference transforms them."""
    d = str(scene_dir).rstrip("/") if str(scene_dir) != "/" else "/"
    with open(f"{d}/scene.json", encoding="latin-1") as f:
        js = _parse_json(f.read())
    props = {k: _prop_str(v) for k, v in js.items() if not isinstance(v, list)}
    instances = [inst for v in js.values() if isinstance(v, list) for inst in v]
    width = _as_int(props.get("width", ""), 1920)
    height = _as_int(props.get("height", ""), 1080)
    fov = _as_float(props.get("fov", ""), 45.0)
    cam = dict(from_=_as_vec3(props.get("from", "")), to=_as_vec3(props.get("to", "")),
               up=_as_vec3(props.get("up", "")), fov=fov, width=width, height=height,
               flip_x=int(_as_int(props.get("flipX", ""), 0) == 1))
    textures: list[np.ndarray] = []
    tex_ids: dict[str, int] = {}

    def texture(name: str) -> int:
        key = f"{d}/{name}"
        if key not in tex_ids:
            tex_ids[key] = len(textures)
            textures.append(load_texture(key))
        return tex_ids[key]

    mats = []
    tris = []
    for inst in instances:
        if not isinstance(inst, dict):
            continue
        keys = {k: _prop_str(v) for k, v in inst.items() if k not in ("filename", "world")}
        mesh_file = _prop_str(inst.get("filename", ""))
        meshes = read_gem(f"{d}/{mesh_file}")
        m = _instance_material(keys, texture)
        if m is None:
            print("Error in loading")  # SceneLoader.h:177-181
            continue
        mat_index = len(mats)
        mats.append(m)
        w = inst.get("world")
        world = np.array([float(w[i]) if isinstance(w[i], float) else 0.0 for i in range(16)]
                         if isinstance(w, list) else np.eye(4).ravel(), F32)
        vec_t = _invert(world).reshape(4, 4).T.ravel()
        verts, idx = [], []
        for _, v, ind in meshes:
            idx.append(ind.astype(np.int64) + sum(len(x) for x in idx))
            verts.append(v)
        if not verts:
            continue
        v = np.concatenate(verts)
        ind = np.concatenate(idx)
        p = _mul_point(world, v[:, 0:3])
        n = _normalize(_mul_vec(vec_t, v[:, 3:6]))
        ind = ind[: len(ind) // 3 * 3].reshape(-1, 3)
        t = np.zeros(len(ind), TRIANGLE)
        t["v"]["p"] = p[ind]
        t["v"]["n"] = n[ind]
        t["v"]["u"] = v[ind, 9]
        t["v"]["v"] = v[ind, 10]
        t["material"] = mat_index
        area = _tri_area(t["v"]["p"][:, 0], t["v"]["p"][:, 1], t["v"]["p"][:, 2])
        tris.append(t[area > 0])
    env = None
    if props.get("envmap", "") != "":
        env = load_texture(f"{d}/{props['envmap']}")
    triangles = np.concatenate(tris) if tris else np.zeros(0, TRIANGLE)
    return SceneDesc(triangles, np.array(mats, MATERIAL).reshape(-1), cam, env=env, textures=textures,
                     name=Path(d).name)


def _write_png(path: Path, rgb8: np.ndarray) -> None:
    from .api import write_png
    write_png(str(path), rgb8)


def _write_hdr(path: Path, img: np.ndarray) -> None:
    from .api import write_hdr
    write_hdr(str(path), img)


def write_scene(desc: SceneDesc, scene_dir: str | Path) -> Path:
    """A SceneDesc in the reference's format: one .gem mesh and one instance
    per material (identity world matrix), albedo as an 8-bit PNG (constant
    albedos become 1x1 images, quantised to 1/255), environment as .hdr."""
    d = Path(scene_dir)
    d.mkdir(parents=True, exist_ok=True)
    kinds = {BSDF_DIFFUSE: "diffuse", BSDF_ORENNAYAR: "orennayar", BSDF_GLASS: "glass", BSDF_MIRROR: "mirror",
             BSDF_PLASTIC: "plastic", BSDF_DIELECTRIC: "dielectric", BSDF_CONDUCTOR: "conductor"}
    c = desc.camera
    js = {"width": str(c["width"]), "height": str(c["height"]), "fov": repr(float(c["fov"])),
          "from": " ".join(repr(float(x)) for x in c["from_"]), "to": " ".join(repr(float(x)) for x in c["to"]),
          "up": " ".join(repr(float(x)) for x in c["up"])}
    if desc.env is not None:
        _write_hdr(d / "env.hdr", desc.env)
        js["envmap"] = "env.hdr"
    ident = [1.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0, 1.0]
    insts = []
    tris = desc.triangles
    for mi, m in enumerate(desc.materials):
        sel = tris[tris["material"] == mi]
        if len(sel) == 0:
            continue
        v = np.zeros((len(sel) * 3, 11), F32)
        v[:, 0:3] = sel["v"]["p"].reshape(-1, 3)
        v[:, 3:6] = sel["v"]["n"].reshape(-1, 3)
        v[:, 9] = sel["v"]["u"].reshape(-1)
        v[:, 10] = sel["v"]["v"].reshape(-1)
        write_gem(d / f"mesh{mi:05d}.gem", [(v, np.arange(len(v), dtype=np.uint32))])
        tex = f"albedo{mi:05d}.png"
        if int(m["albedo_texture"]) >= 0:
            img = desc.textures[int(m["albedo_texture"])]
        else:
            img = np.asarray(m["albedo"], F32).reshape(1, 1, 3)
        _write_png(d / tex, np.clip(np.rint(np.asarray(img) * 255.0), 0, 255).astype(np.uint8))
        inst = {"filename": f"mesh{mi:05d}.gem", "world": ident, "bsdf": kinds[int(m["kind"])], "reflectance": tex}
        if int(m["kind"]) in (BSDF_GLASS, BSDF_PLASTIC, BSDF_DIELECTRIC):
            inst["intIOR"] = repr(float(m["int_ior"]))
            inst["extIOR"] = repr(float(m["ext_ior"]))
        if int(m["kind"]) in (BSDF_PLASTIC, BSDF_DIELECTRIC, BSDF_CONDUCTOR):
            inst["roughness"] = repr(float(m["roughness"]))
        if int(m["kind"]) == BSDF_CONDUCTOR:
            inst["eta"] = " ".join(repr(float(x)) for x in m["eta"])
            inst["k"] = " ".join(repr(float(x)) for x in m["k"])
        if int(m["kind"]) == BSDF_ORENNAYAR:
            inst["alpha"] = repr(float(m["sigma"]))
        if float(np.max(m["emission"])) > 0:
            inst["emission"] = " ".join(repr(float(x)) for x in m["emission"])
        insts.append(inst)
    js["instances"] = insts
    (d / "scene.json").write_text(json.dumps(js, indent=1))
    return d
