"""Builds libpgx.so, the CUDA library behind the C ABI in include/pgx.h.

Each .cu file under csrc/ is compiled by nvcc for sm_103a only, in parallel,
then linked into ``pathguidingdissertation_gb300/libpgx.so`` (git-ignored).
Host code is compiled with ``-ffp-contract=off`` so host-side set-up math
(camera matrices, light tables) rounds like the reference on both x86_64 and
aarch64.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "libpgx.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
    "-I", str(INCLUDE),
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpgx")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _deps() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))


# Per-file flags: the integrator and the cache round every product and sum
# separately, like the reference's scalar code and the float32 checks
# (traversal uses explicit _rn intrinsics and is exact regardless).
FILE_FLAGS = {"render.cu": ["-fmad=false"], "cache.cu": ["-fmad=false"], "bsdf.cu": ["-fmad=false"]}


def _compile(src: Path, extra: list[str]) -> Path:
    OBJ.mkdir(parents=True, exist_ok=True)
    obj = OBJ / (src.stem + ".o")
    newest_dep = max([src.stat().st_mtime] + [d.stat().st_mtime for d in _deps()])
    if obj.exists() and obj.stat().st_mtime >= newest_dep and not extra:
        return obj
    cmd = [nvcc(), *NVCC_FLAGS, *FILE_FLAGS.get(src.name, []), *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout[-6000:]}")
    if extra:
        sys.stdout.write(r.stdout)
    return obj


def _platform_stamp() -> str:
    import platform
    return f"{platform.machine()} {nvcc()}"


def build(force: bool = False, verbose_ptxas: bool = False) -> Path:
    """Compile and link libpgx.so; returns its path."""
    stamp = OBJ / "platform.txt"
    if OBJ.exists() and (not stamp.exists() or stamp.read_text() != _platform_stamp()):
        force = True  # objects from another machine (e.g. x86_64 vs aarch64)
    if force and OBJ.exists():
        shutil.rmtree(OBJ)
    OBJ.mkdir(parents=True, exist_ok=True)
    stamp.write_text(_platform_stamp())
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    if LIB.exists() and LIB.stat().st_mtime >= max(o.stat().st_mtime for o in objs) and not force:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout[-4000:])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv)
    print("built", p)
