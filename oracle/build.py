"""Build recipe for the oracle — test infrastructure only.

Two products, both loaded with ctypes by tests and by bench.py's CPU leg:

* ``oracle/_build/liboracle.so`` — the C restatement in pgx_oracle.c, built
  with ``-O2 -ffp-contract=off -fno-fast-math`` so float expressions keep the
  reference's rounding.
* ``oracle/_ref/liborcref.so`` (parity flags) and ``oracle/_ref/liborcref_fast.so``
  (``-O3``, timing) — the reference renderer itself, compiled headless.
  When the reference checkout is present its headers are staged into
  ``oracle/_ref/src`` with the platform header replaced by ``oracle/ref_shim``;
  on a machine without the checkout the staged copy, if any, is compiled.
  The reference's complete scenes (every mesh present) are staged into
  ``oracle/_ref/scenes`` so that tests can render them where the checkout is
  absent.  Nothing is written outside ``oracle/_ref`` and ``oracle/_build``.

The checkout is ``$PGX_REFERENCE_DIR`` (the project root holding
``PathGuidingDissertation/`` and ``Scenes/``; a path to the source directory
itself is accepted too), by default the directory ``reference`` beside this
repository.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
REF_SRC = REF_OUT / "src"
REF_SCENES = REF_OUT / "scenes"
# Reference scenes whose meshes are all present (the others name mesh files
# that are missing from the checkout, on which loadScene exits).
COMPLETE_SCENES = ["cornell-box", "veach-mis", "veach-bidir", "MaterialsScene", "staircase2", "living-room",
                   "dining-room"]
REF_HEADERS = [
    "MyMath.h", "Sampling.h", "Imaging.h", "Geometry.h", "Materials.h",
    "Lights.h", "Scene.h", "Renderer.h", "SceneLoader.h", "QuadTree.h", "Metrics.h",
]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout[-4000:])


def _newer(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(s.stat().st_mtime <= t for s in sources if s.exists())


def build_oracle(force: bool = False) -> Path:
    """Compile the C restatement into oracle/_build/liboracle.so."""
    BUILD.mkdir(parents=True, exist_ok=True)
    out = BUILD / "liboracle.so"
    srcs = [HERE / "pgx_oracle.c", HERE / "pgx_oracle.h", HERE / "pgx_oracle_rng.h",
            HERE.parent / "include" / "pgx.h"]
    if force or not _newer(out, srcs):
        tmp = out.with_suffix(".so.tmp")
        _run(["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
              "-pthread", str(HERE / "pgx_oracle.c"), "-o", str(tmp), "-lm"])
        os.replace(tmp, out)
    return out


def reference_root() -> Path:
    """The reference checkout's root (may not exist on this machine)."""
    env = os.environ.get("PGX_REFERENCE_DIR")
    if env:
        p = Path(env)
        return p.parent if (p / "Renderer.h").exists() else p
    return HERE.parent.parent / "reference"


def reference_sources() -> Path:
    return reference_root() / "PathGuidingDissertation"


def scenes_dir() -> Path:
    """The reference's scenes: the staged copy when present, else the checkout's."""
    return REF_SCENES if REF_SCENES.is_dir() else reference_root() / "Scenes"


def stage_scenes() -> None:
    """Copy the complete reference scenes into oracle/_ref/scenes."""
    src = reference_root() / "Scenes"
    if not src.is_dir():
        return
    for name in COMPLETE_SCENES:
        s, d = src / name, REF_SCENES / name
        if not s.is_dir():
            continue
        d.mkdir(parents=True, exist_ok=True)
        for f in s.iterdir():
            if f.is_file() and (not (d / f.name).exists() or (d / f.name).stat().st_size != f.stat().st_size):
                shutil.copy2(f, d / f.name)


def stage_reference(reference_dir: str | None = None) -> bool:
    """Copy the reference headers into oracle/_ref/src (returns False when
    neither the checkout nor a staged copy exists)."""
    ref = Path(reference_dir) if reference_dir else reference_sources()
    if ref.is_dir():
        REF_SRC.mkdir(parents=True, exist_ok=True)
        for h in REF_HEADERS:
            shutil.copy2(ref / h, REF_SRC / h)
        stb = REF_SRC / "ThirdParty" / "stb"
        stb.mkdir(parents=True, exist_ok=True)
        for f in (ref / "ThirdParty" / "stb").iterdir():
            shutil.copy2(f, stb / f.name)
        ge = REF_SRC / "ThirdParty" / "GamesEngineering"
        ge.mkdir(parents=True, exist_ok=True)
        shutil.copy2(ref / "ThirdParty" / "GamesEngineering" / "GEMLoader.h", ge / "GEMLoader.h")
    if not (REF_SRC / "Renderer.h").exists():
        return False
    ge = REF_SRC / "ThirdParty" / "GamesEngineering"
    ge.mkdir(parents=True, exist_ok=True)
    shutil.copy2(HERE / "ref_shim" / "ThirdParty" / "GamesEngineering" / "GamesEngineeringBase.h",
                 ge / "GamesEngineeringBase.h")
    return True


def build_reference(force: bool = False) -> Path | None:
    """Compile the reference harness; None when the reference is unavailable."""
    if not stage_reference():
        return None
    srcs = [HERE / "ref_harness.cpp", HERE / "ref_shim" / "prelude.h", HERE / "pgx_oracle_rng.h",
            HERE.parent / "include" / "pgx.h"] + [REF_SRC / h for h in REF_HEADERS]
    common = ["g++", "-std=c++20", "-fPIC", "-shared", "-pthread", "-w",
              "-include", str(HERE / "ref_shim" / "prelude.h"), "-I", str(REF_SRC),
              str(HERE / "ref_harness.cpp")]
    # Plain-integrator variant: the reference selects its integrator with the
    # compile-time switch `#define GUIDED_PATH true` (Renderer.h:25); the
    # plain build stages a copy of Renderer.h with that one value false.
    plain_dir = REF_OUT / "src_plain"
    plain_dir.mkdir(parents=True, exist_ok=True)
    text = (REF_SRC / "Renderer.h").read_text()
    if "#define GUIDED_PATH true" not in text:
        raise RuntimeError("Renderer.h: GUIDED_PATH switch not found")
    plain_h = plain_dir / "Renderer.h"
    new_text = text.replace("#define GUIDED_PATH true", "#define GUIDED_PATH false", 1)
    if not plain_h.exists() or plain_h.read_text() != new_text:
        plain_h.write_text(new_text)
    # SceneLoader.h includes "Renderer.h" from its own directory first, so the
    # plain variant needs its own copy beside the edited Renderer.h.
    loader_text = (REF_SRC / "SceneLoader.h").read_text()
    plain_loader = plain_dir / "SceneLoader.h"
    if not plain_loader.exists() or plain_loader.read_text() != loader_text:
        plain_loader.write_text(loader_text)
    outs = {
        "liborcref.so": ["-O2", "-ffp-contract=off", "-fno-fast-math"],
        "liborcref_fast.so": ["-O3"],
        "liborcref_plain_fast.so": ["-O3", "-I", str(plain_dir)],
    }
    procs = []
    for name, flags in outs.items():
        out = REF_OUT / name
        if force or not _newer(out, srcs + [plain_h]):
            tmp = out.with_suffix(".so.tmp")
            procs.append((subprocess.Popen(common[:1] + flags + common[1:] + ["-o", str(tmp)],
                                           stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True),
                          tmp, out))
    for p, tmp, out in procs:
        log, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("reference harness build failed:\n" + log[-4000:])
        os.replace(tmp, out)
    return REF_OUT / "liborcref.so"


def _stale_platform(d: Path) -> bool:
    import platform
    stamp = d / "platform.txt"
    stale = d.exists() and (not stamp.exists() or stamp.read_text() != platform.machine())
    d.mkdir(parents=True, exist_ok=True)
    stamp.write_text(platform.machine())
    return stale


def build(force: bool = False) -> None:
    build_oracle(force or _stale_platform(BUILD))
    build_reference(force or _stale_platform(REF_OUT))
    stage_scenes()


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print("oracle built:", BUILD / "liboracle.so", "reference:", REF_OUT / "liborcref.so")
