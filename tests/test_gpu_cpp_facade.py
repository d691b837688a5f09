"""The C++ façade (include/pgx.hpp) compiles against the C ABI and renders."""
from __future__ import annotations

import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _build_example(tmp_path, pgx_lib):
    exe = tmp_path / "render_box"
    lib_dir = ROOT / "pathguidingdissertation_gb300"
    cmd = ["g++", "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(ROOT / "tests" / "cpp" / "render_box.cpp"),
           "-L", str(lib_dir), "-lpgx", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_facade_compiles(tmp_path, pgx_lib):
    assert _build_example(tmp_path, pgx_lib).exists()


@pytest.mark.gpu
def test_cpp_facade_renders(tmp_path, pgx_lib):
    exe = _build_example(tmp_path, pgx_lib)
    out = tmp_path / "box.hdr"
    r = subprocess.run([str(exe), str(out)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "spp=8" in r.stdout and "expected error" in r.stdout
    assert out.stat().st_size > 64 * 64 * 4
