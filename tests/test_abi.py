"""The C ABI library loads and exports every entry point include/*.h declares."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

INCLUDE = Path(__file__).resolve().parents[1] / "include"


def declared_functions() -> list[str]:
    names = []
    for h in sorted(INCLUDE.glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        names += re.findall(r"\b(pgx_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "pgx_create" in names and "pgx_render" in names and "pgx_trace_closest" in names


def test_headers_compile_standalone(tmp_path):
    """pgx.h is valid C11 (for C FFI users) and pgx.hpp valid C++17, each
    included on its own."""
    import shutil
    import subprocess
    cc, cxx = shutil.which("gcc"), shutil.which("g++")
    if not cc or not cxx:
        import pytest
        pytest.skip("no host compiler")
    (tmp_path / "a.c").write_text('#include "pgx.h"\nint main(void) { return PGX_OK; }\n')
    (tmp_path / "b.cpp").write_text('#include "pgx.hpp"\nint main() { pgx::RayTracer rt; (void)rt; return 0; }\n')
    for comp, std, src in ((cc, "-std=c11", "a.c"), (cxx, "-std=c++17", "b.cpp")):
        r = subprocess.run([comp, std, "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only", "-I", str(INCLUDE),
                            str(tmp_path / src)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_library_exports_all_declared(pgx_lib):
    missing = [n for n in declared_functions() if not hasattr(pgx_lib, n)]
    assert not missing, missing


def test_signatures_cover_header(pgx_lib):
    from pathguidingdissertation_gb300 import abi
    assert set(declared_functions()) == set(abi.SIGNATURES)


def test_version_and_null_ctx(pgx_lib):
    assert pgx_lib.pgx_version().startswith(b"pgx")
    assert pgx_lib.pgx_destroy(None) == 0
    assert pgx_lib.pgx_bvh_build(None) == 1  # PGX_ERR_INVALID_ARG
    assert pgx_lib.pgx_guide_configure(None, None) == 1
    assert pgx_lib.pgx_guide_get_params(None, None) == 1
    assert pgx_lib.pgx_cache_export_weights(None, None, None) == 1


def test_create_without_gpu_fails_cleanly(pgx_lib):
    import torch
    if torch.cuda.is_available():
        import pytest
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = pgx_lib.pgx_create(0, ctypes.byref(h))
    assert rc != 0 and not h.value
    assert pgx_lib.pgx_last_error(None)
