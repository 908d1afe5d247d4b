"""The C-ABI library loads and exports every entry point include/*.h declares."""
import ctypes as C
import os
import re

from fcl_gb300 import build as B
from fcl_gb300 import native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            names |= set(re.findall(r"FCLGPU_API\s+[\w\s\*]+?\b(fclgpu_\w+)\s*\(", txt))
    return names


def test_library_builds_and_exports_all_declared_symbols():
    path = B.build()
    lib = C.CDLL(path)
    declared = _declared()
    assert declared, "no declarations found"
    for name in declared:
        assert hasattr(lib, name), name
    assert declared <= set(N.exported_symbols()) | declared


def test_status_strings_without_gpu():
    L = N.lib()
    assert L.fclgpu_status_string(0) == b"ok"
    assert L.fclgpu_status_string(-4) == b"output capacity too small"


def test_header_is_plain_c(tmp_path):
    """include/fclgpu.h is a C header: it compiles as C99 with warnings as errors."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    src = tmp_path / "t.c"
    src.write_text('#include "fclgpu.h"\nint main(void) { return FCLGPU_OK; }\n')
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only",
                        "-I", os.path.join(ROOT, "include"), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_fcl_binding_compiles():
    """The binding a maintainer would add inside FCL (tests/native/fcl_shim_check.cpp:
    fcl::collide with and without contact geometry, fcl::continuousCollide, a broadphase
    manager's collide forms) compiles against include/fclgpu.h with stand-ins for the
    FCL types it touches."""
    import shutil
    import subprocess
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        import pytest
        pytest.skip("no C++ compiler")
    src = os.path.join(ROOT, "tests", "native", "fcl_shim_check.cpp")
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only",
                        "-I", os.path.join(ROOT, "include"), src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
