"""CPU checks of the C ABI: the built library loads and exports every
function that include/jif3d_gb300.h declares; without a GPU it refuses to
create a context instead of falling back to the CPU."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in sorted(os.listdir(os.path.join(ROOT, "include")))
           if f.endswith(".h")]


def declared_functions():
    names = []
    for h in HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-z_ ]+\s*\*?\s*(j3g_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from jif3d_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_functions():
    names = declared_functions()
    assert "j3g_forward" in names and "j3g_lqderivative" in names and len(names) >= 15


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from jif3d_gb300 import capi
    assert set(declared_functions()) == set(capi.SIGNATURES), \
        set(declared_functions()) ^ set(capi.SIGNATURES)


def test_status_strings(lib):
    f = lib.j3g_status_string
    f.restype = ctypes.c_char_p
    assert f(0) == b"ok"
    assert f(2) == b"CUDA error"
    assert f(99) == b"unknown status"


def test_no_cpu_fallback_without_gpu(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = lib.j3g_create(ctypes.byref(h), 0)
    assert rc != 0 and not h.value
    from jif3d_gb300 import capi
    with pytest.raises(capi.J3GError):
        capi.Context(0)


def test_null_context_is_rejected(lib):
    lib.j3g_forward.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    assert lib.j3g_forward(None, None, None) == 1
    assert lib.j3g_destroy(None) == 0


def test_cpp_implementation_header_compiles():
    """The C++ implementation objects and the refiner compile against the
    stand-in jif3D declarations (no GPU needed: syntax and template
    instantiation only)."""
    import shutil
    import subprocess
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for src in ("host_adapter_check.cpp", "refiner_check.cpp"):
        r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-Werror",
                            "-I", os.path.join(root, "include"),
                            "-I", os.path.join(root, "jif3d_gb300", "host"),
                            os.path.join(root, "tests", "cpp", src)],
                           capture_output=True, text=True)
        assert r.returncode == 0, (src, r.stderr)
