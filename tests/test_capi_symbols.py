"""The C ABI library loads and exports every entry point include/pbr_capi.h
declares (no compute calls: runs without a GPU)."""
import ctypes
import os
import re

import pytest

from pybatchrender_gb300 import _capi
from pybatchrender_gb300.build import LIB_PATH, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions() -> list[str]:
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(pbr_[a-z_0-9]+)\s*\(", text, flags=re.M)
    return names


@pytest.fixture(scope="module")
def lib():
    build()
    return ctypes.CDLL(LIB_PATH)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "pbr_render" in names and "pbr_create" in names and len(names) >= 15


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"missing exports: {missing}"


def test_python_binding_covers_every_symbol():
    names = set(declared_functions()) - {"pbr_last_error"}
    assert names <= set(_capi.SIGNATURES), sorted(names - set(_capi.SIGNATURES))


def test_version_and_error_paths_without_gpu(lib):
    lib.pbr_version.restype = ctypes.c_int
    assert lib.pbr_version() >= 100
    lib.pbr_last_error.restype = ctypes.c_char_p
    lib.pbr_last_error.argtypes = [ctypes.c_void_p]
    ctx = ctypes.c_void_p()
    # invalid arguments are rejected before any CUDA call
    rc = lib.pbr_create(ctypes.byref(ctx), 0, 64, 64, 3, 0)
    assert rc == _capi.PBR_ERR_INVALID
    assert b"positive" in lib.pbr_last_error(None)
    rc = lib.pbr_create(ctypes.byref(ctx), 4, 64, 64, 7, 0)
    assert rc == _capi.PBR_ERR_INVALID
    assert lib.pbr_render(None, None, None, None, None) == _capi.PBR_ERR_INVALID


def test_cartpole_step_argument_checks_without_gpu(lib):
    """pbr_cartpole_step validates its arguments before any CUDA call."""
    f = lib.pbr_cartpole_step
    f.restype = ctypes.c_int
    f.argtypes = _capi.SIGNATURES["pbr_cartpole_step"]
    consts = (ctypes.c_double * 9)(9.8, 1.0, 0.1, 0.5, 10.0, 0.02, 2.4, 0.2, 500)
    p16, p20 = 0x10000, 0x10004  # aligned / misaligned stand-in addresses, never dereferenced
    args = [p16, p16, None, None, None, None, None, p16, p16, p16, p16, p16]
    assert f(*args, 0, consts, 0, None) == _capi.PBR_OK                     # no scenes: nothing to do
    assert f(*args, -1, consts, 0, None) == _capi.PBR_ERR_INVALID
    assert f(*args, 8, None, 0, None) == _capi.PBR_ERR_INVALID
    assert f(*args, 8, consts, 1, None) == _capi.PBR_ERR_INVALID             # auto-reset needs the reset states
    bad = list(args)
    bad[0] = p20
    assert f(*bad, 8, consts, 0, None) == _capi.PBR_ERR_INVALID              # [n,4] arrays must be 16-byte aligned
    bad = list(args)
    bad[1] = None
    assert f(*bad, 8, consts, 0, None) == _capi.PBR_ERR_INVALID


def test_camera_update_validates_before_any_cuda_call(lib):
    """pbr_camera_update takes no context: a missing view buffer, a view-projection
    without a projection, or a negative scene count are rejected before any
    launch; zero scenes is a no-op."""
    f = lib.pbr_camera_update
    f.argtypes, f.restype = _capi.SIGNATURES["pbr_camera_update"], ctypes.c_int
    P = (ctypes.c_float * 16)()
    assert f(None, None, None, None, P, None, 4, None) == _capi.PBR_ERR_INVALID
    assert f(None, None, None, 1024, None, 2048, 4, None) == _capi.PBR_ERR_INVALID
    assert f(None, None, None, 1024, P, None, -1, None) == _capi.PBR_ERR_INVALID
    assert f(None, None, None, 1024, P, 2048, 0, None) == _capi.PBR_OK


_NULL_CTX_PROBE = r"""
import ctypes, sys
from pybatchrender_gb300 import _capi
from pybatchrender_gb300.build import LIB_PATH
lib = ctypes.CDLL(LIB_PATH)
lib.pbr_last_error.restype = ctypes.c_char_p
lib.pbr_last_error.argtypes = [ctypes.c_void_p]
bad = []
for name, sig in _capi.SIGNATURES.items():
    if not sig or sig[0] is not ctypes.c_void_p or name in ("pbr_destroy", "pbr_cartpole_step", "pbr_camera_update"):
        continue
    args = []
    for t in sig:
        if t in (ctypes.c_int, ctypes.c_long, ctypes.c_longlong):
            args.append(0)
        elif t in (ctypes.c_float, ctypes.c_double):
            args.append(0.0)
        elif isinstance(t, type) and issubclass(t, ctypes.Array):
            args.append(t())
        else:
            args.append(None)
    f = getattr(lib, name)
    f.argtypes, f.restype = sig, ctypes.c_int
    rc = f(*args)
    if rc != _capi.PBR_ERR_INVALID or lib.pbr_last_error(None) != b"null context":
        bad.append((name, rc))
print("checked", len([n for n in _capi.SIGNATURES]), "bad", bad)
sys.exit(1 if bad else 0)
"""


def test_every_context_call_rejects_a_null_context(lib):
    """Each entry point that takes a context returns PBR_ERR_INVALID for a
    null one before touching anything (run in a child process, so that a
    missing check cannot take the test session down)."""
    import subprocess
    import sys
    res = subprocess.run([sys.executable, "-c", _NULL_CTX_PROBE], cwd=ROOT, capture_output=True, text=True,
                         timeout=120)
    assert res.returncode == 0, res.stdout + res.stderr
