"""ctypes binding of ``libpbr.so`` (declared in ``include/pbr_capi.h``).

The product path has no fallback: if the library cannot be loaded, every call
that would render raises :class:`RendererUnavailable`.
"""
from __future__ import annotations

import ctypes
import os
import threading

from .build import LIB_PATH

PBR_OK = 0
PBR_ERR_INVALID = 1
PBR_ERR_CUDA = 2
PBR_ERR_CAPACITY = 3
PBR_ERR_STATE = 4
PBR_ERR_DEVICE = 5

MODE_HPR, MODE_ROT, MODE_MAT = 0, 1, 2

_vp = ctypes.c_void_p
_i = ctypes.c_int
_f = ctypes.c_float
_pi = ctypes.POINTER(ctypes.c_int)
_pf = ctypes.POINTER(ctypes.c_float)
_f3 = ctypes.c_float * 3
_f4 = ctypes.c_float * 4

# name -> argtypes; every function returns int except pbr_last_error
SIGNATURES: dict[str, list] = {
    "pbr_version": [],
    "pbr_create": [ctypes.POINTER(_vp), _i, _i, _i, _i, _i],
    "pbr_destroy": [_vp],
    "pbr_mesh_register": [_vp, _vp, _vp, _vp, _i, _i, _i, _pi],
    "pbr_mesh_set_bounds": [_vp, _i, _f, _f, _f, _f],
    "pbr_mesh_set_uv": [_vp, _i, _vp],
    "pbr_mesh_set_clusters": [_vp, _i, _vp, _i, _i],
    "pbr_node_add": [_vp, _i, _i, _i, _pi],
    "pbr_node_set_texture": [_vp, _i, _vp, _i, _i],
    "pbr_node_set_buffers": [_vp, _i, _i, _vp, _vp, _vp, _vp, _vp],
    "pbr_camera_bind": [_vp, _vp, _f, _f],
    "pbr_light_set": [_vp, _f3, _f3, _f3, _f],
    "pbr_background_set": [_vp, _f4],
    "pbr_raster_config": [_vp, _i, _i, _i, _i, _i],
    "pbr_tile_pretest": [_vp, _i],
    "pbr_autotune": [_vp, _vp, _vp, _pi, _pi, _pi, _pi, _pi, _pf],
    "pbr_render": [_vp, _vp, _vp, _vp, _vp],
    "pbr_node_bind_state": [_vp, _i, _i, _i],
    "pbr_state_source": [_vp, _vp, ctypes.c_longlong, _i, ctypes.c_longlong],
    "pbr_render_state": [_vp, _vp, ctypes.c_longlong, _i, ctypes.c_longlong, _vp, _vp, _vp, _vp],
    "pbr_plain_clear": [_vp, _vp],
    "pbr_plain_draw": [_vp, _i, _vp],
    "pbr_plain_resolve": [_vp, _vp, _vp, _vp],
    "pbr_plain_render_noalloc": [_vp, _vp, _vp, _vp],
    "pbr_soft_config": [_vp, _f, _f, _i],
    "pbr_node_set_grads": [_vp, _i, _vp, _vp, _vp, _vp],
    "pbr_render_soft": [_vp, _vp, _vp, _vp],
    "pbr_backward_soft": [_vp, _vp, _vp, _vp, _vp, _vp],
    "pbr_debug_transforms": [_vp, _i, _vp, _vp],
    "pbr_device_status": [_vp, ctypes.POINTER(ctypes.c_int32)],
    "pbr_camera_update": [_vp, _vp, _vp, _vp, ctypes.POINTER(ctypes.c_float), _vp, _i, _vp],
    "pbr_cartpole_step": [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_longlong,
                          ctypes.POINTER(ctypes.c_double), _i, _vp],
}


class RendererUnavailable(RuntimeError):
    """The CUDA renderer library could not be loaded or no GPU is present."""


class PBRError(RuntimeError):
    """A C ABI call returned a non-zero status."""

    def __init__(self, func: str, code: int, message: str):
        super().__init__(f"{func} failed (status {code}): {message}")
        self.func, self.code, self.message = func, code, message


_lib = None
_lock = threading.Lock()


def library_path() -> str:
    return LIB_PATH


def load(build_if_missing: bool = False) -> ctypes.CDLL:
    """Load ``libpbr.so`` (optionally building it first) and declare its
    signatures.  Raises :class:`RendererUnavailable` when it is missing."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            if not build_if_missing:
                raise RendererUnavailable(
                    f"{LIB_PATH} is missing; build it with `python -m pybatchrender_gb300.build` "
                    "(the renderer has no CPU fallback)")
            from .build import build
            build()
        try:
            import torch  # noqa: F401  (loads the CUDA runtime that libpbr shares)
        except Exception:  # pragma: no cover
            pass
        try:
            lib = ctypes.CDLL(LIB_PATH)
        except OSError as e:
            raise RendererUnavailable(f"cannot load {LIB_PATH}: {e}") from e
        for name, argtypes in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = argtypes
            fn.restype = ctypes.c_int
        lib.pbr_last_error.argtypes = [_vp]
        lib.pbr_last_error.restype = ctypes.c_char_p
        _lib = lib
        return lib


def call(lib: ctypes.CDLL, ctx, name: str, *args) -> None:
    """Call ``name(ctx, *args)`` and raise :class:`PBRError` on failure."""
    rc = getattr(lib, name)(ctx, *args)
    if rc != PBR_OK:
        msg = lib.pbr_last_error(ctx).decode("utf-8", "replace")
        raise PBRError(name, rc, msg)


def ptr(t) -> int | None:
    """Raw device pointer of a tensor (None for None)."""
    return None if t is None else t.data_ptr()
