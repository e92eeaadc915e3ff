"""Loader of the GPU library (ctypes).

There is no CPU fallback: if the library is absent it is built from
``csrc/`` with nvcc, and if that fails the error propagates.
"""
import ctypes
import os
import threading

from .. import build as _build

_lock = threading.Lock()
_handles = {}


def library_path():
    return os.path.join(_build.LIBDIR, _build.LIBNAME)


def shim_path(dimension, variable_density, float64):
    return os.path.join(_build.LIBDIR, _build.shim_name(
        dimension, 1 if variable_density else 0, 1 if float64 else 0))


def ensure_built():
    """Build the library if any of its files is missing."""
    needed = [library_path()] + [
        shim_path(d, vd, f) for d, vd, f in _build.VARIANTS]
    if not all(os.path.exists(p) for p in needed):
        _build.build()


def load(path=None):
    """ctypes handle of ``path`` (default: libsimwave_gb300.so)."""
    with _lock:
        ensure_built()
        path = path or library_path()
        if path not in _handles:
            _handles[path] = ctypes.CDLL(path)
        return _handles[path]


def last_error():
    lib = load()
    lib.simwave_last_error.restype = ctypes.c_char_p
    msg = lib.simwave_last_error()
    return msg.decode() if msg else ""


class Stats(ctypes.Structure):
    """Mirror of ``simwave_stats`` (include/simwave_gb300.h)."""
    _fields_ = [("seconds", ctypes.c_double),
                ("stencil_ms", ctypes.c_double),
                ("updates", ctypes.c_double),
                ("stencil_launches", ctypes.c_size_t),
                ("kernel_launches", ctypes.c_size_t),
                ("h2d_bytes", ctypes.c_size_t),
                ("d2h_bytes", ctypes.c_size_t),
                ("stencil_variant", ctypes.c_int),
                ("stencil_kernel", ctypes.c_int)]


def last_stats():
    lib = load()
    out = Stats()
    lib.simwave_last_stats(ctypes.byref(out))
    return {name: getattr(out, name) for name, _ in Stats._fields_}
