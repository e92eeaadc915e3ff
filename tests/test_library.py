"""The C-ABI library: builds, loads without a GPU, exports every symbol the
header declares, rejects bad arguments before touching the device, and the
Python drop-in layer mirrors the reference's Compiler/Middleware."""
import ctypes
import os
import re

import numpy as np
import pytest

import simwave_gb300 as sw
from simwave_gb300 import build
from simwave_gb300.backend import _lib
from simwave_gb300.backend.middleware import (Middleware, normalise,
                                              ordered_arguments)
from _cases import fixture_kwargs

HEADER = os.path.join(os.path.dirname(build.HERE), "include", "simwave_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(simwave_\w+)\s*\(",
                                 text, flags=re.M)))


def test_header_declares_expected_entry_points():
    names = declared_functions()
    for d in (2, 3):
        for v in ("cd", "vd"):
            for p in ("f32", "f64"):
                assert "simwave_forward_{}d_{}_{}".format(d, v, p) in names
    for extra in ("simwave_last_error", "simwave_forward_device",
                  "simwave_last_stats", "simwave_layout"):
        assert extra in names


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_shims_export_forward():
    for d, vd, f64 in build.VARIANTS:
        lib = _lib.load(_lib.shim_path(d, vd, f64))
        assert hasattr(lib, "forward")


def test_layout_query():
    from simwave_gb300.device import layout
    pitch, lead = layout(472, 8, 4)
    assert (lead + 4) * 4 % 128 == 0 and pitch >= lead + 472 and pitch % 32 == 0
    pitch, lead = layout(517, 4, 8)
    assert (lead + 2) * 8 % 128 == 0 and pitch >= lead + 517


def test_invalid_order_rejected_before_device_use():
    kw, *_ = fixture_kwargs("2d_cd_so4_mixed_s0_f32")
    kw["space_order"] = 5
    nkw = normalise(kw)
    args, types = ordered_arguments(nkw)
    lib = _lib.load()
    fn = lib.simwave_forward_2d_cd_f32
    fn.restype = ctypes.c_double
    fn.argtypes = types
    status = fn(*args)
    assert status == -1.0
    assert "space_order" in _lib.last_error()


def test_window_outside_grid_rejected():
    kw, *_ = fixture_kwargs("2d_cd_so4_mixed_s0_f32")
    iv = kw["rec_points_interval"].copy()
    iv[1] = kw["velocity_model"].shape[0] + 3
    kw["rec_points_interval"] = iv
    args, types = ordered_arguments(normalise(kw))
    fn = _lib.load().simwave_forward_2d_cd_f32
    fn.restype = ctypes.c_double
    fn.argtypes = types
    assert fn(*args) == -1.0
    assert "outside the grid" in _lib.last_error()


def test_slot_shortage_rejected():
    kw, *_ = fixture_kwargs("2d_cd_so12_s1_f32")  # stride 1 needs T + 2 slots
    kw["num_snapshots"] = 5
    kw["u_full"] = kw["u_full"][:5].copy()
    args, types = ordered_arguments(normalise(kw))
    fn = _lib.load().simwave_forward_2d_cd_f32
    fn.restype = ctypes.c_double
    fn.argtypes = types
    assert fn(*args) == -2.0
    assert "slot" in _lib.last_error()


def test_compiler_mirrors_reference_whitelist():
    assert sw.Compiler().language == "cuda_sm100a"
    assert sw.Compiler(language="cuda_sm103a").language == "cuda_sm103a"
    for bad in ("c", "cpu_openmp", "cuda", "cpu_mpi"):
        with pytest.raises(ValueError):
            sw.Compiler(language=bad)
    with pytest.raises(TypeError):
        sw.Compiler(cc=3)
    path = sw.Compiler().compile(3, "variable_density", "-DFLOAT", "forward")
    assert path.endswith("libsimwave_forward_3d_vd_f32.so")
    with pytest.raises(ValueError):
        sw.Compiler().compile(3, "variable_density", "-DFLOAT", "adjoint")


def test_middleware_argument_order_matches_reference():
    kw, *_ = fixture_kwargs("3d_vd_so8_cube_s4_f32")
    nkw = normalise(kw)
    args, types = ordered_arguments(nkw)
    # u, vel, den, damp, wavelet, 2 sizes, c2, c1, bc, 5 src, 5 rec, rec,
    # nsrc, nrec, nz, nx, ny, dz, dx, dy, stride, dt, begin, end, order, nsnap
    # (variable_density/3d/wave.c:23-36)
    assert len(args) == 35
    assert types[-7] == ctypes.c_float  # dy
    assert types[-5] == ctypes.c_float  # dt
    assert types[-6] == ctypes.c_size_t  # saving_stride
    kw2, *_ = fixture_kwargs("2d_cd_so4_mixed_s0_f32")
    assert len(ordered_arguments(normalise(kw2))[0]) == 31
    mw = Middleware()
    assert mw.compiler.language == "cuda_sm100a"
