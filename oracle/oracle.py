"""ctypes front for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module; the product package never imports it.

Two native back ends share one calling convention, the reference's
``forward(...)`` argument order (simwave/kernel/backend/middleware.py:160-204):

* ``port``: ``oracle/_build/liboracle.so``, the C restatement in
  ``wave_oracle.c`` (always buildable, here and on the GPU machine);
* ``ref``: ``oracle/_ref/ref_<d>d_<cd|vd>_<f32|f64>_<c|omp>.so``, the
  reference's own kernels compiled by ``make -C oracle ref`` (only where the
  reference tree exists).

``forward(backend, **kwargs)`` takes the same keyword arguments the
reference's ``Middleware.exec('forward', ...)`` receives from
``Solver.forward`` (solver.py:121-161) and returns ``(u_full, shot_record,
seconds)``; ``u_full`` and ``shot_record`` are updated in place.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")

_BC_CODES = {'none': 0, 'null_dirichlet': 1, 'null_neumann': 2}

# argument keys in the reference's C order (middleware.py:160-204)
_ORDER = [
    'u_full', 'velocity_model', 'density_model', 'damping_mask', 'wavelet',
    'wavelet_size', 'wavelet_count', 'second_order_fd_coefficients',
    'first_order_fd_coefficients', 'boundary_condition',
    'src_points_interval', 'src_points_interval_size', 'src_points_values',
    'src_points_values_size', 'src_points_values_offset',
    'rec_points_interval', 'rec_points_interval_size', 'rec_points_values',
    'rec_points_values_size', 'rec_points_values_offset', 'shot_record',
    'num_sources', 'num_receivers', 'nz', 'nx', 'ny', 'dz', 'dx', 'dy',
    'saving_stride', 'dt', 'begin_timestep', 'end_timestep', 'space_order',
    'num_snapshots',
]
_SIZE_KEYS = {
    'wavelet_size', 'wavelet_count', 'src_points_interval_size',
    'src_points_values_size', 'rec_points_interval_size',
    'rec_points_values_size', 'num_sources', 'num_receivers', 'nz', 'nx',
    'ny', 'saving_stride', 'begin_timestep', 'end_timestep', 'space_order',
    'num_snapshots',
}
_REAL_SCALARS = {'dz', 'dx', 'dy', 'dt'}
_INDEX_ARRAYS = {'boundary_condition', 'src_points_interval',
                 'src_points_values_offset', 'rec_points_interval',
                 'rec_points_values_offset'}

_LIBS = {}


def build_port():
    """Compile liboracle.so (make -C oracle)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def _port_lib():
    path = os.path.join(BUILD_DIR, "liboracle.so")
    if not os.path.exists(path):
        build_port()
    if path not in _LIBS:
        _LIBS[path] = ctypes.CDLL(path)
    return _LIBS[path]


def ref_available():
    return os.path.isdir(REF_DIR) and any(
        f.endswith(".so") for f in os.listdir(REF_DIR))


def _ref_lib(dim, vd, tag, language):
    path = os.path.join(REF_DIR, "ref_{}d_{}_{}_{}.so".format(
        dim, 'vd' if vd else 'cd', tag, language))
    if not os.path.exists(path):
        raise FileNotFoundError(
            "{} missing: run `make -C oracle ref` where the reference "
            "sources exist".format(path))
    if path not in _LIBS:
        _LIBS[path] = ctypes.CDLL(path)
    return _LIBS[path]


def _normalise(kwargs):
    """Same key rewriting as middleware.py:53-105."""
    kw = dict(kwargs)
    bc = kw['boundary_condition']
    kw['boundary_condition'] = np.asarray(
        [_BC_CODES[b] if isinstance(b, str) else int(b) for b in bc],
        dtype=np.uint64)
    if kw.get('density_model') is None:
        kw.pop('density_model', None)
        kw.pop('first_order_fd_coefficients', None)
    shape = kw['velocity_model'].shape
    for key, val in zip(('nz', 'nx', 'ny'), shape):
        kw[key] = val
    spacing = kw.pop('grid_spacing')
    for key, val in zip(('dz', 'dx', 'dy'), spacing):
        kw[key] = val
    return kw


def forward(backend="port", x_stride="reference", language="c", **kwargs):
    """Run the CPU forward loop on the reference's argument list.

    backend: "port" (the restatement) or "ref" (reference kernels).
    x_stride: for the 3D variable-density port only, "reference" keeps the
        reference's x first-derivative stride nx, "layout" uses ny.
    language: for "ref", "c" (sequential) or "omp" (cpu_openmp build).
    """
    kw = _normalise(kwargs)
    vel = kw['velocity_model']
    dim = vel.ndim
    vd = 'density_model' in kw
    dtype = vel.dtype
    real = ctypes.c_float if dtype == np.float32 else ctypes.c_double
    tag = 'f32' if dtype == np.float32 else 'f64'
    args, types = [], []
    for key in _ORDER:
        if key not in kw or kw[key] is None:
            continue
        val = kw[key]
        if key in _INDEX_ARRAYS:
            arr = np.ascontiguousarray(val, dtype=np.uint64)
            kw[key] = arr
            args.append(arr.ctypes.data_as(ctypes.c_void_p))
            types.append(ctypes.c_void_p)
        elif isinstance(val, np.ndarray):
            if val.dtype != dtype or not val.flags['C_CONTIGUOUS']:
                raise TypeError("{} must be C-contiguous {}".format(key, dtype))
            args.append(val.ctypes.data_as(ctypes.c_void_p))
            types.append(ctypes.c_void_p)
        elif key in _SIZE_KEYS:
            args.append(int(val))
            types.append(ctypes.c_size_t)
        elif key in _REAL_SCALARS:
            args.append(float(val))
            types.append(real)
        else:
            raise TypeError("unexpected argument " + key)
    if backend == "port":
        lib = _port_lib()
        name = "oracle_forward_{}d_{}_{}".format(
            dim, ('vdfix' if x_stride == "layout" and dim == 3 else 'vd')
            if vd else 'cd', tag)
        fn = getattr(lib, name)
    elif backend == "ref":
        fn = _ref_lib(dim, vd, tag, language).forward
    else:
        raise ValueError(backend)
    fn.restype = ctypes.c_double
    fn.argtypes = types
    seconds = fn(*args)
    return kwargs['u_full'], kwargs['shot_record'], seconds


def problem_kwargs(space_model, time_model, sources, receivers, wavelet,
                   u_full=None):
    """The keyword arguments ``Solver.forward`` hands to the middleware.

    Restates the marshalling at simwave/kernel/frontend/solver.py:121-161 for
    front-end objects of either this package's front end or the reference's.
    """
    src_points, src_values, src_offsets = sources.interpolated_points_and_values
    rec_points, rec_values, rec_offsets = receivers.interpolated_points_and_values
    T = time_model.timesteps
    stride = time_model.saving_stride
    nsnap = 1 if stride == 0 else len(range(0, T, stride))
    if u_full is None:
        u_full = np.zeros((nsnap + 2,) + tuple(space_model.extended_shape),
                          dtype=space_model.dtype)
    return dict(
        u_full=u_full,
        velocity_model=space_model.extended_velocity_model,
        density_model=space_model.extended_density_model,
        damping_mask=space_model.damping_mask,
        wavelet=wavelet.values,
        wavelet_size=wavelet.timesteps,
        wavelet_count=wavelet.num_sources,
        second_order_fd_coefficients=space_model.fd_coefficients(2),
        first_order_fd_coefficients=space_model.fd_coefficients(1),
        boundary_condition=space_model.boundary_condition,
        src_points_interval=src_points,
        src_points_interval_size=len(src_points),
        src_points_values=src_values,
        src_points_values_offset=src_offsets,
        src_points_values_size=len(src_values),
        rec_points_interval=rec_points,
        rec_points_interval_size=len(rec_points),
        rec_points_values=rec_values,
        rec_points_values_offset=rec_offsets,
        rec_points_values_size=len(rec_values),
        shot_record=np.zeros((T, receivers.count), dtype=space_model.dtype),
        num_sources=sources.count,
        num_receivers=receivers.count,
        grid_spacing=space_model.grid_spacing,
        saving_stride=stride,
        dt=time_model.dt,
        begin_timestep=1,
        end_timestep=T,
        space_order=space_model.space_order,
        num_snapshots=nsnap + 2,
    )
