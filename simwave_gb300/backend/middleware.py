"""Python -> C-ABI glue mirroring simwave's ``Middleware`` (middleware.py).

``exec('forward', **kwargs)`` takes the keyword arguments ``Solver.forward``
builds (solver.py:121-161), applies the reference's conversions (boundary
names -> uint64 codes, density-less calls drop the density and first-order
weights, grid shape and spacing unpacked; middleware.py:53-105), loads the
variant's library and calls its ``forward`` with the reference's argument
order (middleware.py:160-204).
"""
import ctypes

import numpy as np

from . import _lib
from .compiler import Compiler

_BC = {'none': 0, 'null_dirichlet': 1, 'null_neumann': 2}

KEY_ORDER = [
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

_INT_KEYS = {
    'wavelet_size', 'wavelet_count', 'src_points_interval_size',
    'src_points_values_size', 'rec_points_interval_size',
    'rec_points_values_size', 'num_sources', 'num_receivers', 'nz', 'nx',
    'ny', 'saving_stride', 'begin_timestep', 'end_timestep', 'space_order',
    'num_snapshots'}
_REAL_KEYS = {'dz', 'dx', 'dy', 'dt'}
_INDEX_KEYS = {'boundary_condition', 'src_points_interval',
               'src_points_values_offset', 'rec_points_interval',
               'rec_points_values_offset'}


def convert_boundary_condition(boundary_condition):
    """Names to codes: none 0, null_dirichlet 1, null_neumann 2."""
    return np.asarray([_BC[b] for b in boundary_condition], dtype=np.uint64)


def normalise(kwargs):
    """The reference's argument rewriting (middleware.py:53-105)."""
    kw = dict(kwargs)
    kw['boundary_condition'] = convert_boundary_condition(
        kw['boundary_condition'])
    if kw.get('density_model') is None:
        kw.pop('density_model', None)
        kw.pop('first_order_fd_coefficients', None)
    shape = kw['velocity_model'].shape
    if len(shape) not in (2, 3):
        raise ValueError("velocity model must be 2D or 3D")
    for key, val in zip(('nz', 'nx', 'ny'), shape):
        kw[key] = val
    for key, val in zip(('dz', 'dx', 'dy'), kw.pop('grid_spacing')):
        kw[key] = val
    return kw


def ordered_arguments(kw):
    """``(args, argtypes)`` in the C order; arrays are checked for dtype and
    contiguity (the reference's ``ndpointer(..., C_CONTIGUOUS)``)."""
    dtype = kw['velocity_model'].dtype
    if dtype not in (np.float32, np.float64):
        raise TypeError("models must be float32 or float64")
    real = ctypes.c_float if dtype == np.float32 else ctypes.c_double
    args, types = [], []
    for key in KEY_ORDER:
        if key not in kw or kw[key] is None:
            continue
        val = kw[key]
        if key in _INDEX_KEYS:
            arr = np.asarray(val)
            if arr.dtype != np.uint64 or not arr.flags['C_CONTIGUOUS']:
                raise TypeError("{} must be C-contiguous uint64".format(key))
            args.append(arr.ctypes.data_as(ctypes.c_void_p))
            types.append(ctypes.c_void_p)
        elif isinstance(val, np.ndarray):
            if val.dtype != dtype or not val.flags['C_CONTIGUOUS']:
                raise TypeError("{} must be C-contiguous {}".format(key, dtype))
            args.append(val.ctypes.data_as(ctypes.c_void_p))
            types.append(ctypes.c_void_p)
        elif key in _INT_KEYS:
            args.append(int(val))
            types.append(ctypes.c_size_t)
        elif key in _REAL_KEYS:
            args.append(float(val))
            types.append(real)
        else:
            raise TypeError("unexpected argument {}".format(key))
    return args, types


class Middleware:
    """Communication between the front end and the GPU library."""

    def __init__(self, compiler=None):
        self._compiler = Compiler() if compiler is None else compiler

    @property
    def compiler(self):
        return self._compiler

    def library(self, dimension, density, dtype):
        """ctypes handle of the variant's library (middleware.py:26-51)."""
        precision = {'float32': '-DFLOAT', 'float64': '-DDOUBLE'}[str(dtype)]
        path = self.compiler.compile(
            dimension=dimension,
            density="variable_density" if density is not None
            else "constant_density",
            float_precision=precision, operator="forward")
        _lib.load()  # the shims resolve their calls in the main library
        return _lib.load(path)

    def exec(self, operator, **kwargs):
        if operator != 'forward':
            raise ValueError("Only forward operator available.")
        return self._exec_forward(**normalise(kwargs))

    def _exec_forward(self, **kw):
        vel = kw['velocity_model']
        lib = self.library(vel.ndim, kw.get('density_model'), vel.dtype)
        args, types = ordered_arguments(kw)
        fn = lib.forward
        fn.restype = ctypes.c_double
        fn.argtypes = types
        seconds = fn(*args)
        if seconds < 0:
            raise RuntimeError("simwave GPU forward failed ({}): {}".format(
                int(-seconds), _lib.last_error()))
        print('Run forward in %f seconds.' % seconds)
        return kw['u_full'], kw['shot_record']
