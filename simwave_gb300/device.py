"""Device-resident forward problems (torch tensors + ``simwave_forward_device``).

PyTorch provides the device memory and streams; the computation is the C
library's. Grids are stored in the library's pitched layout (each row of the
fastest axis starts so that the first interior point is 128-byte aligned),
exposed as views of the logical ``(nz, nx[, ny])`` shape.
"""
import ctypes

import numpy as np
import torch

from .backend import _lib
from .backend.middleware import normalise


class Problem(ctypes.Structure):
    """Mirror of ``simwave_problem`` (include/simwave_gb300.h)."""
    _fields_ = [
        ("dim", ctypes.c_int), ("variable_density", ctypes.c_int),
        ("precision", ctypes.c_int), ("space_order", ctypes.c_int),
        ("nz", ctypes.c_size_t), ("nx", ctypes.c_size_t),
        ("ny", ctypes.c_size_t), ("pitch", ctypes.c_size_t),
        ("lead", ctypes.c_size_t), ("slot_stride", ctypes.c_size_t),
        ("dz", ctypes.c_double), ("dx", ctypes.c_double),
        ("dy", ctypes.c_double), ("dt", ctypes.c_double),
        ("u", ctypes.c_void_p), ("num_snapshots", ctypes.c_size_t),
        ("velocity", ctypes.c_void_p), ("density", ctypes.c_void_p),
        ("damp", ctypes.c_void_p), ("wavelet", ctypes.c_void_p),
        ("wavelet_size", ctypes.c_size_t), ("wavelet_count", ctypes.c_size_t),
        ("coeff_order2", ctypes.c_void_p), ("coeff_order1", ctypes.c_void_p),
        ("boundary_conditions", ctypes.c_void_p),
        ("src_points_interval", ctypes.c_void_p),
        ("src_points_values", ctypes.c_void_p),
        ("src_points_values_offset", ctypes.c_void_p),
        ("src_points_values_size", ctypes.c_size_t),
        ("num_sources", ctypes.c_size_t),
        ("rec_points_interval", ctypes.c_void_p),
        ("rec_points_values", ctypes.c_void_p),
        ("rec_points_values_offset", ctypes.c_void_p),
        ("rec_points_values_size", ctypes.c_size_t),
        ("num_receivers", ctypes.c_size_t),
        ("receivers", ctypes.c_void_p),
        ("saving_stride", ctypes.c_size_t),
        ("begin_timestep", ctypes.c_size_t),
        ("end_timestep", ctypes.c_size_t),
        ("flags", ctypes.c_uint),
    ]


FLAG_TIME_KERNELS = 1
FLAG_WINDOWS_CHECKED = 2
FLAG_GENERIC_KERNEL = 4
FLAG_STEP_LAUNCHES = 8


def layout(fastest_extent, space_order, precision):
    """``(pitch, lead)`` the library prefers for a row of ``fastest_extent``."""
    lib = _lib.load()
    pitch, lead = ctypes.c_size_t(), ctypes.c_size_t()
    status = lib.simwave_layout(ctypes.c_size_t(fastest_extent),
                                ctypes.c_int(space_order),
                                ctypes.c_int(precision), ctypes.byref(pitch),
                                ctypes.byref(lead))
    if status != 0:
        raise ValueError("invalid layout request")
    return pitch.value, lead.value


def _check_windows(points, offsets, values_size, count, dim, shape):
    """Host check of KWS windows (inside the grid, offsets consistent)."""
    if count == 0:
        return
    iv = np.asarray(points, dtype=np.uint64).reshape(count, dim, 2)
    if np.any(iv[:, :, 0] > iv[:, :, 1]) or np.any(
            iv[:, :, 1] >= np.asarray(shape, dtype=np.uint64)[None, :]):
        raise ValueError("KWS window outside the grid")
    lengths = (iv[:, :, 1] - iv[:, :, 0] + 1).sum(axis=1)
    off = np.asarray(offsets, dtype=np.uint64)[:count]
    if np.any(off + lengths > values_size):
        raise ValueError("KWS values offsets out of range")


class DeviceProblem:
    """One forward problem with every array resident on ``device``.

    ``kwargs`` are the middleware keyword arguments of ``Solver.forward``
    (``Solver.forward_arguments()``); ``u_full`` and ``shot_record`` give the
    initial contents.
    """

    def __init__(self, kwargs, device="cuda"):
        kw = normalise(kwargs)
        vel = kw['velocity_model']
        self.dtype = vel.dtype
        self.dim = vel.ndim
        self.shape = vel.shape
        self.vd = 'density_model' in kw
        self.device = torch.device(device)
        tdt = torch.float32 if self.dtype == np.float32 else torch.float64
        prec = 4 if self.dtype == np.float32 else 8
        order = int(kw['space_order'])
        nfast = self.shape[-1]
        self.pitch, self.lead = layout(nfast, order, prec)
        rows = int(np.prod(self.shape[:-1]))
        self.slot = rows * self.pitch
        nslots = int(kw['num_snapshots'])
        self._u = torch.zeros(nslots * self.slot, dtype=tdt, device=self.device)
        self.u = self._view(self._u, nslots)
        u0 = kw['u_full']
        if np.any(u0):
            self.u.copy_(torch.from_numpy(np.ascontiguousarray(u0)))

        def grid(a):
            flat = torch.zeros(self.slot, dtype=tdt, device=self.device)
            self._view(flat, None).copy_(torch.from_numpy(np.ascontiguousarray(a)))
            return flat

        self.vel = grid(vel)
        self.den = grid(kw['density_model']) if self.vd else None
        self.damp = grid(kw['damping_mask'])

        def dev(a, dtype=None):
            a = np.ascontiguousarray(a if dtype is None else np.asarray(a, dtype=dtype))
            if a.size == 0:
                a = np.zeros(1, dtype=a.dtype)
            return torch.from_numpy(a).to(self.device)

        nsrc, nrec = int(kw['num_sources']), int(kw['num_receivers'])
        _check_windows(kw['src_points_interval'], kw['src_points_values_offset'],
                       len(kw['src_points_values']), nsrc, self.dim, self.shape)
        _check_windows(kw['rec_points_interval'], kw['rec_points_values_offset'],
                       len(kw['rec_points_values']), nrec, self.dim, self.shape)
        u64 = np.uint64
        self.wavelet = dev(kw['wavelet'], self.dtype)
        self.src_iv = dev(kw['src_points_interval'], u64)
        self.src_val = dev(kw['src_points_values'], self.dtype)
        self.src_off = dev(kw['src_points_values_offset'], u64)
        self.rec_iv = dev(kw['rec_points_interval'], u64)
        self.rec_val = dev(kw['rec_points_values'], self.dtype)
        self.rec_off = dev(kw['rec_points_values_offset'], u64)
        T = int(kw['end_timestep'])
        self.receivers = torch.zeros((max(T, 1), max(nrec, 1)), dtype=tdt,
                                     device=self.device)
        rec0 = kw['shot_record']
        if rec0.size and np.any(rec0):
            self.receivers[:rec0.shape[0], :rec0.shape[1]].copy_(
                torch.from_numpy(np.ascontiguousarray(rec0)))
        # host-side small arrays, kept alive for the ctypes struct
        self._c2 = np.ascontiguousarray(kw['second_order_fd_coefficients'], dtype=self.dtype)
        self._c1 = np.ascontiguousarray(
            kw.get('first_order_fd_coefficients', self._c2), dtype=self.dtype)
        self._bc = np.ascontiguousarray(kw['boundary_condition'], dtype=u64)
        spacing = [float(kw['dz']), float(kw['dx']),
                   float(kw.get('dy', 1.0))]
        p = Problem()
        p.dim = self.dim
        p.variable_density = 1 if self.vd else 0
        p.precision = prec
        p.space_order = order
        p.nz = self.shape[0]
        p.nx = self.shape[1]
        p.ny = self.shape[2] if self.dim == 3 else 1
        p.pitch = self.pitch
        p.lead = self.lead
        p.slot_stride = self.slot
        p.dz, p.dx, p.dy = spacing
        p.dt = float(kw['dt'])
        p.u = self._u.data_ptr()
        p.num_snapshots = nslots
        p.velocity = self.vel.data_ptr()
        p.density = self.den.data_ptr() if self.vd else None
        p.damp = self.damp.data_ptr()
        p.wavelet = self.wavelet.data_ptr()
        p.wavelet_size = int(kw['wavelet_size'])
        p.wavelet_count = int(kw['wavelet_count'])
        p.coeff_order2 = self._c2.ctypes.data
        p.coeff_order1 = self._c1.ctypes.data
        p.boundary_conditions = self._bc.ctypes.data
        p.src_points_interval = self.src_iv.data_ptr()
        p.src_points_values = self.src_val.data_ptr()
        p.src_points_values_offset = self.src_off.data_ptr()
        p.src_points_values_size = len(kw['src_points_values'])
        p.num_sources = nsrc
        p.rec_points_interval = self.rec_iv.data_ptr()
        p.rec_points_values = self.rec_val.data_ptr()
        p.rec_points_values_offset = self.rec_off.data_ptr()
        p.rec_points_values_size = len(kw['rec_points_values'])
        p.num_receivers = nrec
        p.receivers = self.receivers.data_ptr()
        p.saving_stride = int(kw['saving_stride'])
        p.begin_timestep = int(kw['begin_timestep'])
        p.end_timestep = T
        p.flags = FLAG_WINDOWS_CHECKED
        self.problem = p
        self.nslots = nslots
        self.nrec = nrec
        self.timesteps = T - int(kw['begin_timestep']) + 1

    def _view(self, flat, nslots):
        """Logical view of a pitched buffer (one grid, or ``nslots`` slots)."""
        rows_shape = tuple(self.shape[:-1])
        nfast = self.shape[-1]
        if nslots is None:
            full = flat.view(rows_shape + (self.pitch,))
        else:
            full = flat.view((nslots,) + rows_shape + (self.pitch,))
        return full[..., self.lead:self.lead + nfast]

    def reset(self):
        """Zero the wavefield slots and the shot record."""
        self._u.zero_()
        self.receivers.zero_()

    def run(self, stream=None, time_kernels=False, generic=False, step_launches=False):
        """Launch the forward loop on ``stream`` (torch stream or None).

        ``generic`` forces the one-thread-per-point stencil kernel;
        ``step_launches`` keeps per-step launches for small 2D grids."""
        lib = _lib.load()
        self.problem.flags = FLAG_WINDOWS_CHECKED | (
            FLAG_TIME_KERNELS if time_kernels else 0) | (
            FLAG_GENERIC_KERNEL if generic else 0) | (
            FLAG_STEP_LAUNCHES if step_launches else 0)
        handle = None
        if stream is not None:
            handle = ctypes.c_void_p(stream.cuda_stream)
        else:
            handle = ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        status = lib.simwave_forward_device(ctypes.byref(self.problem), handle)
        if status != 0:
            raise RuntimeError("simwave_forward_device failed ({}): {}".format(
                status, _lib.last_error()))
        return _lib.last_stats()

    def status(self, stream=None):
        """Wait for the stream and raise if a device-side wait expired."""
        lib = _lib.load()
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        status = lib.simwave_device_status(ctypes.c_void_p(s.cuda_stream))
        if status != 0:
            raise RuntimeError("device status {}: {}".format(status, _lib.last_error()))

    def grid_view(self, flat):
        """The logical ``(nz, nx[, ny])`` view of one pitched grid buffer
        (``slot`` elements)."""
        return self._view(flat, None)

    @property
    def wavefield_bytes(self):
        """Device bytes of the wavefield slots (0 once released)."""
        return 0 if self._u is None else self._u.numel() * self._u.element_size()

    def release_wavefield(self):
        """Drop the device wavefield slots; returns the bytes freed."""
        freed = self.wavefield_bytes
        self._u = None
        self.u = None
        return freed

    def release_inputs(self):
        """Drop the device copies of the models and tables; the wavefield
        slots and the shot record stay."""
        self.vel = self.den = self.damp = self.wavelet = None
        self.src_iv = self.src_val = self.src_off = None
        self.rec_iv = self.rec_val = self.rec_off = None

    def u_full_numpy(self):
        return self.u.cpu().numpy()

    def shot_record_numpy(self):
        return self.receivers[:, :self.nrec].cpu().numpy()
