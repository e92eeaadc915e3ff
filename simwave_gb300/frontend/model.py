"""Space and time models: grid, padding, damping layer, CFL step, time axis.

Restates simwave/kernel/frontend/model.py with the same constructor
arguments, properties, validation and numerics. Two host-cost fixes keep the
results bit-identical:

* ``interpolate`` returns the input unchanged when it already has the grid's
  shape: ``RegularGridInterpolator`` evaluated on its own nodes is the identity
  (the reference always re-interpolates, model.py:56-63, 210-261, which costs
  tens of seconds for a 384^3 model);
* derived arrays (damping mask, padded models) are computed once and cached
  instead of being rebuilt on every property access.
"""
import numpy as np
from scipy.interpolate import RegularGridInterpolator

from . import fd

_BOUNDARY_CONDITIONS = ('none', 'null_dirichlet', 'null_neumann')


class SpaceModel:
    """Spatial model of a simulation (reference: model.py:6-515).

    Parameters
    ----------
    bounding_box : tuple of float
        ``(z_min, z_max, x_min, x_max[, y_min, y_max])`` in metres.
    grid_spacing : tuple of float
        Spacing per axis ``(z, x[, y])`` in metres.
    velocity_model : ndarray
        P-wave velocity (m/s), 2D or 3D.
    density_model : ndarray, optional
        Density; selects the variable-density operator when given.
    space_order : int, optional
        Even spatial order 2..20 (default 2).
    dtype : numpy float type, optional
        ``np.float32`` (default) or ``np.float64``.
    """

    def __init__(self, bounding_box, grid_spacing, velocity_model,
                 density_model=None, space_order=2, dtype=np.float32):
        self._dtype = dtype
        self._bounding_box = tuple(self.dtype(v) for v in bounding_box)
        self._grid_spacing = tuple(self.dtype(v) for v in grid_spacing)
        self._space_order = space_order
        if space_order % 2 != 0:
            raise ValueError(
                "Odd space order {} not supported".format(space_order))
        if not 2 <= space_order <= 20:
            raise ValueError("Space order limited from 2 to 20.")
        self._dimension = len(velocity_model.shape)
        self._velocity_model = self.interpolate(velocity_model)
        self._density_model = (None if density_model is None
                               else self.interpolate(density_model))
        self._cache = {}

    # -- plain attributes -------------------------------------------------
    @property
    def bounding_box(self):
        return self._bounding_box

    @property
    def grid_spacing(self):
        return self._grid_spacing

    @property
    def velocity_model(self):
        return self._velocity_model

    @property
    def density_model(self):
        return self._density_model

    @property
    def space_order(self):
        return self._space_order

    @property
    def dimension(self):
        return self._dimension

    @property
    def dtype(self):
        return self._dtype

    # -- grid geometry ------------------------------------------------------
    @property
    def shape(self):
        """Grid points per axis: ``int((max - min) / h) + 1`` (model.py:93-112)."""
        box = self.bounding_box
        return tuple(
            int((box[2 * a + 1] - box[2 * a]) / self.grid_spacing[a]) + 1
            for a in range(self.dimension))

    @property
    def halo_size(self):
        """``space_order // 2`` on every edge (model.py:263-269)."""
        return (self.space_order // 2,) * self.dimension * 2

    @property
    def nbl(self):
        """Damping-layer points per edge, 0 until configured (model.py:135-145)."""
        return getattr(self, '_nbl', (0,) * self.dimension * 2)

    @property
    def damping_length(self):
        return getattr(self, '_damping_length', (0.0,) * self.dimension * 2)

    @property
    def boundary_condition(self):
        return getattr(self, '_boundary_condition',
                       ('none',) * self.dimension * 2)

    @property
    def damping_polynomial_degree(self):
        return getattr(self, '_damping_polynomial_degree', 3)

    @property
    def damping_alpha(self):
        return getattr(self, '_damping_alpha', 0.001)

    @property
    def extended_shape(self):
        """Shape plus damping layer plus halo per axis (model.py:114-133)."""
        return tuple(
            self.shape[a] + self.nbl[2 * a] + self.nbl[2 * a + 1]
            + self.halo_size[2 * a] + self.halo_size[2 * a + 1]
            for a in range(self.dimension))

    @property
    def grid(self):
        return np.zeros(self.shape, dtype=self.dtype)

    @property
    def nbl_pad_width(self):
        return tuple((self.nbl[2 * a], self.nbl[2 * a + 1])
                     for a in range(self.dimension))

    @property
    def halo_pad_width(self):
        return tuple((self.halo_size[2 * a], self.halo_size[2 * a + 1])
                     for a in range(self.dimension))

    def fd_coefficients(self, derivative_order):
        """Half-stencil weights ``[c0..cr]`` in the model dtype (model.py:192-208)."""
        return self.dtype(
            fd.half_coefficients(derivative_order, self.space_order))

    def interpolate(self, data):
        """Resample ``data`` onto the model grid (model.py:210-261).

        Multilinear interpolation over the bounding box; identity when the
        input already has the grid's shape.
        """
        shape = self.shape
        if tuple(data.shape) == tuple(shape):
            return self.dtype(data)
        box = self.bounding_box
        src_axes = tuple(np.linspace(box[2 * a], box[2 * a + 1], data.shape[a])
                         for a in range(self.dimension))
        interpolant = RegularGridInterpolator(src_axes, data)
        dst_axes = [np.linspace(box[2 * a], box[2 * a + 1], shape[a])
                    for a in range(self.dimension)]
        mesh = np.meshgrid(*dst_axes, indexing='ij')
        return self.dtype(interpolant(tuple(mesh)))

    # -- boundary configuration --------------------------------------------
    def config_boundary(self, damping_length=0.0, boundary_condition="none",
                        damping_polynomial_degree=3, damping_alpha=0.001):
        """Damping layer (metres per edge) and per-edge boundary conditions.

        Same argument forms and validation as model.py:271-349; the layer
        width per edge is ``int(length / h)`` points.
        """
        self._damping_polynomial_degree = damping_polynomial_degree
        self._damping_alpha = damping_alpha
        if isinstance(damping_length, (float, int)):
            self._damping_length = (self.dtype(damping_length),) \
                * self.dimension * 2
        else:
            self._damping_length = tuple(self.dtype(v) for v in damping_length)
        if isinstance(boundary_condition, str):
            self._boundary_condition = (boundary_condition,) \
                * self.dimension * 2
        else:
            self._boundary_condition = boundary_condition
        for bc in self.boundary_condition:
            if bc not in _BOUNDARY_CONDITIONS:
                raise ValueError('Boundary condition {} not available.'.format(
                    self.boundary_condition))
        self._nbl = tuple(
            int(self._damping_length[e] / self.grid_spacing[e // 2])
            for e in range(2 * self.dimension))
        self._cache = {}

    # -- padded arrays -------------------------------------------------------
    @property
    def damping_mask(self):
        """``alpha * d**degree`` in the layer, 0 inside and in the halo.

        ``d`` is the linear ramp ``np.pad(mode='linear_ramp')`` builds from the
        domain edge to the outer edge (model.py:377-406).
        """
        if 'damp' not in self._cache:
            ramp = np.pad(np.zeros(self.shape, dtype=self.dtype),
                          pad_width=self.nbl_pad_width, mode="linear_ramp",
                          end_values=self.nbl_pad_width)
            # in place, the same float32 operations; with degree >= 1 the
            # zero core stays zero, so only the layer slabs are raised
            deg = self.damping_polynomial_degree
            views = _layer_slabs(ramp, self.nbl_pad_width) if deg >= 1 else [ramp]
            for v in views:
                np.power(v, deg, out=v)
                v *= self.damping_alpha
            self._cache['damp'] = np.pad(ramp, pad_width=self.halo_pad_width)
        return self._cache['damp']

    def _edge_padded(self, data):
        # edge padding of an edge-padded array is one edge padding with the
        # summed widths: the layer and the halo in a single copy
        width = tuple((a + c, b + d) for (a, b), (c, d)
                      in zip(self.nbl_pad_width, self.halo_pad_width))
        return np.pad(data, pad_width=width, mode="edge")

    @property
    def extended_grid(self):
        grid = np.pad(self.grid, pad_width=self.nbl_pad_width)
        return np.pad(grid, pad_width=self.halo_pad_width)

    @property
    def extended_velocity_model(self):
        """Velocity edge-padded into the layer and halo (model.py:420-443)."""
        if 'vel' not in self._cache:
            self._cache['vel'] = self._edge_padded(self.velocity_model)
        return self._cache['vel']

    @property
    def extended_density_model(self):
        """Density edge-padded into the layer and halo (model.py:445-466)."""
        if self.density_model is None:
            return None
        if 'den' not in self._cache:
            self._cache['den'] = self._edge_padded(self.density_model)
        return self._cache['den']

    def remove_halo_region(self, u):
        """Strip the halo from every snapshot (model.py:468-492)."""
        halo = self.halo_size[0]
        if self.dimension not in (2, 3):
            raise Exception("Wavefield dimension not supported.")
        index = (slice(None),) + (slice(halo, -halo),) * self.dimension
        return u[index]

    def remove_nbl(self, u):
        """Strip the damping layer from every snapshot (model.py:494-515)."""
        nbl = self.nbl
        if self.dimension not in (2, 3):
            raise Exception("Wavefield dimension not supported.")
        index = (slice(None),) + tuple(
            slice(nbl[2 * a], -nbl[2 * a + 1]) for a in range(self.dimension))
        return u[index]


def _layer_slabs(a, widths):
    """Views of ``a`` covering each point outside the core box (``widths``
    per axis: before, after) exactly once: for each axis, the before and
    after slabs over the core range of the axes before it."""
    views = []
    for axis in range(a.ndim):
        index = [slice(widths[b][0], a.shape[b] - widths[b][1]) if b < axis else slice(None)
                 for b in range(a.ndim)]
        lo, hi = widths[axis]
        if lo:
            index[axis] = slice(0, lo)
            views.append(a[tuple(index)])
        if hi:
            index[axis] = slice(a.shape[axis] - hi, a.shape[axis])
            views.append(a[tuple(index)])
    return views


class TimeModel:
    """Time axis of a simulation (reference: model.py:518-643).

    Parameters
    ----------
    space_model : SpaceModel
    tf : float
        End time (s).
    dt : float, optional
        Time step; may only shrink the CFL step.
    t0 : float, optional
        Start time (s), default 0.
    saving_stride : int, optional
        Keep every ``saving_stride``-th wavefield; 0 keeps only the last.
    """

    def __init__(self, space_model, tf, dt=None, t0=0.0, saving_stride=0):
        self._space_model = space_model
        self._tf = self.space_model.dtype(tf)
        self._t0 = self.space_model.dtype(t0)
        self._saving_stride = saving_stride
        self._dt = fd.calculate_dt(
            dimension=self.space_model.dimension,
            space_order=self.space_model.space_order,
            grid_spacing=self.space_model.grid_spacing,
            velocity_model=self.space_model.velocity_model)
        if dt is not None:
            self.dt = dt
        if not (0 <= self.saving_stride <= self.timesteps):
            raise Exception(
                "Saving jumps can not be less than zero or "
                "greater than the number of timesteps.")

    @property
    def space_model(self):
        return self._space_model

    @property
    def tf(self):
        return self._tf

    @property
    def t0(self):
        return self._t0

    @property
    def saving_stride(self):
        return self._saving_stride

    @property
    def dtype(self):
        return self.space_model.dtype

    @property
    def dt(self):
        return self.dtype(self._dt)

    @dt.setter
    def dt(self, value):
        if value < 0:
            raise ValueError("Time step cannot be negative.")
        if value > self.dt:
            raise ValueError("Time step value violates CFL condition.")
        self._dt = value

    @property
    def timesteps(self):
        """``ceil((tf - t0 + dt) / dt)``, grown until ``T % stride == 1``.

        Same arithmetic (model dtype) as model.py:599-609.
        """
        steps = int(np.ceil((self.tf - self.t0 + self.dt) / self.dt))
        stride = self.saving_stride
        if 1 < stride <= steps:
            steps += (1 - steps) % stride
        return steps

    @property
    def time_indexes(self):
        return np.linspace(0, self.timesteps - 1, self.timesteps, dtype=np.uint)

    @property
    def time_values(self):
        """``linspace(t0, tf, T)`` in the model dtype (model.py:617-621)."""
        return np.linspace(self.t0, self.tf, self.timesteps, dtype=self.dtype)

    def remove_time_halo_region(self, u):
        """Keep the returned snapshot slots (model.py:623-643).

        Stride 0: the slot ``T % 3`` that holds the last time level; otherwise
        every slot but the first and the last.
        """
        if self.saving_stride == 0:
            last = self.timesteps % 3
            return u[last:last + 1]
        return u[1:-1]
