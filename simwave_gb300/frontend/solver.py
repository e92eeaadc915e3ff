"""Acoustic forward solver mirroring simwave's ``Solver`` (solver.py:5-169)."""
import numpy as np

from ..backend.middleware import Middleware


class Solver:
    """Forward modelling of one shot.

    Parameters mirror the reference: ``space_model``, ``time_model``,
    ``sources``, ``receivers``, ``wavelet`` and an optional ``compiler``
    (default: the sm_103a GPU library).
    """

    def __init__(self, space_model, time_model, sources, receivers, wavelet,
                 compiler=None):
        self._space_model = space_model
        self._time_model = time_model
        self._sources = sources
        self._receivers = receivers
        self._wavelet = wavelet
        self._compiler = compiler
        self._middleware = Middleware(compiler=compiler)

    @property
    def space_model(self):
        return self._space_model

    @property
    def time_model(self):
        return self._time_model

    @property
    def sources(self):
        return self._sources

    @property
    def receivers(self):
        return self._receivers

    @property
    def wavelet(self):
        return self._wavelet

    @property
    def compiler(self):
        return self._middleware.compiler

    @property
    def snapshot_indexes(self):
        """Time indexes kept: the last one for stride 0, else every
        ``saving_stride``-th from 0 (solver.py:67-83)."""
        tm = self.time_model
        if tm.saving_stride == 0:
            return [tm.time_indexes[-1]]
        return list(range(tm.time_indexes[0], tm.timesteps, tm.saving_stride))

    @property
    def num_snapshots(self):
        return len(self.snapshot_indexes)

    @property
    def shot_record(self):
        """Zeroed ``(timesteps, receivers)`` array (solver.py:90-98)."""
        return np.zeros((self.time_model.timesteps, self.receivers.count),
                        dtype=self.space_model.dtype)

    @property
    def u_full(self):
        """Zeroed ``(snapshots + 2, *extended_shape)`` array (solver.py:100-110)."""
        shape = (self.num_snapshots + 2,) + tuple(self.space_model.extended_shape)
        return np.zeros(shape, dtype=self.space_model.dtype)

    def forward_arguments(self):
        """Keyword arguments of the middleware call (solver.py:121-161)."""
        sm, tm = self.space_model, self.time_model
        src_points, src_values, src_offsets = \
            self.sources.interpolated_points_and_values
        rec_points, rec_values, rec_offsets = \
            self.receivers.interpolated_points_and_values
        u_full = self.u_full
        return dict(
            u_full=u_full,
            velocity_model=sm.extended_velocity_model,
            density_model=sm.extended_density_model,
            damping_mask=sm.damping_mask,
            wavelet=self.wavelet.values,
            wavelet_size=self.wavelet.timesteps,
            wavelet_count=self.wavelet.num_sources,
            second_order_fd_coefficients=sm.fd_coefficients(2),
            first_order_fd_coefficients=sm.fd_coefficients(1),
            boundary_condition=sm.boundary_condition,
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
            shot_record=self.shot_record,
            num_sources=self.sources.count,
            num_receivers=self.receivers.count,
            grid_spacing=sm.grid_spacing,
            saving_stride=tm.saving_stride,
            dt=tm.dt,
            begin_timestep=1,
            end_timestep=tm.timesteps,
            space_order=sm.space_order,
            num_snapshots=u_full.shape[0],
        )

    def forward(self):
        """Run the propagator; returns ``(u_full, shot_record)``.

        ``u_full`` keeps the returned snapshots with the halo removed (damping
        layer kept), as solver.py:163-169 does.
        """
        u_full, recv = self._middleware.exec('forward', **self.forward_arguments())
        u_full = self.time_model.remove_time_halo_region(u_full)
        u_full = self.space_model.remove_halo_region(u_full)
        return u_full, recv
