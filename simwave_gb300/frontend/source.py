"""Sources, receivers and wavelets (reference: simwave/kernel/frontend/source.py)."""
import numpy as np

from . import kws


class Source:
    """A set of point sources (or receivers) placed with KWS interpolation.

    Parameters
    ----------
    space_model : SpaceModel
    coordinates : array-like, ``(n, 2)`` or ``(n, 3)`` metres (one point may be
        given flat)
    window_radius : int, optional
        KWS half-width 1..10 (default 4).
    """

    def __init__(self, space_model, coordinates, window_radius=4):
        self._space_model = space_model
        self._window_radius = window_radius
        if not isinstance(coordinates, (list, tuple, np.ndarray)):
            raise ValueError("Source/Receiver coordinates must be "
                             "represented as lists, tuples or ndarrays.")
        coords = np.asarray(coordinates, dtype=self.space_model.dtype)
        if coords.ndim == 1:
            coords = coords.reshape((1,) + coords.shape)
        elif coords.ndim != 2 or coords.shape[1] not in (2, 3):
            raise ValueError("Invalid source/receiver coordinates format.")
        self._coordinates = coords

    @property
    def space_model(self):
        return self._space_model

    @property
    def coordinates(self):
        return self._coordinates

    @property
    def window_radius(self):
        return self._window_radius

    @property
    def count(self):
        return self.coordinates.shape[0]

    @property
    def grid_positions(self):
        """Positions in grid points, ``(coord - min) / h`` (source.py:62-103)."""
        sm = self.space_model
        coords = self.coordinates
        ndim = coords.shape[1]
        if ndim != sm.dimension:
            raise Exception("Dimension %d not supported." % ndim)
        box = sm.bounding_box
        lo = np.array([box[2 * a] for a in range(ndim)], dtype=sm.dtype)
        hi = np.array([box[2 * a + 1] for a in range(ndim)], dtype=sm.dtype)
        inside = np.all((coords >= lo) & (coords <= hi), axis=1)
        if not np.all(inside):
            bad = coords[np.argmin(inside)]
            raise Exception("Coordinates %s out of bounds." % bad)
        h = np.array(sm.grid_spacing, dtype=sm.dtype)
        return np.asarray((coords - lo) / h, dtype=sm.dtype)

    @property
    def adjusted_grid_positions(self):
        """Grid positions shifted by the damping layer and halo (source.py:105-121)."""
        sm = self.space_model
        origin = np.array([sm.nbl[2 * a] + sm.halo_size[2 * a]
                           for a in range(sm.dimension)])
        return np.asarray(self.grid_positions + origin.astype(sm.dtype),
                          dtype=sm.dtype)

    @property
    def interpolated_points_and_values(self):
        """``(points, values, offsets)`` in the layout of source.py:123-159."""
        sm = self.space_model
        return kws.interpolated_points_and_values(
            sm.extended_shape, self.adjusted_grid_positions,
            self.window_radius, sm.dtype)


# a receiver samples the wavefield with the same KWS window as a source
Receiver = Source


class Wavelet:
    """A source time function given by ``function(**kwargs)`` (source.py:171-209)."""

    def __init__(self, function, **kwargs):
        self._function = function
        self._kwargs = kwargs

    @property
    def function(self):
        return self._function

    @property
    def kwargs(self):
        return self._kwargs

    @property
    def values(self):
        return self.function(**self.kwargs)

    @property
    def num_sources(self):
        return 1

    @property
    def timesteps(self):
        return len(self.values)


class RickerWavelet(Wavelet):
    """``A (1 - 2 r^2) exp(-r^2)``, ``r = pi f (t - 1/f)`` on the model time axis.

    Reference: source.py:212-257; sampled on ``TimeModel.time_values``.
    """

    def __init__(self, peak_frequency, time_model, amplitude=1):
        self._peak_frequency = peak_frequency
        self._time_model = time_model
        self._amplitude = amplitude
        super().__init__(self._ricker, peak_frequency=peak_frequency,
                         time_model=time_model, amplitude=amplitude)

    @property
    def peak_frequency(self):
        return self._peak_frequency

    @property
    def time_model(self):
        return self._time_model

    @property
    def amplitude(self):
        return self._amplitude

    @staticmethod
    def _ricker(peak_frequency, time_model, amplitude):
        delay = 1 / peak_frequency
        r = np.pi * peak_frequency * (time_model.time_values - delay)
        return amplitude * (1 - 2.0 * r ** 2) * np.exp(-r ** 2)


class MultiWavelet(Wavelet):
    """One wavelet per source, ``values[timestep, source]`` (source.py:260-302)."""

    def __init__(self, values, time_model):
        self._values = values
        self._time_model = time_model
        if self.timesteps != self.time_model.timesteps:
            raise ValueError("Wavelet must have {} timesteps.".format(
                self.time_model.timesteps))

    @property
    def values(self):
        return np.ascontiguousarray(self._values, dtype=self.dtype)

    @property
    def num_sources(self):
        return self.values.shape[1]

    @property
    def timesteps(self):
        return self.values.shape[0]

    @property
    def time_model(self):
        return self._time_model

    @property
    def dtype(self):
        return self.time_model.dtype
