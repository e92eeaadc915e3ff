"""Kaiser-windowed sinc (KWS) positioning of sources and receivers.

Restates simwave/kernel/frontend/kws.py (Hicks 2002, "Arbitrary source and
receiver positioning in finite-difference schemes using Kaiser windowed sinc
functions") in vectorised form: the reference evaluates the window over the
whole axis one source at a time in a Python loop (kws.py:44-135, called per
position from source.py:144-159); here every position of one axis is
evaluated at once on a narrow band of candidate indices. The element-wise
expression and its dtype flow are the reference's, so the values are the same:

* ``x = float32(index) - position`` in the position dtype (kws.py:70-75);
* ``sqrt(1 - (x / w) ** 2)``, NaN outside the window (kws.py:78-80);
* ``i0(b * sqrt) / i0(b)`` with ``i0(b)`` a float64 scalar, so the Kaiser
  window is float64 (kws.py:83-86);
* ``np.sinc(x)`` in the position dtype, product in float64 (kws.py:89-92);
* the valid (non-NaN) values of each axis are rounded to float32
  (kws.py:126-133).
"""
import warnings

import numpy as np
from scipy.special import i0

# Kaiser ``b`` parameter per window half-width (Hicks 2002, table 2), the
# values listed by the reference at kws.py:28-39.
_KAISER_B = {1: 1.24, 2: 2.94, 3: 4.53, 4: 6.31, 5: 7.91,
             6: 9.42, 7: 10.95, 8: 12.53, 9: 14.09, 10: 14.18}


def get_kaiser_half_width(half_width):
    """Kaiser ``b`` for a window half-width of 1..10 (kws.py:6-41)."""
    if half_width not in _KAISER_B:
        raise Exception(
            "Kaiser windowing half-width {} not supported".format(half_width))
    return _KAISER_B[half_width]


def _kws_values(x, half_width):
    """KWS of distances ``x`` (any shape, contiguous); NaN outside the window."""
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        root = np.sqrt(1 - (x / half_width) ** 2)
    b = get_kaiser_half_width(half_width)
    kaiser = i0(b * root) / i0(b)
    return kaiser * np.sinc(x)


def kaiser_windowing_sinc(num_points, source_point, half_width):
    """KWS over a whole axis of ``num_points`` (kws.py:44-94)."""
    x = np.linspace(0, num_points - 1, num_points, dtype=np.float32)
    return _kws_values(x - source_point, half_width)


def axis_windows(num_points, positions, half_width):
    """Window of every position along one axis.

    Returns ``(begin, end, values)``: int64 arrays of the first/last valid
    index per position and a float32 array ``(npos, band)`` whose row ``i``
    holds the valid values in columns ``0 .. end[i]-begin[i]`` (NaN after).
    """
    positions = np.asarray(positions)
    npos = positions.shape[0]
    # every index whose distance can pass the window test lies in
    # [floor(p) - w - 1, floor(p) + w + 2]; clip the band to the axis
    band = 2 * half_width + 4
    start = np.floor(positions.astype(np.float64)).astype(np.int64) - half_width - 1
    start = np.clip(start, 0, max(num_points - band, 0))
    band = min(band, num_points)
    idx = start[:, None] + np.arange(band, dtype=np.int64)[None, :]
    grid = idx.astype(np.float32)
    x = np.ascontiguousarray(grid - positions[:, None])
    kws = _kws_values(x, half_width)
    valid = ~np.isnan(kws)
    if not np.all(valid.any(axis=1)):
        raise Exception(
            "There is no valid point in the source/receiver location")
    first = np.argmax(valid, axis=1)
    last = band - 1 - np.argmax(valid[:, ::-1], axis=1)
    begin = start + first
    end = start + last
    # the window is contiguous: shift each row so its first valid value is col 0
    cols = np.arange(band)[None, :] + first[:, None]
    take = np.take_along_axis(kws, np.minimum(cols, band - 1), axis=1)
    take = np.where(cols <= last[:, None], take, np.nan)
    return begin, end, take.astype(np.float32)


def get_source_points(grid_shape, source_location, half_width):
    """Interval and values of one position (kws.py:138-183)."""
    if len(grid_shape) != len(source_location):
        raise Exception(
            "Grid and source/receiver location must have the same dimension.")
    points, values, _ = interpolated_points_and_values(
        grid_shape, np.asarray([source_location]), half_width, np.float32)
    return points, values


def interpolated_points_and_values(grid_shape, positions, half_width, dtype):
    """Intervals, concatenated values and offsets of every position.

    Same layout as simwave/kernel/frontend/source.py:123-159: ``points`` is
    uint64 ``[z_b, z_e, x_b, x_e(, y_b, y_e)]`` per position, ``values`` the
    per-position concatenation of the z, x (and y) windows, and ``offsets``
    uint64 ``[0, n_0, n_0 + n_1, ..]``.
    """
    positions = np.asarray(positions)
    npos, ndim = positions.shape
    if ndim != len(grid_shape):
        raise Exception(
            "Grid and source/receiver location must have the same dimension.")
    if npos == 0:
        return (np.array([], dtype=np.uint), np.array([], dtype=dtype),
                np.zeros(1, dtype=np.uint))
    begins, ends, rows = [], [], []
    for axis in range(ndim):
        b, e, v = axis_windows(grid_shape[axis], positions[:, axis], half_width)
        begins.append(b)
        ends.append(e)
        rows.append(v)
    points = np.empty((npos, 2 * ndim), dtype=np.uint)
    for axis in range(ndim):
        points[:, 2 * axis] = begins[axis]
        points[:, 2 * axis + 1] = ends[axis]
    lengths = np.stack([ends[a] - begins[a] + 1 for a in range(ndim)], axis=1)
    counts = lengths.sum(axis=1)
    offsets = np.zeros(npos + 1, dtype=np.uint)
    np.cumsum(counts, out=offsets[1:])
    # gather: per position, axis-major concatenation of the valid values
    width = max(r.shape[1] for r in rows)
    padded = np.full((npos, ndim, width), np.nan, dtype=np.float32)
    for axis in range(ndim):
        padded[:, axis, :rows[axis].shape[1]] = rows[axis]
    mask = np.arange(width)[None, None, :] < lengths[:, :, None]
    values = padded[mask].astype(dtype)
    return points.reshape(-1), values, offsets
