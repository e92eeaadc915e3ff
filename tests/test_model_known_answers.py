"""Model known answers: the expected values of the reference's
tests/test_space_model.py (defaults, shapes, extended shapes with damping
layers and halos, layer widths in points, FD weights, halo sizes, boundary
configuration, padded array shapes), of tests/test_time_model.py:8-31
(TimeModel properties) and of tests/test_source.py:8-116 (Source
properties, grid positions, positions on the extended grid), checked on this
package's front end. The time-step counts with stride padding and the KWS
interpolation points and values are in test_frontend.py. CPU only."""
import numpy as np
import pytest

import simwave_gb300 as sw


def _model(dim, bbox=None, spacing=None, order=2, side=50, density=False, **kw):
    vel = 1500 * np.ones((side,) * dim)
    den = 15 * np.ones((side,) * dim) if density else None
    return sw.SpaceModel(bounding_box=bbox or (0, 1000) * dim,
                         grid_spacing=spacing or (10,) * dim, velocity_model=vel,
                         density_model=den, space_order=order, **kw)


@pytest.mark.parametrize("dim", [2, 3])
def test_defaults_and_properties(dim):
    # tests/test_space_model.py:8-35
    m = _model(dim, order=4, side=101, density=True, dtype=np.float32)
    assert m.bounding_box == (0, 1000) * dim
    assert m.grid_spacing == (10,) * dim
    assert np.array_equal(m.velocity_model, 1500 * np.ones((101,) * dim))
    assert np.array_equal(m.density_model, 15 * np.ones((101,) * dim))
    assert (m.space_order, m.dimension, m.dtype) == (4, dim, np.float32)
    assert m.damping_length == (0.0,) * 2 * dim
    assert m.boundary_condition == ("none",) * 2 * dim
    assert (m.damping_polynomial_degree, m.damping_alpha) == (3, 0.001)


# tests/test_space_model.py:37-56
SHAPES = [
    ((0, 1000, 0, 1000), (10, 10), (101, 101)),
    ((100.0, 1000, 0, 1250.5), (10, 10), (91, 126)),
    ((-100, 1000, 500, 1000), (20, 10), (56, 51)),
    ((0, 1000, 0, 1000, 0, 1000.0), (5, 10, 20), (201, 101, 51)),
    ((10, 100, -10, 100, 0.0, 100.0), (5, 5, 5), (19, 23, 21)),
]


@pytest.mark.parametrize("bbox, spacing, shape", SHAPES)
def test_shape(bbox, spacing, shape):
    assert _model(len(spacing), bbox, spacing).shape == shape


# tests/test_space_model.py:58-87: (dim, damping length, order, extended shape)
EXTENDED = [
    (2, 100, 2, (123, 123)),
    (2, 100, 4, (125, 125)),
    (2, 150, 16, (147, 147)),
    (2, (150, 100, 150, 100), 8, (134, 134)),
    (2, (150, 100, 0, 100), 8, (134, 119)),
    (3, 100, 2, (123, 123, 123)),
    (3, 100, 4, (125, 125, 125)),
    (3, 150, 16, (147, 147, 147)),
    (3, (150, 100, 150, 100, 150, 100), 8, (134, 134, 134)),
    (3, (150, 100, 0, 100, 0, 150), 8, (134, 119, 124)),
]


@pytest.mark.parametrize("dim, length, order, extended", EXTENDED)
def test_extended_shape(dim, length, order, extended):
    m = _model(dim, order=order)
    m.config_boundary(damping_length=length)
    assert m.extended_shape == extended


@pytest.mark.parametrize("dim, length, order, extended", EXTENDED)
def test_padded_arrays_take_the_extended_shape(dim, length, order, extended):
    # tests/test_space_model.py:234-267
    m = _model(dim, order=order, density=True)
    m.config_boundary(damping_length=length)
    for a in (m.damping_mask, m.extended_grid, m.extended_velocity_model,
              m.extended_density_model):
        assert a.shape == extended


@pytest.mark.parametrize("dim", [2, 3])
def test_grid(dim):
    # tests/test_space_model.py:89-102
    m = _model(dim)
    assert m.grid.shape == m.shape and m.grid.dtype == m.dtype


@pytest.mark.parametrize("dim, length, nbl", [
    (2, None, (0, 0, 0, 0)),
    (3, None, (0,) * 6),
    (2, 120, (12,) * 4),
    (3, 90, (9,) * 6),
    (2, (50, 60, 75, 80), (5, 6, 7, 8)),
    (3, (0, 10, 8, 50, 20, 30), (0, 1, 0, 5, 2, 3)),
])
def test_layer_points(dim, length, nbl):
    # tests/test_space_model.py:104-126: widths rounded down to whole points
    m = _model(dim)
    if length is not None:
        m.config_boundary(damping_length=length)
    assert m.nbl == nbl


@pytest.mark.parametrize("order, weights", [
    (2, [-2.0, 1.0]),
    (4, [-2.5, 1.3333334, -0.08333334]),
    (8, [-2.8472223, 1.6, -0.2, 2.5396826e-02, -1.7857143e-03]),
])
def test_second_derivative_weights(order, weights):
    # tests/test_space_model.py:128-149
    m = _model(2, (0, 500, 0, 500), order=order)
    assert np.allclose(m.fd_coefficients(2), np.asarray(weights, dtype=m.dtype))


@pytest.mark.parametrize("dim, order, halo", [
    (2, 2, (1,) * 4), (2, 4, (2,) * 4), (2, 20, (10,) * 4),
    (3, 2, (1,) * 6), (3, 8, (4,) * 6), (3, 10, (5,) * 6),
])
def test_halo_size(dim, order, halo):
    # tests/test_space_model.py:151-170
    assert _model(dim, (0, 500) * dim, order=order).halo_size == halo


@pytest.mark.parametrize("dim, length, bc, degree, alpha", [
    (2, 500, "none", 2, 0.1),
    (2, (50, 50, 40, 40), "null_neumann", 4, 0.001),
    (3, 100, "null_dirichlet", 4, 0.001),
    (2, 75, ("none", "null_neumann", "none", "null_dirichlet"), 4, 0.001),
    (3, (5, 5, 5, 5, 6, 6), "null_dirichlet", 1, 0.001),
])
def test_config_boundary(dim, length, bc, degree, alpha):
    # tests/test_space_model.py:172-232: scalars apply to every side
    m = _model(dim, (0, 500) * dim)
    m.config_boundary(damping_length=length, boundary_condition=bc,
                      damping_polynomial_degree=degree, damping_alpha=alpha)
    sides = 2 * dim
    assert m.damping_length == ((length,) * sides if np.isscalar(length) else tuple(length))
    assert m.boundary_condition == ((bc,) * sides if isinstance(bc, str) else bc)
    assert (m.damping_polynomial_degree, m.damping_alpha) == (degree, alpha)


def test_time_model_properties():
    # tests/test_time_model.py:8-31: dt is held in the model's precision
    sm = sw.SpaceModel(bounding_box=(0, 100, 0, 100), grid_spacing=(10, 10),
                       velocity_model=1500 * np.ones((10, 10)))
    tm = sw.TimeModel(space_model=sm, tf=1.0, t0=0.0, saving_stride=1)
    tm.dt = 0.001
    assert tm.space_model == sm
    assert (tm.tf, tm.t0, tm.saving_stride) == (1.0, 0.0, 1)
    assert tm.dt == sm.dtype(0.001)


@pytest.mark.parametrize("dim, coords", [
    (2, [(0, 25)]), (2, [(0, 25), [250, 250]]), (3, [(0.5, 50.8, 500)]),
])
def test_source_properties(dim, coords):
    # tests/test_source.py:8-43
    sm = _model(dim, (0, 500) * dim)
    src = sw.Source(sm, coordinates=coords, window_radius=8)
    assert src.space_model == sm
    assert (src.window_radius, src.count) == (8, len(coords))
    assert np.array_equal(src.coordinates, sm.dtype(coords))


@pytest.mark.parametrize("bbox, spacing, coords, positions", [
    ((0, 5120, 0, 5120), (10, 10), (0, 512), (0, 51.2)),
    ((0, 5120, 0, 5120), (10, 5), (120, 500), (12, 100)),
    ((0, 500, 20, 500, 0, 200), (20, 20, 20), (10, 20, 100), (0.5, 0.0, 5.0)),
])
def test_source_grid_positions(bbox, spacing, coords, positions):
    # tests/test_source.py:45-76: coordinates in grid units from the box origin
    sm = _model(len(spacing), bbox, spacing)
    src = sw.Source(sm, coordinates=coords, window_radius=4)
    assert np.array_equal(src.grid_positions, np.asarray([positions], dtype=sm.dtype))


@pytest.mark.parametrize("dim, length, order, coords, positions", [
    (2, 500, 2, (0, 0), [(51, 51)]),
    (2, 0, 2, (0, 0), [(1, 1)]),
    (2, 0, 4, (250, 100), [(27, 12)]),
    (2, 50, 16, (255, 255), [(38.5, 38.5)]),
    (3, (50, 0, 50, 0, 0, 0), 16, (255, 255, 0), [(38.5, 38.5, 8)]),
    (3, 2, 4, (250, 100, 100), [(27, 12, 12)]),
])
def test_source_positions_on_the_extended_grid(dim, length, order, coords, positions):
    # tests/test_source.py:78-116: shifted by the layer and the halo
    sm = _model(dim, (0, 500) * dim, order=order)
    sm.config_boundary(damping_length=length)
    src = sw.Source(sm, coordinates=coords)
    assert np.array_equal(src.adjusted_grid_positions, sm.dtype(positions))
