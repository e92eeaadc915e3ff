"""Front-end restatement: known answers from the reference's unit tests and
bit-identity with the reference's own front-end output (golden fixtures)."""
import numpy as np
import pytest

import simwave_gb300 as sw
from simwave_gb300.frontend import fd, kws
from _cases import CASE_FIXTURES, load_fixture

import make_golden  # tests/golden/make_golden.py (case table + builders)


# reference tests/test_space_model.py:133-155
@pytest.mark.parametrize("order, coeffs", [
    (2, [-2., 1.]),
    (4, [-2.5, 1.3333334, -0.08333334]),
    (8, [-2.8472223e+00, 1.6e+00, -2.0e-01, 2.5396826e-02, -1.7857143e-03]),
])
def test_fd_coefficients_known(order, coeffs):
    vel = 1500 * np.ones((50, 50))
    sm = sw.SpaceModel((0, 500, 0, 500), (10, 10), vel, space_order=order)
    assert np.allclose(sm.fd_coefficients(2), np.asarray(coeffs, np.float32))


@pytest.mark.parametrize("order", range(2, 22, 2))
def test_fd_weights_moments(order):
    r = order // 2
    off = np.arange(-r, r + 1, dtype=np.float64)
    for deriv in (1, 2):
        w = fd.coefficients(deriv, order)
        for m in range(order + 1):
            target = 2.0 if (deriv == 2 and m == 2) else (1.0 if (deriv == 1 and m == 1) else 0.0)
            assert abs(np.sum(w * off ** m) - target) < 1e-9 * max(1, r ** m)


# reference tests/test_time_model.py:33-65
@pytest.mark.parametrize("dt, tf, t0, stride, steps", [
    (0.001, 1.0, 0.0, 0, 1001), (0.001, 1.0, 0.5, 0, 501),
    (0.002, 2.0, 0.0, 0, 1001), (0.001, 1.0, 0.0, 1, 1001),
    (0.001, 1.0, 0.5, 1, 501), (0.002, 2.0, 0.0, 1, 1001),
    (0.001, 1.0, 0.0, 2, 1001), (0.001, 1.0, 0.5, 6, 505),
    (0.002, 2.0, 0.0, 3, 1003),
])
def test_timesteps(dt, tf, t0, stride, steps):
    sm = sw.SpaceModel((0, 100, 0, 100), (10, 10), 1500 * np.ones((10, 10)))
    tm = sw.TimeModel(space_model=sm, tf=tf, t0=t0, saving_stride=stride)
    tm.dt = dt
    assert tm.timesteps == steps


# reference tests/test_source.py:111-164 (values to float32 precision; the
# reference's own array_equal differs by 1 ulp under scipy 1.18 as well)
@pytest.mark.parametrize("dim, radius, damping, order, coords, points, values", [
    (2, 1, 50, 2, (250, 250), [30, 32, 30, 32],
     [-1.9556131e-08, 1.0000001e+00, -1.9556131e-08,
      -1.9556131e-08, 1.0000001e+00, -1.9556131e-08]),
    (3, 4, 0, 4, (255, 250, 100), [24, 31, 23, 31, 8, 16],
     [-5.1983586e-03, 3.6357623e-02, -1.3933791e-01, 6.0838646e-01,
      6.0838646e-01, -1.3933791e-01, 3.6357623e-02, -5.1983586e-03,
      3.1170111e-10, -3.7239498e-10, 1.2889303e-08, -2.3163784e-08,
      9.9999994e-01, -2.3163784e-08, 1.2889303e-08, -3.7239498e-10,
      3.1170111e-10, 3.1170111e-10, -3.7239498e-10, 1.2889303e-08,
      -2.3163784e-08, 9.9999994e-01, -2.3163784e-08, 1.2889303e-08,
      -3.7239498e-10, 3.1170111e-10]),
])
def test_kws_known_values(dim, radius, damping, order, coords, points, values):
    shape = (50,) * dim
    sm = sw.SpaceModel((0, 500) * dim, (10,) * dim, 1500 * np.ones(shape),
                       space_order=order)
    sm.config_boundary(damping_length=damping)
    src = sw.Source(sm, coordinates=coords, window_radius=radius)
    p, v, off = src.interpolated_points_and_values
    assert np.array_equal(p, np.asarray(points))
    np.testing.assert_allclose(v, np.float32(values), rtol=2e-7, atol=1e-12)
    assert list(off) == [0, len(values)]


def test_kws_matches_full_axis_evaluation():
    rng = np.random.default_rng(3)
    for radius in range(1, 11):
        n = 64
        pos = rng.uniform(0, n - 1, size=(17, 2)).astype(np.float32)
        p, v, off = kws.interpolated_points_and_values((n, n), pos, radius, np.float32)
        for i in range(len(pos)):
            expect = []
            for a in range(2):
                full = kws.kaiser_windowing_sinc(n, pos[i, a], radius)
                idx = np.nonzero(~np.isnan(full))[0]
                assert (p[4 * i + 2 * a], p[4 * i + 2 * a + 1]) == (idx[0], idx[-1])
                expect.append(full[idx].astype(np.float32))
            assert np.array_equal(v[off[i]:off[i + 1]], np.concatenate(expect))


def test_kws_rejects_bad_half_width():
    with pytest.raises(Exception):
        kws.get_kaiser_half_width(11)


def test_space_model_validation():
    vel = 1500 * np.ones((10, 10))
    with pytest.raises(ValueError):
        sw.SpaceModel((0, 90, 0, 90), (10, 10), vel, space_order=3)
    with pytest.raises(ValueError):
        sw.SpaceModel((0, 90, 0, 90), (10, 10), vel, space_order=22)
    sm = sw.SpaceModel((0, 90, 0, 90), (10, 10), vel, space_order=4)
    with pytest.raises(ValueError):
        sm.config_boundary(boundary_condition="periodic")


def test_shapes_and_padding():
    # reference tests/test_space_model.py shape/extended-shape/nbl semantics
    vel = 1500 * np.ones((50, 60))
    sm = sw.SpaceModel((0, 490, 0, 590), (10, 10), vel, space_order=8)
    sm.config_boundary(damping_length=(30, 50, 0, 100))
    assert sm.shape == (50, 60)
    assert sm.nbl == (3, 5, 0, 10)
    assert sm.extended_shape == (50 + 8 + 8, 60 + 10 + 8)
    assert sm.damping_mask.shape == sm.extended_shape
    assert sm.extended_velocity_model.shape == sm.extended_shape
    u = np.zeros((2,) + sm.extended_shape)
    assert sm.remove_halo_region(u).shape == (2, 58, 70)


def test_interpolation_resamples_when_shape_differs():
    vel = np.linspace(1500, 2500, 512 * 512).reshape(512, 512).astype(np.float32)
    sm = sw.SpaceModel((0, 5120, 0, 5120), (10, 10), vel, space_order=4)
    assert sm.velocity_model.shape == (513, 513)
    assert sm.velocity_model.dtype == np.float32
    assert abs(float(sm.velocity_model[0, 0]) - 1500) < 1e-3


@pytest.mark.parametrize("name", CASE_FIXTURES)
def test_frontend_matches_reference_frontend(name):
    """Every kernel input this front end builds equals the reference's."""
    meta, ref = load_fixture(name)
    spec = make_golden.CASES[name]
    seed = 100 + 7 * list(make_golden.CASES).index(name)
    sm, tm, src, rec, wav = make_golden.build_case(sw, name, spec, seed)
    assert tm.timesteps == meta["timesteps"]
    assert float(tm.dt) == meta["dt"]
    assert list(sm.extended_shape) == meta["extended_shape"]
    assert np.array_equal(sm.extended_velocity_model, ref["velocity_model"])
    if "density_model" in ref:
        assert np.array_equal(sm.extended_density_model, ref["density_model"])
    assert np.array_equal(sm.damping_mask, ref["damping_mask"])
    assert np.array_equal(wav.values, ref["wavelet"])
    assert np.array_equal(sm.fd_coefficients(2), ref["second_order_fd_coefficients"])
    assert np.array_equal(sm.fd_coefficients(1), ref["first_order_fd_coefficients"])
    for obj, tag in ((src, "src"), (rec, "rec")):
        p, v, o = obj.interpolated_points_and_values
        assert np.array_equal(p, ref[tag + "_points_interval"])
        assert np.array_equal(o, ref[tag + "_points_values_offset"])
        assert np.array_equal(v, ref[tag + "_points_values"])


def test_solver_snapshot_bookkeeping():
    vel = 1500 * np.ones((20, 20), dtype=np.float32)
    sm = sw.SpaceModel((0, 190, 0, 190), (10, 10), vel, space_order=4)
    for stride in (0, 1, 2, 5):
        tm = sw.TimeModel(sm, tf=0.3, saving_stride=stride)
        src = sw.Source(sm, coordinates=[(100, 100)])
        solver = sw.Solver(sm, tm, src, src, sw.RickerWavelet(10, tm))
        T = tm.timesteps
        if stride == 0:
            assert solver.snapshot_indexes == [T - 1]
        else:
            assert T % stride == 1 or stride == 1
            assert solver.snapshot_indexes == list(range(0, T, stride))
        assert solver.u_full.shape == (solver.num_snapshots + 2,) + sm.extended_shape
        assert solver.shot_record.shape == (T, 1)
