"""Accuracy against the analytic solution and convergence rates.

Restates the reference's numerical-analysis tests
(tests/test_convergence.py:77-139 and tests/test_gpu_convergence.py of the
reference) on this package's front end and GPU path: a constant-velocity
2D model (c = 1.5 on the box (-40, 440)^2, no damping layer), a Ricker
source at (200, 200) and one receiver at (260, 260), compared with the
analytic 2D solution. Same cases and thresholds as the reference:

* accuracy: order 8, h = 0.5, dt = 0.1, tf = 150.075: RMS error < 1e-4;
* time convergence: dt in {0.1, 0.075, 0.04, 0.025}: the slope of
  log(error) against log(dt) > 1.7;
* space convergence: h in {2, 2.5, 4} at dt = 0.025: slopes above
  1.7, 4, 6, 7.7, 8.7 for orders 2, 4, 6, 8, 10.

The numerical trace is the shot record divided by h^2, as the reference's
test scales it (tests/test_convergence.py:66). The CPU oracle passes the
accuracy case as well (`test_oracle_accuracy`, in the CPU suite), which pins
the comparison itself.
"""
import numpy as np
import pytest

import simwave_gb300 as sw

BBOX = (-40.0, 440.0, -40.0, 440.0)
VEL = 1.5
F0 = 0.09
SRC = [(200.0, 200.0)]
REC = [(260.0, 260.0)]
T0, TF = 0.0, 150.075


def _problem(spacing, order, dt):
    """Solver of the reference's convergence model with ``dt`` imposed."""
    sm = sw.SpaceModel(bounding_box=BBOX, grid_spacing=(spacing, spacing),
                       velocity_model=VEL * np.ones((100, 100), dtype=np.float64),
                       space_order=order)
    tm = sw.TimeModel(space_model=sm, t0=T0, tf=TF)
    tm.dt = dt
    src = sw.Source(sm, coordinates=SRC)
    rec = sw.Receiver(sm, coordinates=REC)
    wav = sw.RickerWavelet(F0, tm)
    return sw.Solver(sm, tm, src, rec, wav), sm, tm


def analytic_trace(space_model, dt):
    """Pressure at the receiver from the 2D Green's function of the
    constant-velocity wave equation, convolved with the Ricker wavelet in
    the frequency domain: u(f) = -i pi H0^(2)(2 pi f r / c) q(f) / (2 pi),
    with q the spectrum of the wavelet sampled at ``dt`` over 0..3000 (a
    window long enough that the periodic inverse transform does not wrap
    within the simulated time)."""
    from scipy.special import hankel2
    long_tm = sw.TimeModel(space_model=space_model, t0=0.0, tf=3000.0)
    long_tm.dt = dt
    w = sw.RickerWavelet(F0, long_tm).values
    n = long_tm.timesteps
    nf = n // 2 + 1
    freqs = np.arange(nf) / long_tm.tf
    q = np.fft.fft(w)[:nf]
    r = np.hypot(REC[0][0] - SRC[0][0], REC[0][1] - SRC[0][1])
    k = 2.0 * np.pi * freqs / VEL
    g = np.zeros(nf, dtype=complex)
    g[1:-1] = hankel2(0, k[1:-1] * r)  # zero at f = 0 and at the last bin
    return np.real(np.fft.ifft(-1j * np.pi * g * q, n)) / (2.0 * np.pi)


def rms_error(trace, space_model, time_model, dt):
    spacing = space_model.grid_spacing[0]
    num = np.asarray(trace, dtype=np.float64).ravel() / spacing ** 2
    exact = analytic_trace(space_model, dt)[:time_model.timesteps]
    return np.linalg.norm(num - exact) / np.sqrt(num.size)


def gpu_error(spacing, order, dt):
    solver, sm, tm = _problem(spacing, order, dt)
    _, rec = solver.forward()
    return rms_error(rec, sm, tm, dt)


def slope(x, y):
    return np.polyfit(np.log(x), np.log(y), 1)[0]


@pytest.mark.gpu
def test_accuracy():
    assert gpu_error(0.5, 8, 0.1) < 1e-4


@pytest.mark.gpu
def test_convergence_in_time():
    dts = [0.1, 0.075, 0.04, 0.025]
    errs = [gpu_error(0.5, 8, dt) for dt in dts]
    assert slope(dts, errs) > 1.7, errs


@pytest.mark.gpu
def test_convergence_in_space():
    spacings = [2.0, 2.5, 4.0]
    for order, rate in zip([2, 4, 6, 8, 10], [1.7, 4, 6, 7.7, 8.7]):
        errs = [gpu_error(h, order, 0.025) for h in spacings]
        assert slope(spacings, errs) > rate, (order, errs)


def test_oracle_accuracy():
    """The CPU oracle (the reference's kernels restated in C) on the
    accuracy case: the analytic comparison accepts it too."""
    import oracle
    solver, sm, tm = _problem(0.5, 8, 0.1)
    kw = solver.forward_arguments()
    _, rec, _ = oracle.forward("port", x_stride="layout", **kw)
    assert rms_error(rec, sm, tm, 0.1) < 1e-4
