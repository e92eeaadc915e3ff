"""Oracle parity at the benchmark workloads' own sizes.

* The 3D benchmark shot: 384^3 model at 12.5 m -> 472^3 extended grid,
  order 8, Gardner density, 40-point damping layer, 16384 receivers, saving
  stride 50, truncated to its first 51 time steps (same dt, wavelet and
  windows), through the drop-in host call and through the device entry under
  the default kernel policy.
* A batched shot at the largest size and order of the batch workload: a
  2048^2 model (2168^2 extended) at order 20, the full 883 time steps,
  through the batch engine.
* A served 3D shot at the largest size of the served workload: a 320^3
  Gardner-density model (396^3 extended) at order 16, first 41 time steps.

Each is compared with the CPU oracle (the C restatement of the reference's
kernels, OpenMP on all host cores) on the same inputs: relative L2 of the
whole wavefield array and of the shot record <= 1e-4 (float32).
"""
import numpy as np
import pytest

import oracle
import simwave_gb300 as sw
from _cases import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-4
# SIMWAVE_POLICY_* of the kernel the default policy runs for order 8 with
# variable density (the kernel the benchmark times)
BENCH_KERNEL = 10  # SIMWAVE_POLICY_STAGE_RELEASE


def _oracle(kw):
    k = dict(kw, u_full=np.zeros_like(kw["u_full"]),
             shot_record=np.zeros_like(kw["shot_record"]))
    u, rec, _ = oracle.forward("port", x_stride="layout", **k)
    return u, rec


def _check(got_u, got_rec, want_u, want_rec, what):
    assert np.all(np.isfinite(got_u)), what + ": wavefield not finite"
    eu, er = rel_l2(got_u, want_u), rel_l2(got_rec, want_rec)
    assert eu <= TOL, "%s: wavefield rel L2 %.3e" % (what, eu)
    assert er <= TOL, "%s: shot record rel L2 %.3e" % (what, er)


@pytest.fixture(scope="module")
def headline():
    import bench
    kw = bench.vd3d_arguments(timesteps=51, stride=50)
    assert kw["u_full"].shape[1:] == (472, 472, 472)
    assert kw["num_receivers"] == 16384 and kw["space_order"] == 8
    u, rec = _oracle(kw)
    assert np.abs(rec).max() > 0
    return kw, u, rec


def test_headline_shot_dropin(headline):
    from simwave_gb300.backend.middleware import Middleware
    kw, want_u, want_rec = headline
    k = dict(kw, u_full=np.zeros_like(kw["u_full"]),
             shot_record=np.zeros_like(kw["shot_record"]))
    u, rec = Middleware().exec("forward", **k)
    _check(u, rec, want_u, want_rec, "drop-in")


def test_headline_shot_device_default_kernel(headline):
    from simwave_gb300.device import DeviceProblem
    kw, want_u, want_rec = headline
    dp = DeviceProblem(kw)
    stats = dp.run()
    dp.status()
    assert stats["stencil_variant"] == 1  # the tiled 3D kernel
    assert stats["stencil_kernel"] == BENCH_KERNEL
    _check(dp.u_full_numpy(), dp.shot_record_numpy(), want_u, want_rec, "device")


def test_batch_shot_2048sq_order20():
    import bench
    from simwave_gb300.batch import run_batch
    from simwave_gb300.device import DeviceProblem
    rng = np.random.default_rng(5)
    n, h, order = 2048, 10.0, 20
    vel = bench.smooth_velocity((n, n), rng)
    sm = sw.SpaceModel((0, (n - 1) * h, 0, (n - 1) * h), (h, h), vel,
                       space_order=order, dtype=np.float32)
    sm.config_boundary(damping_length=50 * h, boundary_condition="none",
                       damping_polynomial_degree=3, damping_alpha=0.001)
    tm = sw.TimeModel(space_model=sm, tf=1.0, saving_stride=0)
    src = sw.Source(sm, coordinates=[(20.0, 0.37 * (n - 1) * h)], window_radius=4)
    rx = np.linspace(0.0, (n - 1) * h, 1024)
    rec = sw.Receiver(sm, coordinates=np.stack([np.full(1024, 10.0), rx], 1),
                      window_radius=4)
    kw = sw.Solver(sm, tm, src, rec, sw.RickerWavelet(17.0, tm)).forward_arguments()
    assert kw["u_full"].shape[1:] == (2168, 2168) and kw["end_timestep"] == 883
    want_u, want_rec = _oracle(kw)
    (p,) = run_batch([DeviceProblem(kw)])
    _check(p.u_full_numpy(), p.shot_record_numpy(), want_u, want_rec, "batch")


def test_served_3d_shot_320cube_order16():
    from simwave_gb300.backend.middleware import Middleware
    from simwave_gb300.device import DeviceProblem
    n, h, order = 320, 10.0, 16
    shape = (n, n, n)
    z = np.linspace(0, 1, n, dtype=np.float32)[:, None, None]
    vel = np.broadcast_to(1500 + 2500 * z, shape).astype(np.float32)
    vel = (vel * (1 + 0.05 * np.sin(np.linspace(0, 6, n, dtype=np.float32))[None, :, None])
           ).astype(np.float32)
    den = (310.0 * vel ** 0.25).astype(np.float32)
    top = (n - 1) * h
    sm = sw.SpaceModel((0, top, 0, top, 0, top), (h, h, h), vel, den,
                       space_order=order, dtype=np.float32)
    sm.config_boundary(damping_length=30 * h, boundary_condition="none")
    tm = sw.TimeModel(space_model=sm, tf=1.2, saving_stride=0)
    src = sw.Source(sm, coordinates=[[20.0, top / 2, top / 2]], window_radius=4)
    g = np.linspace(0, top, 32)
    gx, gy = np.meshgrid(g, g, indexing="ij")
    coords = np.stack([np.full(gx.size, 10.0), gx.ravel(), gy.ravel()], 1)
    rec = sw.Receiver(sm, coordinates=coords, window_radius=4)
    kw = sw.Solver(sm, tm, src, rec, sw.RickerWavelet(14.0, tm)).forward_arguments()
    T = 41
    kw["end_timestep"] = T
    kw["wavelet"] = np.ascontiguousarray(kw["wavelet"][:T])
    kw["wavelet_size"] = T
    kw["shot_record"] = np.zeros((T, kw["num_receivers"]), np.float32)
    assert kw["u_full"].shape[1:] == (396, 396, 396)
    want_u, want_rec = _oracle(kw)
    dp = DeviceProblem(kw)
    dp.run()
    dp.status()
    _check(dp.u_full_numpy(), dp.shot_record_numpy(), want_u, want_rec, "device")
    k = dict(kw, u_full=np.zeros_like(kw["u_full"]),
             shot_record=np.zeros_like(kw["shot_record"]))
    u, rec = Middleware().exec("forward", **k)
    _check(u, rec, want_u, want_rec, "drop-in")
