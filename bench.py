"""Benchmark: simwave forward propagation on one GB300.

Workload (default): 3D variable-density acoustic forward, 384^3 float32
model at 12.5 m (472^3 extended grid: 40-point damping layer of degree 3 and
alpha 0.001, order-8 halo), velocity 1500 + 3000 smoothstep(depth) with seeded
Gaussian-smoothed noise (sigma 8 points, +-10 %) clipped to [1500, 4500] m/s,
Gardner density 310 v^0.25, boundary 'none', tf 1.5 s (T = 1201 CFL steps),
15 Hz Ricker at the surface centre, 128 x 128 receiver carpet at 10 m depth,
saving stride 50 (25 snapshots). Synthetic, seeded inputs.

One "step" is one complete forward run (all T time steps) of that shot.
Metric: grid-point updates per second (interior points x time steps) in
Gpts/s, whole job over all ranks.

  value       device-resident inputs (simwave_forward_device), CUDA events on
              the launching stream around each run
  e2e         the reference-facing C ABI (the drop-in `forward` the
              Middleware calls) with host numpy buffers; host<->device copies
              inside the timed region
  roofline    stencil kernel: algorithmic bytes per launch (20 B per interior
              point: read u_cur, u_prev, velocity, density, write u_next) over
              its mean launch time (CUDA events on the same stream)
  cpu_baseline the CPU oracle (C restatement, OpenMP, all host cores) on a
              bounded sample of the same workload (fewer time steps)

Extra legs in the same line (rank 0): `batched` (96 2D shots advanced
together vs back-to-back plain device calls), `served` (a Poisson stream of
mixed 2D/3D requests through the continuous-batching server vs the same
requests through the drop-in one after another: p50/p99, shots/s) and
`gradient` (misfit and velocity gradient of 16 2D shots with checkpointed
recomputation, plus a finite-difference check); `--no-batched`,
`--no-served`, `--no-gradient` skip them, `--served` / `--gradient` run one
alone.

`--impl reference` times the reference's CPU algorithm (the C restatement)
on the host cores instead and prints the same metric.
Multi-GPU (torchrun): independent replicas, one shot per rank, no collective
on the data path.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gpts/s (grid-point updates/s) and HBM GB/s vs roofline, 3D VD so8 forward"
BYTES_PER_UPDATE = {False: 16, True: 20}  # float32, constant / variable density

_MODEL_CACHE = {}


def _smooth_noise(shape, sigma, seed):
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    g = gaussian_filter(rng.standard_normal(shape).astype(np.float32), sigma,
                        mode="wrap")
    return g / np.abs(g).max()


def vd3d_model(n=384):
    if n in _MODEL_CACHE:
        return _MODEL_CACHE[n]
    z = np.linspace(0.0, 1.0, n, dtype=np.float32)
    smooth = 3 * z ** 2 - 2 * z ** 3
    base = 1500.0 + 3000.0 * smooth
    noise = _smooth_noise((n, n, n), 8.0, seed=2024)
    vel = base[:, None, None] * (1.0 + 0.1 * noise)
    vel = np.clip(vel, 1500.0, 4500.0).astype(np.float32)
    den = (310.0 * vel ** 0.25).astype(np.float32)
    _MODEL_CACHE[n] = (vel, den)
    return vel, den


def vd3d_arguments(timesteps=None, n=384, stride=50, dtype=np.float32):
    """Middleware keyword arguments of the 3D benchmark shot.

    ``timesteps`` truncates the run (same dt and wavelet samples) for tests
    and bounded CPU samples."""
    import simwave_gb300 as sw
    vel, den = vd3d_model(n)
    h = 12.5
    top = (n - 1) * h
    sm = sw.SpaceModel((0, top, 0, top, 0, top), (h, h, h), vel, den,
                       space_order=8, dtype=dtype)
    sm.config_boundary(damping_length=40 * h, boundary_condition="none",
                       damping_polynomial_degree=3, damping_alpha=0.001)
    tm = sw.TimeModel(space_model=sm, tf=1.5, saving_stride=stride)
    centre = top / 2
    src = sw.Source(sm, coordinates=[(0.0, centre, centre)], window_radius=4)
    g = (np.arange(128) + 0.5) * (top / 128)
    gx, gy = np.meshgrid(g, g, indexing="ij")
    carpet = np.stack([np.full(gx.size, 10.0), gx.ravel(), gy.ravel()], axis=1)
    rec = sw.Receiver(sm, coordinates=carpet, window_radius=4)
    solver = sw.Solver(sm, tm, src, rec, sw.RickerWavelet(15.0, tm))
    kw = solver.forward_arguments()
    if timesteps is not None and timesteps < kw["end_timestep"]:
        T = int(timesteps)
        if stride > 1 and T % stride != 1:
            raise ValueError("a run with saving stride %d needs T %% stride == 1"
                             " (T = %d)" % (stride, T))
        kw["end_timestep"] = T
        kw["wavelet"] = np.ascontiguousarray(kw["wavelet"][:T])
        kw["wavelet_size"] = T
        kw["shot_record"] = np.zeros((T, kw["num_receivers"]), dtype)
        nsnap = 1 if stride == 0 else len(range(0, T, stride))
        kw["num_snapshots"] = nsnap + 2
        kw["u_full"] = np.zeros((nsnap + 2,) + kw["u_full"].shape[1:], dtype)
    return kw


def smooth_velocity(shape, rng, lo=1500.0, hi=4500.0, modes=6):
    """Seeded smooth random field in [lo, hi]: a few low-wavenumber modes."""
    z = np.linspace(0.0, 1.0, shape[0])[:, None]
    x = np.linspace(0.0, 1.0, shape[1])[None, :]
    f = np.zeros(shape)
    for _ in range(modes):
        kz, kx = rng.uniform(0.5, 3.0, size=2)
        pz, px = rng.uniform(0, 2 * np.pi, size=2)
        f += rng.uniform(0.3, 1.0) * np.sin(2 * np.pi * kz * z + pz) * np.cos(
            2 * np.pi * kx * x + px)
    f = (f - f.min()) / max(f.max() - f.min(), 1e-12)
    return (lo + (hi - lo) * f).astype(np.float32)


def batch2d_arguments(nshots=96, seed=7, max_side=2048, dtype=np.float32, pick=None):
    """The batched workload: 2D constant-density shots with seeded grids of
    256..max_side points per side (10 m), orders {4, 8, 12, 16, 20}, smooth
    random velocity 1500-4500 m/s, 50-point damping layer, an 8-25 Hz Ricker
    source and 256-1024 surface receivers, tf = 1.0 s."""
    import simwave_gb300 as sw
    rng = np.random.default_rng(seed)
    out, skipped = [], []
    for _ in range(nshots):
        nz, nx = (int(v) for v in rng.integers(256, max_side + 1, size=2))
        order = int(rng.choice([4, 8, 12, 16, 20]))
        h = 10.0
        vel = smooth_velocity((nz, nx), rng)
        if pick is not None and len(out) + len(skipped) not in pick:
            # skipped shot: the same draws, so later shots are unchanged
            skipped.append(None)
            rng.uniform(0.2, 0.8)
            rng.integers(256, 1025)
            rng.uniform(8.0, 25.0)
            continue
        sm = sw.SpaceModel((0, (nz - 1) * h, 0, (nx - 1) * h), (h, h), vel,
                           space_order=order, dtype=dtype)
        sm.config_boundary(damping_length=50 * h, boundary_condition="none",
                           damping_polynomial_degree=3, damping_alpha=0.001)
        tm = sw.TimeModel(space_model=sm, tf=1.0, saving_stride=0)
        xs = float(rng.uniform(0.2, 0.8) * (nx - 1) * h)
        src = sw.Source(sm, coordinates=[(20.0, xs)], window_radius=4)
        nrec = int(rng.integers(256, 1025))
        rx = np.linspace(0.0, (nx - 1) * h, nrec)
        rec = sw.Receiver(sm, coordinates=np.stack([np.full(nrec, 10.0), rx], 1),
                          window_radius=4)
        wav = sw.RickerWavelet(float(rng.uniform(8.0, 25.0)), tm)
        out.append(sw.Solver(sm, tm, src, rec, wav).forward_arguments())
    return out


def batched_leg(nshots=96, max_side=2048):
    """Shots/s of back-to-back single-shot runs vs one batch (resident)."""
    import torch
    from simwave_gb300.batch import BatchEngine, autotune, run_batch
    from simwave_gb300.device import DeviceProblem
    kws = batch2d_arguments(nshots, max_side=max_side)
    probs = [DeviceProblem(k) for k in kws]
    updates = sum(interior_updates(k)[1] for k in kws)
    stream = torch.cuda.current_stream()
    # plain: one simwave_forward_device call per shot, back to back (every
    # shot once untimed first, so no kernel is loaded inside the timing)
    for p in probs:
        p.run()
    probs[-1].status()
    for p in probs:
        p.reset()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for p in probs:
        p.run(stream)
    e1.record(stream)
    e1.synchronize()
    plain_s = e0.elapsed_time(e1) / 1e3
    # drop-in: the reference-facing host call (what Solver.forward makes),
    # one shot after another with host arrays in and out; one shot per order
    # first so that no kernel is loaded inside the timing
    import contextlib
    import io
    from simwave_gb300.backend.middleware import Middleware
    mw = Middleware()

    def dropin(k):
        with contextlib.redirect_stdout(io.StringIO()):
            mw.exec("forward", **dict(k, u_full=np.zeros_like(k["u_full"]),
                                      shot_record=np.zeros_like(k["shot_record"])))

    for order in sorted({int(k["space_order"]) for k in kws}):
        dropin(next(k for k in kws if int(k["space_order"]) == order))
    t0 = time.perf_counter()
    for k in kws:
        dropin(k)
    dropin_s = time.perf_counter() - t0
    # batch: tile height and time-blocking depth picked per order, then one
    # engine for all shots
    tiles = autotune(probs)
    eng = BatchEngine()
    eng.apply(tiles)
    for p in probs:
        p.reset()
    torch.cuda.synchronize()
    e0.record(stream)
    run_batch(probs, engine=eng)
    e1.record(stream)
    e1.synchronize()
    batch_s = e0.elapsed_time(e1) / 1e3
    launches = eng.launches()
    eng.close()
    return {"workload": "%d 2D CD shots, 256..%d per side, orders 4-20, tf 1 s"
                        % (nshots, max_side),
            "shots_per_s": round(nshots / batch_s, 2),
            "plain_shots_per_s": round(nshots / plain_s, 2),
            "speedup_vs_plain": round(plain_s / batch_s, 2),
            "dropin_shots_per_s": round(nshots / dropin_s, 2),
            "speedup_vs_dropin": round(dropin_s / batch_s, 2),
            "batch_gpts": round(updates / batch_s / 1e9, 2),
            "plain_gpts": round(updates / plain_s / 1e9, 2),
            "tuning": {str(k): v for k, v in tiles.items()}, "batch_launches": int(launches),
            "timing": "CUDA events, inputs resident; batch: admission, steps and release "
                      "of all shots; plain: one device call per shot (its own preparation "
                      "included); drop-in: wall clock of the host calls, copies included"}


def served_requests(nreq=40, seed=11, rate=200.0, frac3d=0.25, max2d=2048, max3d=320,
                     dtype=np.float32, pick=None):
    """The served workload: Poisson arrivals (seeded, ``rate`` per second) of
    2D shots (512..max2d per side) and 3D shots (128..max3d per side), orders
    4-16, float32, constant or Gardner density, tf 0.5-2.0 s, 10 m grids,
    30-point damping layer, one source, surface receivers."""
    import simwave_gb300 as sw
    from simwave_gb300.serve import Request
    rng = np.random.default_rng(seed)
    reqs, t = [], 0.0
    for i in range(nreq):
        t += float(rng.exponential(1.0 / rate))
        is3d = rng.random() < frac3d
        order = int(rng.choice([4, 6, 8, 10, 12, 14, 16]))
        gardner = bool(rng.integers(0, 2))
        tf = float(rng.uniform(0.5, 2.0))
        h = 10.0
        if is3d:
            n = int(rng.integers(128, max3d + 1))
            shape = (n, n, n)
            z = np.linspace(0, 1, n, dtype=np.float32)[:, None, None]
            vel = np.broadcast_to(1500 + 2500 * z, shape).astype(np.float32)
            vel = vel * (1 + 0.05 * np.sin(np.linspace(0, 6, n, dtype=np.float32))[None, :, None])
        else:
            shape = tuple(int(v) for v in rng.integers(512, max2d + 1, size=2))
            vel = smooth_velocity(shape, rng)
        vel = vel.astype(np.float32)
        den = (310.0 * vel ** 0.25).astype(np.float32) if gardner else None
        box = []
        for a in range(len(shape)):
            box += [0.0, (shape[a] - 1) * h]
        if pick is not None and i not in pick:
            rng.uniform(8.0, 20.0)  # the skipped request's Ricker draw
            continue
        sm = sw.SpaceModel(tuple(box), (h,) * len(shape), vel, den, space_order=order,
                           dtype=dtype)
        sm.config_boundary(damping_length=30 * h, boundary_condition="none")
        tm = sw.TimeModel(space_model=sm, tf=tf, saving_stride=0)
        mid = [(shape[a] - 1) * h / 2 for a in range(len(shape))]
        src = sw.Source(sm, coordinates=[[20.0] + mid[1:]], window_radius=4)
        if is3d:
            g = np.linspace(0, (shape[1] - 1) * h, 32)
            gx, gy = np.meshgrid(g, g, indexing="ij")
            coords = np.stack([np.full(gx.size, 10.0), gx.ravel(), gy.ravel()], 1)
        else:
            coords = np.stack([np.full(256, 10.0), np.linspace(0, (shape[1] - 1) * h, 256)], 1)
        rec = sw.Receiver(sm, coordinates=coords, window_radius=4)
        wav = sw.RickerWavelet(float(rng.uniform(8.0, 20.0)), tm)
        kw = sw.Solver(sm, tm, src, rec, wav).forward_arguments()
        reqs.append(Request(kw, t, tag=i))
    return reqs


def warm_arguments(dim, order, vd, big=False):
    """A short shot (tf 0.03 s) of the given class on a 48^2 / 32^3 model, or
    on a 1300^2 one (`big`: past the persistent-launch size of 2D runs), to
    load its kernels before timing (CUDA loads a kernel's code at its first
    launch)."""
    import simwave_gb300 as sw
    n, h = ((1300 if big else 48), 10.0) if dim == 2 else (32, 10.0)
    shape = (n,) * dim
    vel = np.full(shape, 2000.0, dtype=np.float32)
    den = np.full(shape, 1000.0, dtype=np.float32) if vd else None
    box = []
    for _ in range(dim):
        box += [0.0, (n - 1) * h]
    sm = sw.SpaceModel(tuple(box), (h,) * dim, vel, den, space_order=order, dtype=np.float32)
    sm.config_boundary(damping_length=5 * h, boundary_condition="none")
    tm = sw.TimeModel(space_model=sm, tf=0.03, saving_stride=0)
    mid = [(n - 1) * h / 2] * dim
    src = sw.Source(sm, coordinates=[mid], window_radius=4)
    rec = sw.Receiver(sm, coordinates=[mid], window_radius=4)
    return sw.Solver(sm, tm, src, rec, sw.RickerWavelet(15.0, tm)).forward_arguments()


def served_leg(nreq=40):
    """p50/p99 latency and shots/s of the continuous-batching server against
    the same requests run one after another through the drop-in host path."""
    import contextlib
    import io
    import torch
    from simwave_gb300.backend.middleware import Middleware
    from simwave_gb300.serve import Request, ShotServer, latency_summary
    reqs = served_requests(nreq)
    arrivals = [r.arrival for r in reqs]
    updates = sum(interior_updates(r.kwargs)[1] for r in reqs)
    # load every kernel class of the workload on both paths first
    classes = sorted({(r.kwargs["velocity_model"].ndim, int(r.kwargs["space_order"]),
                       r.kwargs.get("density_model") is not None) for r in reqs})
    warm = [warm_arguments(*c) for c in classes]
    warm += [warm_arguments(*c, big=True) for c in classes if c[0] == 2]
    with contextlib.redirect_stdout(io.StringIO()):
        for kw in warm:
            Middleware().exec("forward", **dict(kw, u_full=np.zeros_like(kw["u_full"]),
                                                shot_record=np.zeros_like(kw["shot_record"])))
    warm_server = ShotServer(epoch_steps=64)
    warm_server.serve([Request(kw, 0.0) for kw in warm])
    warm_server.close()
    # sequential: Solver.forward's host path, one request at a time
    mw = Middleware()
    service = []
    for r in reqs:
        k = dict(r.kwargs, u_full=np.zeros_like(r.kwargs["u_full"]),
                 shot_record=np.zeros_like(r.kwargs["shot_record"]))
        t0 = time.perf_counter()
        with contextlib.redirect_stdout(io.StringIO()):
            mw.exec("forward", **k)
        service.append(time.perf_counter() - t0)
    done, lat = 0.0, []
    for a, sv in zip(arrivals, service):
        done = max(done, a) + sv
        lat.append(done - a)
    seq = {"p50_ms": round(float(np.percentile(lat, 50)) * 1e3, 2),
           "p99_ms": round(float(np.percentile(lat, 99)) * 1e3, 2),
           "shots_per_s": round(len(reqs) / (done - arrivals[0]), 2),
           "service_s_by_kind": {k: round(sum(sv for r, sv in zip(reqs, service)
                                              if r.kind == k), 3)
                                 for k in sorted({r.kind for r in reqs})}}
    # served: continuous batching
    torch.cuda.synchronize()
    # a serving process keeps its device memory: reserve the workload's
    # footprint in the allocator up front (not timed, like model loading)
    server = ShotServer(epoch_steps=64, reserve_bytes=sum(r.bytes for r in reqs))
    server.serve(reqs)
    server.close()
    served = latency_summary(reqs)
    return {"workload": "%d requests, Poisson 200/s, 2D 512^2-2048^2 and 3D 128^3-320^3, "
                        "orders 4-16, tf 0.5-2 s" % len(reqs),
            "updates": updates, "served": served, "sequential_plain": seq,
            "speedup_shots_per_s": round(served["shots_per_s"] / seq["shots_per_s"], 2)}


def readme2d_arguments(dtype=np.float32):
    """The reference README's 2D case: 512^2 model (1500 m/s above row 100,
    2000 below) interpolated onto the 513^2 grid of a 5120 m box at 10 m,
    order 4, no damping layer, boundaries (null_neumann, null_dirichlet,
    none, null_dirichlet), tf 1.0 s (T 328), 10 Hz Ricker at (2560, 2560)
    with window radius 1, 512 receivers at z = 2560 m, x = 0..5110 m."""
    import simwave_gb300 as sw
    vel = np.full((512, 512), 2000.0, dtype=np.float32)
    vel[:100] = 1500.0
    sm = sw.SpaceModel((0.0, 5120.0, 0.0, 5120.0), (10.0, 10.0), vel, space_order=4,
                       dtype=dtype)
    sm.config_boundary(damping_length=0.0, boundary_condition=(
        "null_neumann", "null_dirichlet", "none", "null_dirichlet"))
    tm = sw.TimeModel(space_model=sm, tf=1.0, saving_stride=0)
    src = sw.Source(sm, coordinates=[(2560.0, 2560.0)], window_radius=1)
    rec = sw.Receiver(sm, coordinates=[(2560.0, x) for x in range(0, 5112, 10)],
                      window_radius=1)
    return sw.Solver(sm, tm, src, rec, sw.RickerWavelet(10.0, tm)).forward_arguments()


def plain2d_leg(reps=20):
    """The reference README's 2D shot (513² grid, order 4; L2- and
    launch-bound): Gpts/s of plain device calls, of the
    same shot through the graph-captured batch engine, of the drop-in with
    host buffers, and of the CPU oracle on the full run (with the relative
    L2 difference of the shot record against it)."""
    import contextlib
    import io
    import torch
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # the CPU baseline and oracle of this leg
    from simwave_gb300.backend.middleware import Middleware
    from simwave_gb300.batch import BatchEngine
    from simwave_gb300.device import DeviceProblem
    kw = readme2d_arguments()
    pts, updates = interior_updates(kw)
    dp = DeviceProblem(kw)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            dp.reset()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    plain_ms = timed(lambda: dp.run())
    eng = BatchEngine()

    def batched():
        sid = eng.add(dp)
        eng.run(dp.timesteps)
        eng.release(sid)
    batch_ms = timed(batched)
    eng.close()
    dp.reset()
    dp.run()
    dp.status()
    gpu_rec = dp.shot_record_numpy()
    mw = Middleware()
    e2e = []
    for i in range(reps // 4 + 1):
        k = dict(kw, u_full=np.zeros_like(kw["u_full"]), shot_record=np.zeros_like(kw["shot_record"]))
        t0 = time.perf_counter()
        with contextlib.redirect_stdout(io.StringIO()):
            mw.exec("forward", **k)
        if i:
            e2e.append(1e3 * (time.perf_counter() - t0))
    k = dict(kw, u_full=np.zeros_like(kw["u_full"]), shot_record=np.zeros_like(kw["shot_record"]))
    t0 = time.perf_counter()
    _, cpu_rec, _ = oracle.forward("port", **k)
    cpu_s = time.perf_counter() - t0
    rel = float(np.linalg.norm(gpu_rec - cpu_rec) / np.linalg.norm(cpu_rec))
    gp = lambda ms: round(updates / (ms / 1e3) / 1e9, 2)  # noqa: E731
    return {"workload": "2D CD so4 513^2 (517^2 extended), T %d, 512 receivers"
                        % kw["end_timestep"],
            "updates": updates, "plain_ms": round(plain_ms, 3), "plain_gpts": gp(plain_ms),
            "graph_ms": round(batch_ms, 3), "graph_gpts": gp(batch_ms),
            "e2e_ms": round(float(np.median(e2e)), 3), "e2e_gpts": gp(float(np.median(e2e))),
            "cpu_port_s": round(cpu_s, 3), "cpu_port_gpts": round(updates / cpu_s / 1e9, 3),
            "cpu_threads": os.cpu_count(),
            "shot_record_rel_l2_vs_cpu": rel,
            "hbm_note": "16 B/update algorithmic; the 5 MB state stays in L2"}


def accuracy_leg():
    """Per workload: the float32 error of the GPU and of the reference's
    C path (the CPU port, bit-identical to the reference build) against the
    float64 run (the CPU port in float64 on the same model, built in float64
    by the front end as the reference's front end does), relative L2 over
    the shot record and the final wavefield. The 472³ 3D shot runs its
    first 51 of 1201 steps; the batched, served and inversion workloads use
    representative shots."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # the oracle of this leg
    from simwave_gb300.device import DeviceProblem

    def rel(a, b):
        a = np.asarray(a, np.float64)
        b = np.asarray(b, np.float64)
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    def cpu(kw):
        k = dict(kw, u_full=np.zeros_like(kw["u_full"]),
                 shot_record=np.zeros_like(kw["shot_record"]))
        u, r, _ = oracle.forward("port", x_stride="layout", **k)
        return u, r

    def gpu(kw):
        dp = DeviceProblem(kw)
        dp.run()
        dp.status()
        return dp.u_full_numpy(), dp.shot_record_numpy()

    true, smooth = inversion_models()
    _, dt5 = inversion_arguments(true, nshots=1)
    cases = [
        ("plain 2D, 513^2 so4", lambda d: readme2d_arguments(dtype=d)),
        ("3D VD so8 472^3, steps 1-51", lambda d: vd3d_arguments(timesteps=51, dtype=d)),
        ("batched shot 3 (1665x1127 so4)", lambda d: batch2d_arguments(12, pick={3}, dtype=d)[0]),
        ("batched shot 7 (666x1382 so16)", lambda d: batch2d_arguments(12, pick={7}, dtype=d)[0]),
        ("served 2D Gardner (1330x811 so12)", lambda d: served_requests(40, pick={0}, dtype=d)[0].kwargs),
        ("served 3D VD (204^3 so8)", lambda d: served_requests(40, pick={11}, dtype=d)[0].kwargs),
        ("inversion shot 0 forward (459x1809 so8)",
         lambda d: inversion_arguments(smooth, dt=dt5, nshots=1, dtype=d)[0][0]),
    ]
    rows = []
    for name, build in cases:
        kw32, kw64 = build(np.float32), build(np.float64)
        u64, r64 = cpu(kw64)
        u32, r32 = cpu(kw32)
        gu, gr = gpu(kw32)
        rows.append({"workload": name,
                     "gpu_f32_vs_f64": {"shot_record": rel(gr, r64), "wavefield": rel(gu, u64)},
                     "ref_f32_vs_f64": {"shot_record": rel(r32, r64), "wavefield": rel(u32, u64)},
                     "gpu_vs_ref_f32": {"shot_record": rel(gr, r32), "wavefield": rel(gu, u32)}})
        print(json.dumps(rows[-1]), flush=True)
    return rows


def inversion_models(seed=5):
    """The inversion workload's models on a (351, 1701) grid of 10 m (nz = 351,
    nx = 1701): 12 layers from 1500 to 5500 m/s cut by two dipping faults
    (seeded), and its Gaussian smoothing with sigma = 20 points (the model
    the gradient is evaluated at)."""
    from scipy.ndimage import gaussian_filter
    nz, nx = 351, 1701
    rng = np.random.default_rng(seed)
    z = np.arange(nz, dtype=np.float64)[:, None]
    x = np.arange(nx, dtype=np.float64)[None, :]
    depths = np.sort(rng.uniform(15.0, 340.0, 11))
    speeds = np.clip(np.linspace(1500.0, 5500.0, 12) + rng.uniform(-80.0, 80.0, 12),
                     1500.0, 5500.0)
    speeds[0], speeds[-1] = 1500.0, 5500.0
    shift = np.zeros((nz, nx))
    for x0, dip, throw in ((520.0, 62.0, 24.0), (1180.0, 71.0, -31.0)):
        trace = x0 + z / np.tan(np.radians(dip))
        shift += np.where(x > trace, throw, 0.0)
    layer = np.searchsorted(depths, z - shift)
    true = speeds[layer].astype(np.float32)
    smooth = gaussian_filter(true.astype(np.float64), 20.0, mode="nearest").astype(np.float32)
    return true, smooth


def inversion_arguments(vel, dt=None, nshots=16, damping_points=50, dtype=np.float32):
    """Middleware keyword arguments of the inversion shots on ``vel``: so 8,
    8 Hz Ricker, tf 3.0 s, sources at 20 m depth spread over x, 1701
    receivers at 10 m depth (one per grid column), a 50-point damping layer
    (deg 3, alpha 0.001) and 'none' edges. ``dt`` overrides the CFL step
    (the observed and modelled data share the true model's step)."""
    import simwave_gb300 as sw
    nz, nx = vel.shape
    h = 10.0
    sm = sw.SpaceModel((0.0, (nz - 1) * h, 0.0, (nx - 1) * h), (h, h), vel,
                       space_order=8, dtype=dtype)
    sm.config_boundary(damping_length=damping_points * h, boundary_condition="none",
                       damping_polynomial_degree=3, damping_alpha=0.001)
    tm = sw.TimeModel(space_model=sm, tf=3.0, dt=dt, saving_stride=0)
    rec = sw.Receiver(sm, coordinates=[(10.0, i * h) for i in range(nx)], window_radius=4)
    wav = sw.RickerWavelet(8.0, tm)
    out = []
    for s in range(nshots):
        xs = (s + 0.5) * (nx - 1) * h / nshots
        src = sw.Source(sm, coordinates=[(20.0, xs)], window_radius=4)
        out.append(sw.Solver(sm, tm, src, rec, wav).forward_arguments())
    return out, float(tm.dt)


def gradient_leg(nshots=16, steps=1, interval=None, workers=4):
    """The inversion workload: L2 misfit and its velocity gradient over the
    shots at the smoothed model, observed data from the true model. Reports
    shots/s, the point updates of the forward, recomputation and adjoint
    passes per second, and a finite-difference check of the gradient along
    a random smooth direction on the first shot."""
    import torch
    from simwave_gb300.device import DeviceProblem
    from simwave_gb300.gradient import default_interval, misfit_gradient, shot_record
    true, smooth = inversion_models()
    kw_true, dt = inversion_arguments(true, nshots=nshots)
    kw_model, _ = inversion_arguments(smooth, dt=dt, nshots=nshots)
    observed = []
    for kw in kw_true:
        p = DeviceProblem(kw)
        p.run()
        observed.append(p.receivers[:, :p.nrec].clone())
        del p
    problems = [DeviceProblem(kw) for kw in kw_model]
    v0 = torch.tensor(kw_model[0]["velocity_model"], device="cuda")
    T = problems[0].timesteps
    K = interval or default_interval(T)
    misfit_gradient(v0, problems[:1], observed[:1], K)  # warm-up
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        loss, grad = misfit_gradient(v0, problems, observed, K, workers=workers)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    best = min(times)
    _, interior = interior_updates(kw_model[0])
    interior //= T
    # finite differences of the misfit of shot 0 along a smooth direction
    rng = np.random.default_rng(0)
    from scipy.ndimage import gaussian_filter
    d = gaussian_filter(rng.standard_normal(v0.shape), 15.0)
    d = torch.tensor((50.0 * d / np.abs(d).max()).astype(np.float32), device="cuda")
    _, g0 = misfit_gradient(v0, problems[:1], observed[:1], K)

    def misfit(v):
        with torch.no_grad():
            rec = shot_record(v, problems[0], K)
            return 0.5 * float(torch.sum((rec.double() - observed[0].double()) ** 2))

    eps = 0.5
    fd = (misfit(v0 + eps * d) - misfit(v0 - eps * d)) / (2 * eps)
    ad = float(torch.sum(g0.double() * d.double()))
    return {"workload": "%d shots, (351+pad)x(1701+pad) grid (nz 351, nx 1701, 10 m), "
                        "so 8, 8 Hz Ricker, 1701 receivers, tf 3.0 s, T %d, "
                        "checkpoint interval %d" % (nshots, T, K),
            "grid": list(problems[0].shape), "timesteps": T, "interval": K,
            "workers": workers,
            "seconds": round(best, 4), "shots_per_s": round(nshots / best, 3),
            "gpts_per_s_3pass": round(3.0 * nshots * interior * T / best / 1e9, 2),
            "misfit": loss, "fd_directional": fd, "adjoint_directional": ad,
            "fd_rel_diff": abs(fd - ad) / abs(fd)}


def interior_updates(kw):
    shape = kw["velocity_model"].shape
    r = kw["space_order"] // 2
    pts = 1
    for n in shape:
        pts *= n - 2 * r
    T = kw["end_timestep"] - kw["begin_timestep"] + 1
    return pts, pts * T


# ---------------------------------------------------------------------------
# clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU oracle timing (bounded sample)

def cpu_model():
    """Host CPU model (lscpu, else /proc/cpuinfo) for the CPU-baseline line."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def cpu_sample(steps, threads=None, n=384):
    """Gpts/s of the C restatement on `steps` time steps of the workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    threads = threads or os.cpu_count()
    os.environ["OMP_NUM_THREADS"] = str(threads)
    kw = vd3d_arguments(timesteps=steps, stride=0, n=n)
    pts, updates = interior_updates(kw)
    _, _, secs = oracle.forward("port", x_stride="layout", **kw)
    return updates / secs / 1e9, secs, threads


# ---------------------------------------------------------------------------

def dist_setup(n_gpus, backend=None):
    """Rank, world size and local rank from the launcher's environment; one
    process per GPU (NCCL), or gloo where no GPU is visible. Ranks are
    independent replicas: the only collectives are the timing barrier and
    the max over ranks."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if backend is None:
            backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(value, world):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank, world, ms_per_step):
    """Whole-job rate (units / s, in 1e9) of `world` replicas that each
    process `units_per_rank` per step, timed by the slowest rank."""
    return units_per_rank * world / (ms_per_step / 1e3) / 1e9


def run_reference_arm(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    steps_t = args.cpu_steps
    for _ in range(args.warmup):
        cpu_sample(max(2, steps_t // 4))
    rates, total = [], 0.0
    threads = os.cpu_count()
    for _ in range(args.steps):
        rate, secs, threads = cpu_sample(steps_t)
        rates.append(rate)
        total += secs
    value = float(np.mean(rates))
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4),
        "unit": "Gpts/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1000 * total / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "3d_vd_so8_472cube_T1201_s50",
                   "sample": "%d of 1201 time steps per step" % steps_t,
                   "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": round(value, 4), "unit": "Gpts/s",
                         "cores": threads, "kind": "port", "cpu": cpu_model(),
                         "sample": "%d time steps of the 472^3 grid, OpenMP"
                                   % steps_t},
        "e2e": {"value": round(value, 4), "unit": "Gpts/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--timesteps", type=int, default=None,
                    help="truncate the shot (default: full T = 1201)")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-steps", type=int, default=12)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--n", type=int, default=384,
                    help="model points per axis (default 384)")
    ap.add_argument("--policy", type=int, default=0,
                    help="SIMWAVE_POLICY_* of the 3D stencil (default 0: AUTO)")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the 96-shot batched leg")
    ap.add_argument("--served", action="store_true",
                    help="run only the served (continuous batching) leg")
    ap.add_argument("--gradient", action="store_true",
                    help="run only the inversion (velocity gradient) leg")
    ap.add_argument("--accuracy", action="store_true",
                    help="run only the float32-vs-float64 error table (CPU-heavy)")
    ap.add_argument("--no-served", action="store_true",
                    help="skip the served leg of the default line")
    ap.add_argument("--no-gradient", action="store_true",
                    help="skip the inversion leg of the default line")
    args = ap.parse_args()

    if args.impl == "reference":
        run_reference_arm(args)
        return

    if args.accuracy:
        print(json.dumps({"metric": "float32 error vs the float64 run, per config",
                          "rows": accuracy_leg()}), flush=True)
        return

    if args.gradient:
        print(json.dumps({"metric": "FWI misfit gradient shots/s",
                          **gradient_leg(steps=args.steps)}), flush=True)
        return

    if args.served:
        import torch
        print(json.dumps({"metric": "served p50/p99 latency and shots/s",
                          **served_leg()}), flush=True)
        return

    world, rank, local = dist_setup(args.gpus)
    import torch
    from simwave_gb300.backend import _lib
    from simwave_gb300.backend.middleware import Middleware
    from simwave_gb300.device import DeviceProblem

    torch.cuda.set_device(local)
    if args.policy:
        import ctypes
        if _lib.load().simwave_set_kernel_policy(ctypes.c_int(args.policy)) != 0:
            raise SystemExit("unknown kernel policy %d" % args.policy)
    kw = vd3d_arguments(timesteps=args.timesteps, n=args.n)
    pts, updates = interior_updates(kw)
    dp = DeviceProblem(kw, device="cuda:%d" % local)
    stream = torch.cuda.current_stream()

    # warm-up runs
    for _ in range(args.warmup):
        dp.reset()
        dp.run(stream)
    torch.cuda.synchronize()

    # resident timing: CUDA events around each full forward on its stream
    clocks = ClockSampler(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    ms = []
    launches = 0
    for _ in range(args.steps):
        dp.reset()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = dp.run(stream)
        e1.record(stream)
        launches += st["kernel_launches"]
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    barrier(world)
    clock_info = clocks.stop()
    total_ms = max_over_ranks(float(np.sum(ms)), world)
    ms_per_step = total_ms / args.steps
    value = aggregate_rate(updates, world, ms_per_step)

    # stencil kernel time: events around each stencil launch, same stream
    dp.reset()
    st = dp.run(stream, time_kernels=True)
    stencil_ms = st["stencil_ms"] / max(st["stencil_launches"], 1)
    vd = "density_model" in kw and kw["density_model"] is not None
    bytes_per_launch = pts * BYTES_PER_UPDATE[vd]
    achieved = bytes_per_launch / (stencil_ms / 1e3) / 1e9
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        with open(peaks_path) as f:
            peak = float(json.load(f)["hbm_gbs"])
        peak_src = "measured"
    # DRAM bytes per launch of the kernel that ran, from its ncu capture
    # (profiles/stencil_traffic.json, keyed by SIMWAVE_POLICY_*)
    kernel_policy = int(st.get("stencil_kernel", 0))
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "stencil_traffic.json")
    if os.path.exists(tpath) and args.n == 384:
        with open(tpath) as f:
            t = json.load(f).get("by_policy", {}).get(str(kernel_policy))
        if t:
            traffic = t.get("bytes_per_launch_full_size")
    del dp
    torch.cuda.empty_cache()

    # end-to-end through the reference-facing C ABI with host buffers
    e2e_ms, h2d, d2h = [], 0, 0
    mw = Middleware()
    import contextlib
    import io
    for i in range(args.e2e_steps + 1 if args.e2e_steps > 0 else 0):
        k = dict(kw)
        k["u_full"] = np.zeros_like(kw["u_full"])
        k["shot_record"] = np.zeros_like(kw["shot_record"])
        barrier(world)
        t0 = time.perf_counter()
        with contextlib.redirect_stdout(io.StringIO()):
            mw.exec("forward", **k)
        t1 = time.perf_counter()
        if i > 0:  # first call allocates the library's device buffers
            e2e_ms.append(1000 * (t1 - t0))
            s = _lib.last_stats()
            h2d, d2h = s["h2d_bytes"], s["d2h_bytes"]
            launches_e2e = s["kernel_launches"]
    e2e = None
    if e2e_ms:
        # the median call (host-side page faults and page locking vary from
        # call to call); min and max beside it
        med = max_over_ranks(float(np.median(e2e_ms)), world)
        e2e_value = updates * world / (med / 1e3) / 1e9
        e2e = {"value": round(e2e_value, 3), "unit": "Gpts/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "ms_per_step": round(med, 3), "calls": len(e2e_ms),
               "ms_min": round(min(e2e_ms), 3), "ms_max": round(max(e2e_ms), 3),
               "statistic": "median call"}

    def leg(fn, **kw):
        """An extra leg's JSON; its failure is reported, not fatal to the line."""
        try:
            return fn(**kw)
        except Exception as exc:  # noqa: BLE001 - reported in the JSON line
            return {"error": "%s: %s" % (type(exc).__name__, exc)}

    batched = served = gradient = plain2d = None
    if rank == 0:
        plain2d = leg(plain2d_leg)
    if rank == 0 and not args.no_batched:
        batched = leg(batched_leg)
    if rank == 0 and not args.no_served:
        served = leg(served_leg)
    if rank == 0 and not args.no_gradient:
        gradient = leg(gradient_leg, steps=2)  # best of two

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        rate, secs, threads = cpu_sample(args.cpu_steps, n=args.n)
        cpu = {"value": round(rate, 4), "unit": "Gpts/s", "cores": threads,
               "kind": "port", "cpu": cpu_model(),
               "sample": "%d of 1201 time steps on the full 472^3 grid "
                         "(C restatement, OpenMP, %.1f s)" % (args.cpu_steps, secs)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "Gpts/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms_per_step, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "3d_vd_so8_%dcube_T%d_s50" % (
                           kw["velocity_model"].shape[0], kw["end_timestep"]),
                       "grid": list(kw["velocity_model"].shape),
                       "timesteps": kw["end_timestep"],
                       "updates_per_step": updates,
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs larger than L2 (11.4 GB wavefield slots)"},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1),
                         "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic,
                         "peak_source": peak_src,
                         "kernel_ms": round(stencil_ms, 4),
                         "kernel_policy": kernel_policy,
                         "bytes_per_launch": bytes_per_launch},
            "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clock_info,
            "cpu_baseline": cpu,
            "plain_2d": plain2d,
            "batched": batched,
            "served": served,
            "gradient": gradient,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
