"""Shared problem builders for the tests."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

FIXTURES = sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))
CASE_FIXTURES = [f for f in FIXTURES if not f.startswith("solution_")]


def load_fixture(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(z["meta"]))
    arrays = {k: z[k] for k in z.files if k != "meta"}
    return meta, arrays


def num_slots(timesteps, stride):
    return 3 if stride == 0 else len(range(0, timesteps, stride)) + 2


def fixture_kwargs(name):
    """Middleware keyword arguments rebuilt from a fixture's stored inputs,
    with zeroed outputs; plus the fixture's expected outputs."""
    meta, a = load_fixture(name)
    dtype = np.dtype(meta["dtype"]).type
    T = meta["timesteps"]
    stride = meta["saving_stride"]
    nslots = num_slots(T, stride)
    shape = tuple(meta["extended_shape"])
    kw = dict(
        u_full=np.zeros((nslots,) + shape, dtype=dtype),
        velocity_model=a["velocity_model"],
        density_model=a.get("density_model"),
        damping_mask=a["damping_mask"],
        wavelet=a["wavelet"],
        wavelet_size=a["wavelet"].shape[0],
        wavelet_count=meta["wavelet_count"],
        second_order_fd_coefficients=a["second_order_fd_coefficients"],
        first_order_fd_coefficients=a["first_order_fd_coefficients"],
        boundary_condition=tuple(meta["boundary_condition"]),
        src_points_interval=a["src_points_interval"],
        src_points_interval_size=len(a["src_points_interval"]),
        src_points_values=a["src_points_values"],
        src_points_values_offset=a["src_points_values_offset"],
        src_points_values_size=len(a["src_points_values"]),
        rec_points_interval=a["rec_points_interval"],
        rec_points_interval_size=len(a["rec_points_interval"]),
        rec_points_values=a["rec_points_values"],
        rec_points_values_offset=a["rec_points_values_offset"],
        rec_points_values_size=len(a["rec_points_values"]),
        shot_record=np.zeros((T, meta["num_receivers"]), dtype=dtype),
        num_sources=meta["num_sources"],
        num_receivers=meta["num_receivers"],
        grid_spacing=tuple(dtype(h) for h in meta["grid_spacing"]),
        saving_stride=stride,
        dt=dtype(meta["dt"]),
        begin_timestep=1,
        end_timestep=T,
        space_order=meta["space_order"],
        num_snapshots=nslots,
    )
    expected_u = a["u_full"]
    if "u_full_slot" in meta:  # only the returned slot was stored
        s = meta["u_full_slot"]
        expected_u = (s, expected_u)
    return kw, expected_u, a["shot_record"], meta


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def random_problem(sw, dim, order, vd, bc, stride, dtype=np.float32, n=32,
                   damping=50.0, nsrc=1, nrec=4, tf=0.05, seed=0,
                   src_radius=4, rec_radius=4, shape=None, multi=False):
    """A seeded problem built with ``sw``'s front end (this package's or any
    package with simwave's API). Returns the middleware kwargs."""
    rng = np.random.default_rng(seed)
    shape = tuple(shape) if shape is not None else (n,) * dim
    vel = (1500.0 + 2000.0 * rng.random(shape)).astype(dtype)
    den = (1000.0 + 1500.0 * rng.random(shape)).astype(dtype) if vd else None
    h = 10.0
    bbox = []
    for a in range(dim):
        bbox += [0.0, (shape[a] - 1) * h]
    sm = sw.SpaceModel(bounding_box=tuple(bbox), grid_spacing=(h,) * dim,
                       velocity_model=vel, density_model=den,
                       space_order=order, dtype=dtype)
    sm.config_boundary(damping_length=damping, boundary_condition=bc,
                       damping_polynomial_degree=3, damping_alpha=0.001)
    tm = sw.TimeModel(space_model=sm, tf=tf, saving_stride=stride)
    lo = np.zeros(dim)
    hi = np.array([bbox[2 * a + 1] for a in range(dim)])
    src = lo + (hi - lo) * (0.3 + 0.4 * rng.random((nsrc, dim)))
    rec = lo + (hi - lo) * (0.05 + 0.9 * rng.random((nrec, dim)))
    source = sw.Source(sm, coordinates=src.tolist(), window_radius=src_radius)
    receiver = sw.Receiver(sm, coordinates=rec.tolist(), window_radius=rec_radius)
    if multi:
        w = rng.standard_normal((tm.timesteps, nsrc)).astype(dtype)
        wavelet = sw.MultiWavelet(w, tm)
    else:
        wavelet = sw.RickerWavelet(12.0, tm)
    solver = sw.Solver(space_model=sm, time_model=tm, sources=source,
                       receivers=receiver, wavelet=wavelet)
    return solver.forward_arguments()
