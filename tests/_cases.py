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


def edge_problem(bc, order=4, shape=(22, 26), timesteps=160, seed=0,
                 dtype=np.float64, damping=0.0, nsrc=1, density=False):
    """Middleware kwargs of a small 2D problem whose waves reach every edge
    many times: no damping layer (or a uniform ``damping``), a source window
    near the centre and receiver windows on the first and second interior
    lines of every edge (the lines the boundary conditions act on). Window
    values are random; the wavelet is random per source. ``density``: a
    random density (1000-2500 kg/m^3) on the whole grid, halo included."""
    from simwave_gb300.frontend.fd import half_coefficients
    rng = np.random.default_rng(seed)
    nz, nx = shape
    r = order // 2
    vel = (1500.0 + 1000.0 * rng.random(shape)).astype(dtype)
    den = (1000.0 + 1500.0 * rng.random(shape)).astype(dtype) if density else None
    h, dt = 10.0, 1.0e-3

    def windows(boxes):
        iv, vals, off = [], [], [0]
        for z0, z1, x0, x1 in boxes:
            iv += [z0, z1, x0, x1]
            v = rng.uniform(0.2, 1.0, (z1 - z0 + 1) + (x1 - x0 + 1))
            vals += list(v)
            off.append(off[-1] + len(v))
        return (np.array(iv, dtype=np.uint64), np.array(vals, dtype=dtype),
                np.array(off, dtype=np.uint64))

    cz, cx = nz // 2, nx // 2
    src_boxes = [(cz - 1 + s, cz + 1 + s, cx - 1, cx + 1) for s in range(nsrc)]
    lo_z, hi_z, lo_x, hi_x = r, nz - r - 1, r, nx - r - 1
    rec_boxes = [(lo_z, lo_z + 1, cx - 2, cx + 1), (hi_z - 1, hi_z, cx, cx + 2),
                 (cz - 2, cz, lo_x, lo_x + 1), (cz, cz + 2, hi_x - 1, hi_x),
                 (lo_z, lo_z, lo_x, lo_x + 1), (hi_z, hi_z, hi_x, hi_x),
                 (cz + 3, cz + 4, cx + 3, cx + 4)]
    siv, sval, soff = windows(src_boxes)
    riv, rval, roff = windows(rec_boxes)
    w = rng.standard_normal((timesteps, nsrc)).astype(dtype)
    nslots = 3
    return dict(
        u_full=np.zeros((nslots,) + shape, dtype=dtype),
        velocity_model=vel, density_model=den,
        damping_mask=np.full(shape, damping, dtype=dtype),
        wavelet=w.reshape(-1) if nsrc > 1 else w[:, 0].copy(),
        wavelet_size=timesteps, wavelet_count=nsrc,
        second_order_fd_coefficients=np.asarray(half_coefficients(2, order), dtype=dtype),
        first_order_fd_coefficients=np.asarray(half_coefficients(1, order), dtype=dtype),
        boundary_condition=tuple(bc),
        src_points_interval=siv, src_points_interval_size=len(siv),
        src_points_values=sval, src_points_values_offset=soff,
        src_points_values_size=len(sval),
        rec_points_interval=riv, rec_points_interval_size=len(riv),
        rec_points_values=rval, rec_points_values_offset=roff,
        rec_points_values_size=len(rval),
        shot_record=np.zeros((timesteps, len(rec_boxes)), dtype=dtype),
        num_sources=nsrc, num_receivers=len(rec_boxes),
        grid_spacing=(dtype(h), dtype(h)), saving_stride=0, dt=dtype(dt),
        begin_timestep=1, end_timestep=timesteps, space_order=order,
        num_snapshots=nslots)
