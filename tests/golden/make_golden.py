"""Generate the golden fixtures in this directory from the reference itself.

Run here, where the reference tree exists (it does not exist on the GPU
machine, so the fixtures are committed):

    python tests/golden/make_golden.py [REFERENCE_ROOT]

For every case in ``CASES`` the reference's own front end (SpaceModel,
TimeModel, Source/Receiver KWS, RickerWavelet/MultiWavelet) builds the
problem and the reference's own sequential C path (``Compiler(language='c')``,
compiled by the reference's Compiler with gcc) runs it. The fixture stores the
front-end arrays (the exact kernel inputs) and the outputs ``u_full`` /
``shot_record`` as the C function returns them (before the halo and time-slot
stripping), in a compressed ``.npz``.

The reference imports three packages this image lacks; the script provides
them for the duration of the run only:
  * ``findiff.coefficients(deriv, acc)`` -- the centred finite-difference
    weights, computed by this package's own restatement
    (simwave_gb300.frontend.fd, Fornberg's algorithm in exact arithmetic);
  * empty ``segyio`` and ``matplotlib`` / ``mpl_toolkits`` modules (only the
    SEG-Y reader and the plotting helpers use them).

The 2D golden wavefields the reference ships
(tests/reference_solution/wavefield-2d-so-{2,8}.npy) are re-generated the
same way (``solution_2d_so{2,8}``) and compared with the shipped files; the
comparison is recorded in ``manifest.json``.
"""
import json
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))

# name: (dim, order, variable density, boundary conditions, stride, dtype,
#        n per axis, damping length (m), src radius, rec radius, n src,
#        n rec, tf, multiwavelet, non-cube)
CASES = {
    "2d_cd_so4_mixed_s0_f32": (2, 4, False, ("null_neumann", "null_dirichlet", "none", "null_dirichlet"), 0, "float32", 48, 100.0, 2, 3, 1, 8, 0.12, False, False),
    "2d_vd_so8_neumann_s3_f32": (2, 8, True, "null_neumann", 3, "float32", 40, 60.0, 4, 4, 2, 5, 0.10, False, False),
    "2d_cd_so20_dirichlet_s2_f64": (2, 20, False, "null_dirichlet", 2, "float64", 44, 50.0, 3, 1, 1, 4, 0.08, False, False),
    "2d_vd_so2_multi_s0_f32": (2, 2, True, ("none", "null_neumann", "null_dirichlet", "none"), 0, "float32", 36, 0.0, 1, 2, 3, 6, 0.10, True, False),
    "2d_cd_so12_s1_f32": (2, 12, False, ("null_dirichlet", "null_neumann", "null_neumann", "null_dirichlet"), 1, "float32", 40, 30.0, 5, 6, 1, 3, 0.05, False, False),
    "3d_cd_so4_mixed_s0_f32": (3, 4, False, ("null_neumann", "null_dirichlet", "none", "null_dirichlet", "null_neumann", "null_dirichlet"), 0, "float32", 22, 40.0, 2, 3, 1, 4, 0.06, False, False),
    "3d_vd_so8_cube_s4_f32": (3, 8, True, "null_neumann", 4, "float32", 18, 30.0, 3, 2, 1, 3, 0.05, False, False),
    "3d_vd_so6_noncube_s0_f32": (3, 6, True, ("null_dirichlet", "none", "null_neumann", "none", "null_dirichlet", "null_neumann"), 0, "float32", 20, 20.0, 2, 2, 1, 3, 0.05, False, True),
    "3d_cd_so10_s6_f64": (3, 10, False, ("none", "null_dirichlet", "null_neumann", "null_neumann", "none", "null_dirichlet"), 6, "float64", 18, 20.0, 4, 3, 2, 2, 0.04, False, False),
    "3d_vd_so16_s0_f32": (3, 16, True, "none", 0, "float32", 24, 0.0, 1, 5, 1, 2, 0.04, False, False),
}


def install_shims():
    """Temporary stand-ins for findiff, segyio and matplotlib."""
    sys.path.insert(0, REPO)
    from simwave_gb300.frontend import fd as own_fd

    findiff = types.ModuleType("findiff")

    def coefficients(deriv, acc):
        weights = own_fd.coefficients(deriv, acc)
        half = len(weights) // 2
        return {"center": {"coefficients": weights,
                           "offsets": np.arange(-half, half + 1)}}

    findiff.coefficients = coefficients
    sys.modules["findiff"] = findiff
    sys.modules["segyio"] = types.ModuleType("segyio")
    mpl = types.ModuleType("matplotlib")
    mpl.pyplot = types.ModuleType("matplotlib.pyplot")
    mpl.cm = types.ModuleType("matplotlib.cm")
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = mpl.pyplot
    sys.modules["matplotlib.cm"] = mpl.cm
    tk = types.ModuleType("mpl_toolkits")
    tk.axes_grid1 = types.ModuleType("mpl_toolkits.axes_grid1")
    tk.axes_grid1.make_axes_locatable = None
    sys.modules["mpl_toolkits"] = tk
    sys.modules["mpl_toolkits.axes_grid1"] = tk.axes_grid1


def model_arrays(dim, n, vd, dtype, seed, noncube):
    rng = np.random.default_rng(seed)
    shape = (n, n + 5, n - 3) if (dim == 3 and noncube) else (n,) * dim
    vel = (1500.0 + 2000.0 * rng.random(shape)).astype(dtype)
    den = (1000.0 + 1500.0 * rng.random(shape)).astype(dtype) if vd else None
    return shape, vel, den


def build_case(sw, name, spec, seed):
    (dim, order, vd, bc, stride, dtype, n, damping, srad, rrad, nsrc, nrec,
     tf, multi, noncube) = spec
    dtype = np.dtype(dtype).type
    shape, vel, den = model_arrays(dim, n, vd, dtype, seed, noncube)
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
    rng = np.random.default_rng(seed + 1)
    lo = np.array([bbox[2 * a] for a in range(dim)])
    hi = np.array([bbox[2 * a + 1] for a in range(dim)])
    src = lo + (hi - lo) * (0.3 + 0.4 * rng.random((nsrc, dim)))
    rec = lo + (hi - lo) * (0.1 + 0.8 * rng.random((nrec, dim)))
    source = sw.Source(sm, coordinates=src.tolist(), window_radius=srad)
    receiver = sw.Receiver(sm, coordinates=rec.tolist(), window_radius=rrad)
    if multi:
        T = tm.timesteps
        freqs = 8.0 + 4.0 * np.arange(nsrc)
        t = tm.time_values.astype(np.float64)
        w = np.stack([(1 - 2 * (np.pi * f * (t - 1 / f)) ** 2)
                      * np.exp(-(np.pi * f * (t - 1 / f)) ** 2)
                      for f in freqs], axis=1)
        wavelet = sw.MultiWavelet(w.astype(dtype), tm)
        assert wavelet.values.shape == (T, nsrc)
    else:
        wavelet = sw.RickerWavelet(15.0, tm)
    return sm, tm, source, receiver, wavelet


def run_reference(sw, sm, tm, source, receiver, wavelet):
    """Reference front-end arrays plus the C function's raw outputs."""
    solver = sw.Solver(space_model=sm, time_model=tm, sources=source,
                       receivers=receiver, wavelet=wavelet,
                       compiler=sw.Compiler(language="c"))
    sp, sv, so = source.interpolated_points_and_values
    rp, rv, ro = receiver.interpolated_points_and_values
    captured = {}
    mw = solver._middleware
    original = mw._exec_forward

    def capture(**kw):
        u, rec = original(**kw)
        captured["u_full"] = np.array(u, copy=True)
        captured["shot_record"] = np.array(rec, copy=True)
        return u, rec

    mw._exec_forward = capture
    solver.forward()
    arrays = dict(
        velocity_model=sm.extended_velocity_model,
        damping_mask=sm.damping_mask,
        wavelet=wavelet.values,
        second_order_fd_coefficients=sm.fd_coefficients(2),
        first_order_fd_coefficients=sm.fd_coefficients(1),
        src_points_interval=sp, src_points_values=sv,
        src_points_values_offset=so, rec_points_interval=rp,
        rec_points_values=rv, rec_points_values_offset=ro,
        u_full=captured["u_full"], shot_record=captured["shot_record"],
    )
    if sm.density_model is not None:
        arrays["density_model"] = sm.extended_density_model
    meta = dict(
        grid_spacing=[float(v) for v in sm.grid_spacing],
        boundary_condition=list(sm.boundary_condition),
        dt=float(tm.dt), timesteps=int(tm.timesteps),
        saving_stride=int(tm.saving_stride),
        space_order=int(sm.space_order), num_sources=int(source.count),
        num_receivers=int(receiver.count),
        wavelet_count=int(wavelet.num_sources),
        dtype=str(np.dtype(sm.dtype)), extended_shape=list(sm.extended_shape),
        nbl=list(sm.nbl),
    )
    return arrays, meta


def solution_case(sw, order):
    """The reference's tests/test_solution.py 2D configuration."""
    vel = np.zeros((500, 500), dtype=np.float32)
    vel[:] = 1500.0
    vel[250:] = 2000.0
    sm = sw.SpaceModel(bounding_box=(0, 5000, 0, 5000), grid_spacing=(10, 10),
                       velocity_model=vel, space_order=order,
                       dtype=np.float32)
    sm.config_boundary(damping_length=100, boundary_condition=(
        "null_neumann", "null_dirichlet", "none", "null_dirichlet"),
        damping_polynomial_degree=3, damping_alpha=0.001)
    tm = sw.TimeModel(space_model=sm, tf=1.0, saving_stride=0)
    src = sw.Source(sm, coordinates=[(2500, 2500)], window_radius=1)
    rec = sw.Receiver(sm, coordinates=[(2500, 2500)], window_radius=1)
    return sm, tm, src, rec, sw.RickerWavelet(10.0, tm)


def main():
    ref_root = (sys.argv[1] if len(sys.argv) > 1 else
                os.environ.get("SIMWAVE_REFERENCE_ROOT") or
                os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(HERE))),
                             "reference"))
    if not os.path.isdir(os.path.join(ref_root, "simwave")):
        sys.exit("reference checkout not found: pass its path (or set "
                 "SIMWAVE_REFERENCE_ROOT)")
    install_shims()
    sys.path.insert(0, ref_root)
    import simwave as sw  # the reference package
    manifest = {"reference_root": os.path.basename(os.path.abspath(ref_root)),
                "cases": {}}
    workdir = tempfile.mkdtemp(prefix="simwave_golden_")
    cwd = os.getcwd()
    os.chdir(workdir)  # the reference Compiler writes ./tmp/<sha1>.so
    try:
        for i, (name, spec) in enumerate(CASES.items()):
            parts = build_case(sw, name, spec, seed=100 + 7 * i)
            arrays, meta = run_reference(sw, *parts)
            np.savez_compressed(os.path.join(HERE, name + ".npz"),
                                meta=json.dumps(meta), **arrays)
            manifest["cases"][name] = meta
            print(name, "T", meta["timesteps"], "u max",
                  float(np.abs(arrays["u_full"]).max()), flush=True)
        for order in (2, 8):
            name = "solution_2d_so{}".format(order)
            arrays, meta = run_reference(sw, *solution_case(sw, order))
            shipped = np.load(os.path.join(
                ref_root, "tests", "reference_solution",
                "wavefield-2d-so-{}.npy".format(order)))
            tm_last = meta["timesteps"] % 3
            halo = order // 2
            mine = arrays["u_full"][tm_last:tm_last + 1, halo:-halo, halo:-halo]
            diff = float(np.abs(mine - shipped).max())
            meta["shipped_golden_max_abs_diff"] = diff
            meta["shipped_golden_rel_l2"] = float(
                np.linalg.norm(mine - shipped) / np.linalg.norm(shipped))
            # keep only the returned slot to stay small
            arrays["u_full"] = np.ascontiguousarray(
                arrays["u_full"][tm_last:tm_last + 1])
            meta["u_full_slot"] = tm_last
            np.savez_compressed(os.path.join(HERE, name + ".npz"),
                                meta=json.dumps(meta), **arrays)
            manifest["cases"][name] = meta
            print(name, "vs shipped golden: max abs", diff, "rel L2",
                  meta["shipped_golden_rel_l2"], flush=True)
    finally:
        os.chdir(cwd)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
