"""CPU baselines of the forward path (TEST INFRASTRUCTURE: run where the
reference checkout exists; the figures it prints are quoted in the docs).

    python oracle/cpu_baselines.py [REFERENCE_ROOT] [--steps N]

Three timings on the same synthetic inputs, all OpenMP on every host core:

1. the oracle port (oracle/_build/liboracle.so) against the reference's own
   cpu_openmp build of the same kernels (oracle/_ref/ref_*_omp.so, compiled
   with the reference Compiler's default flags by `make -C oracle ref`), on
   the 3D benchmark grid (472^3 extended, order 8, variable density, N time
   steps) and on the README 2D case: the C functions' own seconds, so the
   port's speed can be compared with the reference's;
2. the reference's own `Solver.forward()` end to end (its front end,
   Compiler with language='cpu_openmp', ctypes call, halo stripping) on the
   README 2D case at full length and on the 3D benchmark model cut to
   tf = 0.05 s, with the C function's seconds beside the wall time.

The reference imports packages this image lacks (findiff, segyio,
matplotlib); the stand-ins of tests/golden/make_golden.py are installed for
the run only.
"""
import argparse
import contextlib
import io
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(REPO, "tests", "golden"))


def cpu_model():
    """The host CPU's model name and core count (lscpu, else /proc/cpuinfo)."""
    name = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                name = line.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    if name is None:
        try:
            for line in open("/proc/cpuinfo"):
                if line.lower().startswith("model name"):
                    name = line.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    return "%s x %d" % (name or "unknown CPU", os.cpu_count() or 1)


def kernel_seconds(backend, kw):
    import oracle
    k = dict(kw, u_full=np.zeros_like(kw["u_full"]),
             shot_record=np.zeros_like(kw["shot_record"]))
    extra = {"x_stride": "reference"} if backend == "port" else {"language": "omp"}
    with contextlib.redirect_stdout(io.StringIO()):
        _, _, secs = oracle.forward(backend, **extra, **k)
    return secs


def port_vs_reference_build(steps):
    import bench
    out = {}
    for name, kw in (("3d_vd_so8_472cube_T%d" % steps, bench.vd3d_arguments(timesteps=steps,
                                                                            stride=0)),
                     ("2d_cd_so4_513sq_T328", bench.readme2d_arguments(np.float32))):
        _, updates = bench.interior_updates(kw)
        kernel_seconds("port", kw)  # warm-up (page faults, thread pool)
        row = {}
        for backend in ("port", "ref"):
            secs = min(kernel_seconds(backend, kw) for _ in range(3))
            row[backend] = {"seconds": round(secs, 4), "gpts": round(updates / secs / 1e9, 4)}
        row["port_over_ref_speed"] = round(row["ref"]["seconds"] / row["port"]["seconds"], 3)
        out[name] = row
    return out


def reference_solver_forward(ref_root):
    """Wall time of the reference's Solver.forward() (cpu_openmp) and the C
    function's own seconds, on the README 2D case and the 3D benchmark model
    cut to tf = 0.05 s."""
    import make_golden
    make_golden.install_shims()
    sys.path.insert(0, ref_root)
    import simwave as ref
    import bench
    work = tempfile.mkdtemp(prefix="simwave_cpu_")
    cwd = os.getcwd()
    os.chdir(work)  # the reference Compiler writes ./tmp/<hash>.so
    out = {}
    try:
        compiler = ref.Compiler(cc="gcc", language="cpu_openmp")
        # README 2D case (README.md:60-120 of the reference)
        vel = np.zeros((512, 512), dtype=np.float32)
        vel[:] = 1500.0
        vel[100:] = 2000.0
        t0 = time.perf_counter()
        sm = ref.SpaceModel(bounding_box=(0, 5120, 0, 5120), grid_spacing=(10, 10),
                            velocity_model=vel, space_order=4, dtype=np.float32)
        sm.config_boundary(damping_length=0, boundary_condition=(
            "null_neumann", "null_dirichlet", "none", "null_dirichlet"),
            damping_polynomial_degree=3, damping_alpha=0.001)
        tm = ref.TimeModel(space_model=sm, tf=1.0, saving_stride=0)
        src = ref.Source(sm, coordinates=[(2560, 2560)], window_radius=1)
        rec = ref.Receiver(sm, coordinates=[(2560, i) for i in range(0, 5112, 10)],
                           window_radius=1)
        solver = ref.Solver(space_model=sm, time_model=tm, sources=src, receivers=rec,
                            wavelet=ref.RickerWavelet(10.0, tm), compiler=compiler)
        solver.forward()  # compiles the kernel
        buf = io.StringIO()
        t0 = time.perf_counter()
        with contextlib.redirect_stdout(buf):
            solver.forward()
        wall = time.perf_counter() - t0
        kern = float(buf.getvalue().split()[-2])
        updates = 513 * 513 * tm.timesteps
        out["2d_cd_so4_513sq_T%d" % tm.timesteps] = {
            "solver_forward_s": round(wall, 4), "kernel_s": round(kern, 4),
            "solver_forward_gpts": round(updates / wall / 1e9, 4)}
        # 3D benchmark model (384^3 at 12.5 m, Gardner density, order 8,
        # 40-point damping layer), tf cut to 0.05 s
        v3, d3 = bench.vd3d_model(384)
        h = 12.5
        top = 383 * h
        t0 = time.perf_counter()
        sm = ref.SpaceModel(bounding_box=(0, top, 0, top, 0, top), grid_spacing=(h, h, h),
                            velocity_model=v3, density_model=d3, space_order=8,
                            dtype=np.float32)
        sm.config_boundary(damping_length=40 * h, boundary_condition="none",
                           damping_polynomial_degree=3, damping_alpha=0.001)
        tm = ref.TimeModel(space_model=sm, tf=0.05, saving_stride=0)
        centre = top / 2
        src = ref.Source(sm, coordinates=[(0.0, centre, centre)], window_radius=4)
        g = (np.arange(128) + 0.5) * (top / 128)
        gx, gy = np.meshgrid(g, g, indexing="ij")
        carpet = np.stack([np.full(gx.size, 10.0), gx.ravel(), gy.ravel()], axis=1)
        rec = ref.Receiver(sm, coordinates=carpet, window_radius=4)
        solver = ref.Solver(space_model=sm, time_model=tm, sources=src, receivers=rec,
                            wavelet=ref.RickerWavelet(15.0, tm), compiler=compiler)
        buf = io.StringIO()
        with contextlib.redirect_stdout(buf):
            solver.forward()
        wall = time.perf_counter() - t0
        kern = float(buf.getvalue().split()[-2])
        updates = 464 ** 3 * tm.timesteps
        out["3d_vd_so8_472cube_T%d" % tm.timesteps] = {
            "solver_forward_s_with_setup": round(wall, 2), "kernel_s": round(kern, 3),
            "kernel_gpts": round(updates / kern / 1e9, 4),
            "setup_and_marshalling_s": round(wall - kern, 2)}
    finally:
        os.chdir(cwd)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("reference_root", nargs="?",
                    default=os.environ.get("SIMWAVE_REFERENCE_ROOT") or
                    os.path.join(os.path.dirname(REPO), "reference"))
    ap.add_argument("--steps", type=int, default=6)
    args = ap.parse_args()
    import oracle
    if not oracle.ref_available():
        sys.exit("oracle/_ref is not built: make -C oracle ref REFERENCE_ROOT=...")
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
    res = {"cpu": cpu_model(), "omp_threads": int(os.environ["OMP_NUM_THREADS"]),
           "port_vs_reference_build": port_vs_reference_build(args.steps),
           "reference_solver_forward": reference_solver_forward(args.reference_root)}
    print(json.dumps(res, indent=1))


if __name__ == "__main__":
    main()
