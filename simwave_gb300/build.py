"""Build step of the GPU library (run by ``__graft_entry__.build()``).

Compiles every ``csrc/*.cu`` for sm_103a with nvcc (one object per file, in
parallel), links ``_lib/libsimwave_gb300.so`` with the static CUDA runtime
(the library loads on machines without a GPU driver; the driver is opened at
the first CUDA call), and builds the eight ``libsimwave_forward_<variant>.so``
shims that export the reference's ``forward`` symbol.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
BUILDDIR = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIBNAME = "libsimwave_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-Wall", "--expt-relaxed-constexpr"]

VARIANTS = [(d, vd, f64) for d in (2, 3) for vd in (0, 1) for f64 in (0, 1)]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed: {}\n{}{}".format(
            " ".join(cmd), res.stdout, res.stderr))
    return res


def shim_name(dim, vd, f64):
    return "libsimwave_forward_{}d_{}_{}.so".format(
        dim, "vd" if vd else "cd", "f64" if f64 else "f32")


def build(verbose=False):
    """Compile and link; returns the path of libsimwave_gb300.so."""
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BUILDDIR, exist_ok=True)
    sources = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
               if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(INCLUDE, "simwave_gb300.h"))
    newest_header = max(os.path.getmtime(h) for h in headers)

    def compile_one(src):
        obj = os.path.join(BUILDDIR, src[:-3] + ".o")
        spath = os.path.join(CSRC, src)
        if (os.path.exists(obj) and os.path.getmtime(obj) >
                max(os.path.getmtime(spath), newest_header)):
            return obj
        cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-I" + INCLUDE, "-I" + CSRC,
                                               "-c", spath, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        _run(cmd)
        return obj

    workers = min(len(sources), os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(workers) as pool:
        objects = list(pool.map(compile_one, sources))
    lib = os.path.join(LIBDIR, LIBNAME)
    _run([nvcc()] + ARCH + ["-shared", "-o", lib] + objects +
         ["-Xlinker", "-rpath,$ORIGIN"])
    shim_src = os.path.join(CSRC, "sw_forward_shim.c")
    cc = shutil.which("gcc") or "cc"
    for dim, vd, f64 in VARIANTS:
        out = os.path.join(LIBDIR, shim_name(dim, vd, f64))
        _run([cc, "-O2", "-fPIC", "-shared", "-std=c99", "-I" + INCLUDE,
              "-DSW_DIM={}".format(dim), "-DSW_VD={}".format(vd),
              "-DSW_F64={}".format(f64), shim_src, "-o", out,
              "-L" + LIBDIR, "-lsimwave_gb300", "-Wl,-rpath,$ORIGIN"])
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
