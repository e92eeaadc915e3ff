"""The allocation-free entry point, simwave_forward_device_noalloc.

It is meant for callers that cannot let the library allocate device memory
while they run it: a framework owning the whole device budget through its own
pool, or a serving loop where an allocation would synchronise the device. Its
scratch lives in a fixed 32 MiB device array shared by all calls, so this
file checks, on two consecutive calls (the second must not see stale status
or coefficients from the first):

* its wavefield and shot record against the CPU oracle and against the
  regular entry point, within the float32 tolerance of the parity tests;
* that the device's stream-ordered memory pool, which the regular entry
  allocates its scratch from, does not grow during the calls;
* that an oversized grid and a stream under graph capture are refused with a
  clear message, before any work is enqueued.

Collected last on purpose: if it fails, a run stopping at the first failure
has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import oracle
import simwave_gb300 as sw
from _cases import random_problem, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-4  # relative L2, the float32 tolerance of the parity tests

# CUmemPool_attribute values (cuda.h): used bytes now / high watermark
_USED_MEM_CURRENT, _USED_MEM_HIGH = 7, 8


def _entry_points():
    from simwave_gb300.backend import _lib
    lib = _lib.load()
    fn = lib.simwave_forward_device_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    return lib, fn


class _DefaultPool:
    """The current device's default memory pool, read through the driver
    API (the pool is a driver object, shared by every runtime in the
    process)."""

    def __init__(self):
        import torch
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.pool = ctypes.c_void_p()
        rc = self.cu.cuDeviceGetDefaultMemPool(ctypes.byref(self.pool),
                                               ctypes.c_int(torch.cuda.current_device()))
        assert rc == 0, "cuDeviceGetDefaultMemPool: %d" % rc

    def get(self, attr):
        v = ctypes.c_uint64()
        rc = self.cu.cuMemPoolGetAttribute(self.pool, ctypes.c_int(attr), ctypes.byref(v))
        assert rc == 0, "cuMemPoolGetAttribute: %d" % rc
        return v.value

    def reset_high(self):
        zero = ctypes.c_uint64(0)
        rc = self.cu.cuMemPoolSetAttribute(self.pool, ctypes.c_int(_USED_MEM_HIGH),
                                           ctypes.byref(zero))
        assert rc == 0, "cuMemPoolSetAttribute: %d" % rc


def _oracle(kw):
    k = dict(kw, u_full=np.zeros_like(kw["u_full"]),
             shot_record=np.zeros_like(kw["shot_record"]))
    u, rec, _ = oracle.forward("port", x_stride="layout", **k)
    return u, rec


@pytest.mark.parametrize("vd, stride", [(True, 2), (False, 3)])
def test_noalloc_matches_oracle_and_regular_entry_twice(vd, stride):
    import torch
    from simwave_gb300.backend import _lib
    from simwave_gb300.device import DeviceProblem
    lib, noalloc = _entry_points()
    bc = ("null_neumann", "null_dirichlet", "none", "null_neumann",
          "null_dirichlet", "none")
    kw = random_problem(sw, 3, 8, vd, bc, stride, shape=(40, 44, 44),
                        tf=0.05, seed=21, nsrc=2, nrec=7)
    ref_u, ref_rec = _oracle(kw)
    assert np.abs(ref_u).max() > 0
    dp = DeviceProblem(kw)
    dp.run()
    dp.status()
    want_u, want_rec = dp.u_full_numpy(), dp.shot_record_numpy()
    assert rel_l2(want_u, ref_u) <= TOL and rel_l2(want_rec, ref_rec) <= TOL
    stream = torch.cuda.current_stream()
    pool = _DefaultPool()
    torch.cuda.synchronize()
    pool.reset_high()
    used = pool.get(_USED_MEM_CURRENT)
    for call in range(2):
        dp.reset()
        status = noalloc(ctypes.addressof(dp.problem), ctypes.c_void_p(stream.cuda_stream))
        assert status == 0, _lib.last_error()
        torch.cuda.synchronize()
        got_u, got_rec = dp.u_full_numpy(), dp.shot_record_numpy()
        assert rel_l2(got_u, ref_u) <= TOL, "call %d wavefield vs oracle" % call
        assert rel_l2(got_rec, ref_rec) <= TOL, "call %d shot record vs oracle" % call
        assert rel_l2(got_u, want_u) <= TOL, "call %d wavefield vs regular entry" % call
        assert rel_l2(got_rec, want_rec) <= TOL, "call %d shot record vs regular entry" % call
    assert pool.get(_USED_MEM_HIGH) <= used, "the default memory pool grew"


def test_noalloc_refuses_grid_beyond_scratch():
    import torch
    from simwave_gb300.backend import _lib
    from simwave_gb300.device import DeviceProblem
    lib, noalloc = _entry_points()
    # 172^3 extended points exceed the 32 MiB scratch (8 bytes per point)
    kw = random_problem(sw, 3, 4, False, "none", 0, shape=(168, 168, 168),
                        tf=0.002, seed=3, nsrc=1, nrec=1)
    dp = DeviceProblem(kw)
    status = noalloc(ctypes.addressof(dp.problem),
                     ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert status == 1  # SIMWAVE_E_ARGUMENT
    assert "exceeds the allocation-free scratch" in _lib.last_error()


def test_noalloc_refuses_capturing_stream():
    """The entry reads results back and waits for its stream mid-call, which
    graph capture forbids: it must refuse before enqueuing anything."""
    import torch
    from simwave_gb300.backend import _lib
    from simwave_gb300.device import DeviceProblem
    lib, noalloc = _entry_points()
    kw = random_problem(sw, 3, 4, False, "none", 0, shape=(24, 24, 24),
                        tf=0.01, seed=5, nsrc=1, nrec=1)
    dp = DeviceProblem(kw)
    side = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.stream(side):
        graph.capture_begin()
        status = noalloc(ctypes.addressof(dp.problem), ctypes.c_void_p(side.cuda_stream))
        # one captured operation so the graph is not empty
        dp.receivers.add_(0.0)
        graph.capture_end()
    assert status == 1  # SIMWAVE_E_ARGUMENT
    assert "captured" in _lib.last_error()
