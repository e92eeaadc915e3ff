"""The allocation-free entry point, simwave_forward_device_noalloc.

It is meant for callers that cannot let the library allocate device memory
while they run it (a framework owning the whole device budget through its own
pool, a serving loop where an allocation would synchronise the device, code
that enqueues work under stream capture). Its scratch lives in a fixed
32 MiB device array shared by all calls, so this file checks it against the
regular entry point on two consecutive calls (the second call must not see
stale status or coefficients from the first) and that an oversized grid is
refused with a clear message.

Collected last on purpose: if it fails, a run stopping at the first failure
has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import simwave_gb300 as sw
from _cases import random_problem, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-4  # relative L2, the float32 tolerance of the parity tests


def _entry_points():
    from simwave_gb300.backend import _lib
    lib = _lib.load()
    fn = lib.simwave_forward_device_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    return lib, fn


@pytest.mark.parametrize("vd, stride", [(True, 2), (False, 3)])
def test_noalloc_matches_regular_entry_twice(vd, stride):
    import torch
    from simwave_gb300.backend import _lib
    from simwave_gb300.device import DeviceProblem
    lib, noalloc = _entry_points()
    bc = ("null_neumann", "null_dirichlet", "none", "null_neumann",
          "null_dirichlet", "none")
    kw = random_problem(sw, 3, 8, vd, bc, stride, shape=(40, 44, 44),
                        tf=0.05, seed=21, nsrc=2, nrec=7)
    dp = DeviceProblem(kw)
    dp.run()
    dp.status()
    want_u, want_rec = dp.u_full_numpy(), dp.shot_record_numpy()
    assert np.abs(want_u).max() > 0
    stream = torch.cuda.current_stream()
    for call in range(2):
        dp.reset()
        status = noalloc(ctypes.addressof(dp.problem), ctypes.c_void_p(stream.cuda_stream))
        assert status == 0, _lib.last_error()
        torch.cuda.synchronize()
        got_u, got_rec = dp.u_full_numpy(), dp.shot_record_numpy()
        assert rel_l2(got_u, want_u) <= TOL, "call %d wavefield" % call
        assert rel_l2(got_rec, want_rec) <= TOL, "call %d shot record" % call


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
