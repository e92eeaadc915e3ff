"""Many 2D shots advanced together (``simwave_batch_*`` of the C library).

``BatchEngine`` keeps device-resident shots (``DeviceProblem``) and advances
all unfinished ones together: one stencil launch per (order, density) group
and one launch per sparse term per time step, captured as a CUDA graph of 16
steps and replayed. ``run_batch`` runs a list of problems to completion;
``autotune`` picks the stencil tile height per order by timing.
"""
import ctypes
import time

import torch

from .backend import _lib
from .device import DeviceProblem

TILE_ROWS = (8, 16, 32)


def _check(status):
    if status != 0:
        raise RuntimeError("simwave batch error {}: {}".format(status, _lib.last_error()))


class BatchEngine:
    """A set of 2D float32 shots advanced in lock step."""

    def __init__(self, device="cuda"):
        self.device = torch.device(device)
        self._lib = _lib.load()
        self._h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _check(self._lib.simwave_batch_create(ctypes.byref(self._h)))
        self._shots = {}

    def close(self):
        if self._h:
            _check(self._lib.simwave_batch_destroy(self._h))
            self._h = ctypes.c_void_p()
            self._shots.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, problem):
        """Admit a ``DeviceProblem``; returns its shot id."""
        if not isinstance(problem, DeviceProblem):
            raise TypeError("expected a DeviceProblem")
        sid = ctypes.c_int()
        _check(self._lib.simwave_batch_add(self._h, ctypes.byref(problem.problem),
                                           ctypes.byref(sid)))
        self._shots[sid.value] = problem
        return sid.value

    def run(self, steps, stream=None):
        """Advance every unfinished shot by up to ``steps`` time steps."""
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        _check(self._lib.simwave_batch_run(self._h, ctypes.c_int(int(steps)),
                                           ctypes.c_void_p(s.cuda_stream)))

    def remaining(self, shot_id):
        out = ctypes.c_int()
        _check(self._lib.simwave_batch_remaining(self._h, ctypes.c_int(shot_id),
                                                 ctypes.byref(out)))
        return out.value

    def release(self, shot_id):
        """Remove a shot (finished shots get their slots in reference order)."""
        _check(self._lib.simwave_batch_release(self._h, ctypes.c_int(shot_id)))
        return self._shots.pop(shot_id)

    def set_tile_rows(self, space_order, rows):
        _check(self._lib.simwave_batch_set_tile_rows(self._h, ctypes.c_int(space_order),
                                                     ctypes.c_int(rows)))

    def launches(self):
        out = ctypes.c_size_t()
        _check(self._lib.simwave_batch_launches(self._h, ctypes.byref(out)))
        return out.value

    @property
    def shot_ids(self):
        return list(self._shots)


def run_batch(problems, engine=None, chunk=256):
    """Run ``DeviceProblem``s to completion together; returns them (results
    in their ``u`` and ``receivers`` tensors) in input order."""
    own = engine is None
    engine = engine or BatchEngine(problems[0].device if problems else "cuda")
    ids = [engine.add(p) for p in problems]
    most = max((engine.remaining(i) for i in ids), default=0)
    done = 0
    while done < most:
        engine.run(min(chunk, most - done))
        done += chunk
    for i in ids:
        engine.release(i)
    if own:
        engine.close()
    return problems


def autotune(problems, steps=32, rows=TILE_ROWS):
    """Pick the stencil tile height per space order by timing ``steps`` steps
    of the given shots with every candidate; returns ``{order: rows}``."""
    orders = sorted({int(p.problem.space_order) for p in problems})
    best = {}
    for order in orders:
        group = [p for p in problems if int(p.problem.space_order) == order]
        timings = {}
        for r in rows:
            eng = BatchEngine(group[0].device)
            eng.set_tile_rows(order, r)
            for p in group:
                p.reset()
                eng.add(p)
            eng.run(16)  # warm-up (graph capture)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            eng.run(steps)
            torch.cuda.synchronize()
            timings[r] = time.perf_counter() - t0
            eng.close()
        best[order] = min(timings, key=timings.get)
    for p in problems:
        p.reset()
    return best
