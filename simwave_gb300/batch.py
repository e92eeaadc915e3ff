"""Many 2D shots advanced together (``simwave_batch_*`` of the C library).

``BatchEngine`` keeps device-resident shots (``DeviceProblem``) and advances
all unfinished ones together: one stencil launch per (order, density, depth)
group and one launch per sparse term per time step, captured as a CUDA graph
of 16 launches per group and replayed. With a time-blocking depth k > 1 for
an order, each launch advances that order's constant-density shots k steps
(sources, boundaries and receiver records inside the kernel). ``run_batch``
runs a list of problems to completion; ``autotune`` picks the tile height and
the depth per order by timing.
"""
import ctypes
import time

import torch

from .backend import _lib
from .device import DeviceProblem

TILE_ROWS = (8, 16, 32, 64, 128, 256)
DEPTHS = (2, 3, 4)


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

    def add(self, problem, ready=None):
        """Admit a ``DeviceProblem``; returns its shot id. The engine reads
        the problem's arrays on its own stream at once, so this waits for
        ``ready`` (the event its uploads complete at) or, without one, for
        the current stream."""
        if not isinstance(problem, DeviceProblem):
            raise TypeError("expected a DeviceProblem")
        if ready is not None:
            ready.synchronize()
        else:
            torch.cuda.current_stream(problem.device).synchronize()
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

    def set_depth(self, space_order, depth):
        """Time-blocking depth (steps per launch) for one space order."""
        _check(self._lib.simwave_batch_set_depth(self._h, ctypes.c_int(space_order),
                                                 ctypes.c_int(depth)))

    def depth(self, shot_id):
        """Steps per launch the shot runs at under the current settings."""
        out = ctypes.c_int()
        _check(self._lib.simwave_batch_depth(self._h, ctypes.c_int(shot_id),
                                             ctypes.byref(out)))
        return out.value

    def apply(self, tuning):
        """Settings from ``autotune``: ``{order: {"rows": r, "depth": k}}``."""
        for order, t in tuning.items():
            self.set_tile_rows(int(order), int(t["rows"]))
            self.set_depth(int(order), int(t["depth"]))

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


def _candidates(order, rows, depths, device):
    """(rows, depth) settings the library accepts for ``order``."""
    out = [(r, 1) for r in rows]
    probe = BatchEngine(device)
    try:
        for k in depths:
            try:
                probe.set_depth(order, k)
            except RuntimeError:
                continue
            out.append((16, k))
    finally:
        probe.close()
    return out


def _time_engine(problems, tuning, steps):
    """Seconds for ``steps`` steps of all ``problems`` in one engine set to
    ``tuning`` (after ``steps`` untimed ones)."""
    eng = BatchEngine(problems[0].device)
    try:
        eng.apply(tuning)
        for p in problems:
            p.reset()
            eng.add(p)
        eng.run(steps)  # warm-up (graph capture, kernel load)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng.run(steps)
        torch.cuda.synchronize()
        return time.perf_counter() - t0
    finally:
        eng.close()


def autotune(problems, steps=64, rows=TILE_ROWS, depths=DEPTHS, margin=0.03):
    """Pick the tile height and the time-blocking depth per space order by
    timing; returns ``{order: {"rows": r, "depth": k}}`` (``BatchEngine.apply``
    takes it).

    Tile heights are timed on each order's shots alone (only that order's
    stencil launch changes). Depths are timed on all the shots together, one
    order at a time: the per-step source, boundary and receiver launches are
    shared by every order's per-step shots, so an order's shots timed alone
    would charge them all to that order. A depth is kept only when the whole
    set runs at least ``margin`` faster with it.
    """
    orders = sorted({int(p.problem.space_order) for p in problems})
    best = {}
    for order in orders:
        group = [p for p in problems if int(p.problem.space_order) == order]
        timings = {r: _time_engine(group, {order: {"rows": r, "depth": 1}}, steps)
                   for r in rows}
        best[order] = {"rows": min(timings, key=timings.get), "depth": 1}
    base = _time_engine(problems, best, steps)
    for order in orders:
        for _, k in [c for c in _candidates(order, rows, depths, problems[0].device)
                     if c[1] > 1]:
            trial = {o: dict(t) for o, t in best.items()}
            trial[order]["depth"] = k
            t = _time_engine(problems, trial, steps)
            if t < base * (1.0 - margin):
                best, base = trial, t
    for p in problems:
        p.reset()
    return best
