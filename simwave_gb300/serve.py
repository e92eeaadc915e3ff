"""Continuous-batching shot server.

Requests (the middleware keyword arguments of one shot plus an arrival time)
are admitted while their device footprint fits the HBM budget; results stay
resident on the device (wavefield slots), the shot record is copied to the
host when the shot completes.

* 2D float32 shots join a running ``BatchEngine``: every epoch advances all
  admitted 2D shots by ``epoch_steps`` time steps in one graph-captured
  sequence, and newly admitted shots join at the next epoch.
* Other shots (3D, or float64) run through the device entry on a
  low-priority stream, shortest first (interior updates), at most
  ``inflight`` queued at a time; each one fills the GPU on its own, so running
  them side by side would only delay all of them. The 2D epochs run on a
  high-priority stream and overlap them at block granularity.

Latency of a request = completion time - arrival time (queueing, upload,
compute and shot-record download included).
"""
import collections
import time

import numpy as np
import torch

from .batch import BatchEngine
from .device import DeviceProblem


def footprint_bytes(kwargs):
    """Device bytes one shot holds: wavefield slots, models, per-point
    coefficients, tables and shot record (pitched rows, float32/64)."""
    vel = kwargs["velocity_model"]
    itemsize = vel.dtype.itemsize
    shape = vel.shape
    row = shape[-1] + 64  # pitch padding bound
    grid = int(np.prod(shape[:-1])) * row * itemsize
    fields = 2 + (1 if kwargs.get("density_model") is not None else 0)  # vel, damp, den
    scratch = 2  # C and Q
    slots = int(kwargs["num_snapshots"])
    record = int(kwargs["end_timestep"]) * max(int(kwargs["num_receivers"]), 1) * itemsize
    return grid * (slots + fields + scratch) + record + (1 << 20)


class Request:
    """One shot to serve."""

    def __init__(self, kwargs, arrival, tag=None):
        self.kwargs = kwargs
        self.arrival = arrival
        self.tag = tag
        self.admitted = None
        self.completed = None
        self.problem = None
        self.shot_record = None
        self.evicted = False  # wavefield dropped to admit later requests
        self.bytes = footprint_bytes(kwargs)
        v = kwargs["velocity_model"]
        self.batchable = v.ndim == 2 and v.dtype == np.float32
        self.updates = int(np.prod(v.shape)) * int(kwargs["end_timestep"])

    @property
    def latency(self):
        return None if self.completed is None else self.completed - self.arrival


class ShotServer:
    """Serve requests with continuous batching on one GPU."""

    def __init__(self, hbm_budget=None, epoch_steps=64, inflight=2, device="cuda",
                 tile_rows=None):
        self.device = torch.device(device)
        free, _ = torch.cuda.mem_get_info(self.device)
        self.budget = int(hbm_budget if hbm_budget is not None else 0.85 * free)
        self.in_use = 0      # bytes of admitted shots (incl. resident results)
        self.resident = 0    # bytes of completed wavefields kept on the device
        self.epoch_steps = int(epoch_steps)
        self.engine = BatchEngine(device)
        for order, rows in (tile_rows or {}).items():
            self.engine.set_tile_rows(order, rows)
        lo, hi = torch.cuda.Stream.priority_range()
        self.epoch_stream = torch.cuda.Stream(self.device, priority=hi)
        self.shot_stream = torch.cuda.Stream(self.device, priority=lo)
        self.inflight = max(int(inflight), 1)
        self.pending = collections.deque()
        self.active2d = {}   # shot id -> request
        self.ready = []      # admitted stream-run shots not yet launched
        self.active = []     # (request, event) of launched stream-run shots
        self.done = []

    # -- admission ----------------------------------------------------------
    def submit(self, request):
        self.pending.append(request)

    def _admit(self, now):
        admitted = False
        while self.pending and self.pending[0].arrival <= now:
            req = self.pending[0]
            if req.bytes > self.budget:
                raise ValueError("request needs {} bytes, budget is {}".format(
                    req.bytes, self.budget))
            if self.in_use + req.bytes > self.budget:
                # completed wavefields are evicted (oldest first) before new
                # work waits for running shots to free memory
                self._evict(req.bytes)
                if self.in_use + req.bytes > self.budget:
                    break
            self.pending.popleft()
            req.admitted = time.perf_counter()
            req.problem = DeviceProblem(req.kwargs, device=self.device)
            self.in_use += req.bytes
            if req.batchable:
                sid = self.engine.add(req.problem)
                self.active2d[sid] = req
            else:
                self.ready.append(req)
            admitted = True
        # the uploads above were queued on the current stream
        if admitted:
            self.epoch_stream.wait_stream(torch.cuda.current_stream(self.device))
            self.shot_stream.wait_stream(torch.cuda.current_stream(self.device))
        self._launch()
        return admitted

    def _launch(self):
        """Queue the shortest admitted stream-run shots on the shot stream."""
        while self.ready and len(self.active) < self.inflight:
            req = min(self.ready, key=lambda r: r.updates)
            self.ready.remove(req)
            req.problem.run(self.shot_stream)
            ev = torch.cuda.Event()
            ev.record(self.shot_stream)
            self.active.append((req, ev))

    def _evict(self, need):
        for req in self.done:
            if self.in_use + need <= self.budget:
                return
            if req.problem is not None and req.problem._u is not None and not req.evicted:
                freed = req.problem._u.numel() * req.problem._u.element_size()
                req.problem._u = None
                req.problem.u = None
                req.evicted = True
                self.in_use -= freed
                self.resident -= freed

    # -- completion ---------------------------------------------------------
    def _complete(self, req):
        req.shot_record = req.problem.shot_record_numpy()
        req.completed = time.perf_counter()
        # the wavefield slots stay resident; models and tables are dropped
        resident = req.problem._u.numel() * req.problem._u.element_size()
        req.problem.release_inputs()
        self.in_use -= req.bytes - resident
        self.resident += resident
        self.done.append(req)

    def _retire(self):
        finished = [sid for sid in self.active2d if self.engine.remaining(sid) == 0]
        if finished:
            self.epoch_stream.synchronize()
            for sid in finished:
                self.engine.release(sid)
                self._complete(self.active2d.pop(sid))
        still = []
        for req, ev in self.active:
            if ev.query():
                req.problem.status()
                self._complete(req)
            else:
                still.append((req, ev))
        self.active = still
        self._launch()

    # -- loop ---------------------------------------------------------------
    def serve(self, requests, clock_start=None, timeout=600.0):
        """Run until every request is complete; arrival times are seconds
        relative to ``clock_start`` (default: now). Returns the requests.
        Raises TimeoutError if the requests are not done within ``timeout``
        seconds."""
        t0 = clock_start if clock_start is not None else time.perf_counter()
        for r in sorted(requests, key=lambda r: r.arrival):
            r.arrival = t0 + r.arrival
            self.submit(r)
        total = len(requests)
        while len(self.done) < total:
            now = time.perf_counter()
            if now - t0 > timeout:
                raise TimeoutError("{} of {} requests done after {} s".format(
                    len(self.done), total, timeout))
            self._admit(now)
            if self.active2d:
                self.engine.run(self.epoch_steps, stream=self.epoch_stream)
                # bound the queue ahead of the host: wait for this epoch
                self.epoch_stream.synchronize()
            elif self.active:
                time.sleep(0.0005)
            elif self.pending:
                wait = self.pending[0].arrival - time.perf_counter()
                if wait > 0:
                    time.sleep(min(wait, 0.01))
            self._retire()
        return requests

    def close(self):
        self.engine.close()


def latency_summary(requests):
    lat = np.array([r.latency for r in requests], dtype=np.float64)
    span = max(r.completed for r in requests) - min(r.arrival for r in requests)
    return {"p50_ms": round(float(np.percentile(lat, 50)) * 1e3, 2),
            "p99_ms": round(float(np.percentile(lat, 99)) * 1e3, 2),
            "mean_ms": round(float(lat.mean()) * 1e3, 2),
            "shots_per_s": round(len(requests) / span, 2),
            "shots": len(requests)}
