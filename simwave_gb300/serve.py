"""Continuous-batching shot server.

Requests (the middleware keyword arguments of one shot plus an arrival time)
are admitted while their device footprint fits the HBM budget; results stay
resident on the device (wavefield slots), the shot record is copied to the
host when the shot completes.

* 2D float32 shots join a running ``BatchEngine``: every epoch advances all
  admitted 2D shots by ``epoch_steps`` time steps in one graph-captured
  sequence, and newly admitted shots join at the next epoch.
* Other shots (3D, or float64) run through the device entry, each on a
  low-priority stream of its own, shortest first (interior updates): up to
  ``inflight_beside_2d`` of them while the 2D batch keeps stepping on its
  high-priority stream, up to ``inflight`` once no 2D shot is in the batch.
  Beside the batch they fill the SMs its short launches leave idle (between
  epochs the host waits for the batch); the block scheduler places the
  batch's blocks first as SMs free up, but a 3D kernel's blocks hold their
  SM's registers until they finish, so each 3D shot running beside the
  batch slows its steps (measured on the served workload: one 3D shot
  beside the batch took the 2D shots' p50 latency from about 0.5 s to
  2.5 s), so by default none runs beside the batch and the 3D shots overlap
  one another once it is empty. ``overlap=False`` keeps every stream-run
  shot out while 2D shots are batched, whatever the caps.

Latency of a request = completion time - arrival time (queueing, upload,
compute and shot-record download included).
"""
import collections
import concurrent.futures
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
        self.started = None  # launch time of a stream-run shot
        self.completed = None
        self.problem = None
        self.shot_record = None
        self.evicted = False  # wavefield dropped to admit later requests
        self.bytes = footprint_bytes(kwargs)
        v = kwargs["velocity_model"]
        self.batchable = v.ndim == 2 and v.dtype == np.float32
        self.updates = int(np.prod(v.shape)) * int(kwargs["end_timestep"])
        self.kind = "{}d".format(v.ndim)
        self._staged = None  # future of (DeviceProblem, upload event)
        self._uploaded = None  # event the device copies complete at

    @property
    def latency(self):
        return None if self.completed is None else self.completed - self.arrival


class ShotServer:
    """Serve requests with continuous batching on one GPU."""

    def __init__(self, hbm_budget=None, epoch_steps=64, inflight=3, device="cuda",
                 tile_rows=None, reserve_bytes=0, stage_workers=2, tuning=None, overlap=True,
                 inflight_beside_2d=0):
        self.device = torch.device(device)
        free, _ = torch.cuda.mem_get_info(self.device)
        self.budget = int(hbm_budget if hbm_budget is not None else 0.85 * free)
        self.in_use = 0      # bytes of admitted shots (incl. resident results)
        self.resident = 0    # bytes of completed wavefields kept on the device
        self.epoch_steps = int(epoch_steps)
        self.engine = BatchEngine(device)
        for order, rows in (tile_rows or {}).items():
            self.engine.set_tile_rows(order, rows)
        if tuning:  # {order: {"rows": r, "depth": k}} from batch.autotune
            self.engine.apply(tuning)
        lo, hi = torch.cuda.Stream.priority_range()
        self.epoch_stream = torch.cuda.Stream(self.device, priority=hi)
        self.inflight = max(int(inflight), 1)
        self.overlap = bool(overlap)
        self.inflight_2d = max(0, min(int(inflight_beside_2d), self.inflight))
        # one stream per stream-run shot in flight
        self.shot_streams = [torch.cuda.Stream(self.device, priority=lo)
                             for _ in range(self.inflight)]
        # uploads of stream-run shots happen on a worker thread and stream
        # so the serving loop keeps stepping the batch meanwhile
        self.stage_stream = torch.cuda.Stream(self.device)
        self._stager = concurrent.futures.ThreadPoolExecutor(max_workers=max(stage_workers, 1))
        if reserve_bytes:
            # keep device memory in the caching allocator (whose free blocks
            # belong to the stream they were allocated on) so that staging
            # carves problems out of it instead of calling cudaMalloc
            with torch.cuda.stream(self.stage_stream):
                torch.empty(int(reserve_bytes), dtype=torch.uint8, device=self.device)
        self.pending = collections.deque()
        self.staging = []    # admitted requests whose device copies are being made
        self.active2d = {}   # shot id -> request
        self.ready = []      # admitted stream-run shots not yet launched
        self.active = []     # (request, event, stream) of launched stream-run shots
        self.done = []

    # -- admission ----------------------------------------------------------
    def submit(self, request):
        self.pending.append(request)

    def prepare(self, requests):
        """Make the device copies of known requests ahead of serving them
        (their memory is counted at admission as usual); returns when done."""
        for req in requests:
            if req._staged is None and req.problem is None:
                req._staged = self._stager.submit(self._stage, req)
        for req in requests:
            if req._staged is not None:
                req._staged.result()

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
            self.in_use += req.bytes
            if req._staged is None:
                req._staged = self._stager.submit(self._stage, req)
            self.staging.append(req)
            admitted = True
        self._collect()
        self._launch()
        return admitted

    def _collect(self):
        """Move requests whose device copies are ready into the batch or the
        stream-run queue."""
        still = []
        for req in self.staging:
            if not req._staged.done():
                still.append(req)
                continue
            req.problem, uploaded = req._staged.result()
            req._staged = None
            if req.batchable:
                self.epoch_stream.wait_event(uploaded)
                sid = self.engine.add(req.problem, ready=uploaded)
                self.active2d[sid] = req
            else:
                req._uploaded = uploaded
                self.ready.append(req)
        self.staging = still

    def _stage(self, req):
        """Worker thread: the request's device copies, on the staging
        stream; returns the problem and the event its uploads complete at."""
        with torch.cuda.device(self.device), torch.cuda.stream(self.stage_stream):
            prob = DeviceProblem(req.kwargs, device=self.device)
            ev = torch.cuda.Event()
            ev.record(self.stage_stream)
        return prob, ev

    def _launch(self):
        """Queue the shortest admitted stream-run shots, each on a free shot
        stream, up to the cap for the batch's state (with ``overlap=False``,
        none while the 2D batch has shots or is about to get some)."""
        busy2d = bool(self.active2d) or any(r.batchable for r in self.staging)
        cap = (self.inflight_2d if self.overlap else 0) if busy2d else self.inflight
        while self.ready and len(self.active) < cap:
            req = min(self.ready, key=lambda r: r.updates)
            self.ready.remove(req)
            used = {id(s) for _, _, s in self.active}
            stream = next(s for s in self.shot_streams if id(s) not in used)
            stream.wait_event(req._uploaded)
            req._uploaded = None
            req.started = time.perf_counter()
            req.problem.run(stream)
            ev = torch.cuda.Event()
            ev.record(stream)
            self.active.append((req, ev, stream))

    def _evict(self, need):
        for req in self.done:
            if self.in_use + need <= self.budget:
                return
            if req.problem is not None and req.problem.wavefield_bytes and not req.evicted:
                freed = req.problem.release_wavefield()
                req.evicted = True
                self.in_use -= freed
                self.resident -= freed

    # -- completion ---------------------------------------------------------
    def _complete(self, req):
        req.shot_record = req.problem.shot_record_numpy()
        req.completed = time.perf_counter()
        # the wavefield slots stay resident; models and tables are dropped
        resident = req.problem.wavefield_bytes
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
        for req, ev, stream in self.active:
            if ev.query():
                req.problem.status(stream)
                self._complete(req)
            else:
                still.append((req, ev, stream))
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
            elif self.active or self.staging:
                time.sleep(0.0005)
            elif self.pending:
                wait = self.pending[0].arrival - time.perf_counter()
                if wait > 0:
                    time.sleep(min(wait, 0.01))
            self._retire()
        return requests

    def close(self):
        self._stager.shutdown(wait=True)
        self.engine.close()


def latency_summary(requests):
    lat = np.array([r.latency for r in requests], dtype=np.float64)
    span = max(r.completed for r in requests) - min(r.arrival for r in requests)
    t0 = min(r.arrival for r in requests)
    kinds = {}
    for kind in sorted({r.kind for r in requests}):
        sub = [r for r in requests if r.kind == kind]
        kl = np.array([r.latency for r in sub])
        kinds[kind] = {"shots": len(sub),
                       "p50_ms": round(float(np.percentile(kl, 50)) * 1e3, 2),
                       "max_ms": round(float(kl.max()) * 1e3, 2),
                       "last_done_s": round(max(r.completed for r in sub) - t0, 3)}
    return {"p50_ms": round(float(np.percentile(lat, 50)) * 1e3, 2),
            "p99_ms": round(float(np.percentile(lat, 99)) * 1e3, 2),
            "mean_ms": round(float(lat.mean()) * 1e3, 2),
            "shots_per_s": round(len(requests) / span, 2),
            "shots": len(requests), "by_kind": kinds}
