"""Velocity gradient of the forward loop (``simwave_gradient_*`` of the C
library) behind ``torch.autograd``.

``shot_record(velocity, problem)`` runs the forward loop of a
``DeviceProblem`` on the given velocity grid and returns its shot record as a
differentiable tensor; ``backward`` runs the discrete adjoint with
checkpointed recomputation (a level pair every ``interval`` steps, ``interval``
= ceil(sqrt(steps)) by default, so memory grows with sqrt(T) instead of T).
2D float32 problems, constant or variable density (the density is held
fixed); the reference offers only the forward operator
(simwave/kernel/backend/compiler.py:128-130).

``misfit_gradient(velocity, problems, observed)`` is the full-waveform
inversion step: the L2 misfit 0.5 * sum((rec - obs)^2) over shots and its
velocity gradient.
"""
import ctypes
import math

import torch

from .backend import _lib
from .device import DeviceProblem


def _check(status, what):
    if status != 0:
        raise RuntimeError("{} failed ({}): {}".format(what, status, _lib.last_error()))


def default_interval(steps):
    return max(1, int(math.ceil(math.sqrt(steps))))


class _ShotRecord(torch.autograd.Function):
    @staticmethod
    def forward(ctx, velocity, problem, interval):
        if velocity.shape != tuple(problem.shape):
            raise ValueError("velocity shape {} != problem grid {}".format(
                tuple(velocity.shape), tuple(problem.shape)))
        lib = _lib.load()
        p = problem.problem
        problem.grid_view(problem.vel).copy_(velocity.detach())
        grids = ctypes.c_size_t()
        _check(lib.simwave_gradient_checkpoints(ctypes.byref(p), ctypes.c_size_t(interval),
                                                ctypes.byref(grids)), "checkpoint count")
        ck = torch.empty(grids.value * problem.slot, dtype=torch.float32,
                         device=problem.device)
        stream = torch.cuda.current_stream(problem.device)
        _check(lib.simwave_gradient_forward(ctypes.byref(p), ctypes.c_size_t(interval),
                                            ctypes.c_void_p(ck.data_ptr()),
                                            ctypes.c_void_p(stream.cuda_stream)),
               "simwave_gradient_forward")
        ctx.problem = problem
        ctx.interval = interval
        ctx.save_for_backward(ck)
        return problem.receivers[:, :problem.nrec].clone()

    @staticmethod
    def backward(ctx, grad_rec):
        (ck,) = ctx.saved_tensors
        problem = ctx.problem
        lib = _lib.load()
        g = grad_rec.detach().to(torch.float32).contiguous()
        out = torch.empty(problem.slot, dtype=torch.float32, device=problem.device)
        stream = torch.cuda.current_stream(problem.device)
        _check(lib.simwave_gradient_backward(
            ctypes.byref(problem.problem), ctypes.c_size_t(ctx.interval),
            ctypes.c_void_p(ck.data_ptr()), ctypes.c_void_p(g.data_ptr()),
            ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream)),
            "simwave_gradient_backward")
        return problem.grid_view(out).contiguous(), None, None


def shot_record(velocity, problem, interval=None):
    """Differentiable shot record ``(end_timestep, num_receivers)`` of
    ``problem`` (a ``DeviceProblem``) on ``velocity`` (the extended grid,
    float32, on the problem's device)."""
    if not isinstance(problem, DeviceProblem):
        raise TypeError("expected a DeviceProblem")
    if problem.dim != 2 or problem.dtype.itemsize != 4:
        raise ValueError("the gradient supports 2D float32 problems")
    steps = problem.timesteps
    return _ShotRecord.apply(velocity, problem, int(interval or default_interval(steps)))


def _lockstep_ok(problems):
    p0 = problems[0]
    q0 = p0.problem
    return len(problems) > 1 and all(
        p.dim == 2 and p.dtype.itemsize == 4 and tuple(p.shape) == tuple(p0.shape) and
        p.slot == p0.slot and p.vd == p0.vd and p.device == p0.device and
        int(p.problem.space_order) == int(q0.space_order) and
        int(p.problem.begin_timestep) == int(q0.begin_timestep) and
        int(p.problem.end_timestep) == int(q0.end_timestep) for p in problems)


def _misfit_gradient_lockstep(velocity, problems, observed, interval):
    """All shots in lockstep through ``simwave_gradient_*_shots``: one launch
    per forward, recomputed and adjoint step for every shot at once."""
    lib = _lib.load()
    p0 = problems[0]
    n = len(problems)
    device = velocity.device
    interval = int(interval or default_interval(p0.timesteps))
    stream = torch.cuda.current_stream(device)
    v = velocity.detach()
    for p in problems:
        p.grid_view(p.vel).copy_(v)
    grids = ctypes.c_size_t()
    _check(lib.simwave_gradient_checkpoints(ctypes.byref(p0.problem), ctypes.c_size_t(interval),
                                            ctypes.byref(grids)), "checkpoint count")
    cks = [torch.empty(grids.value * p.slot, dtype=torch.float32, device=device)
           for p in problems]
    arr = (type(p0.problem) * n)(*[p.problem for p in problems])
    ckp = (ctypes.c_void_p * n)(*[c.data_ptr() for c in cks])
    _check(lib.simwave_gradient_forward_shots(arr, ctypes.c_size_t(n), ctypes.c_size_t(interval),
                                              ckp, ctypes.c_void_p(stream.cuda_stream)),
           "simwave_gradient_forward_shots")
    total = 0.0
    res = []
    for p, obs in zip(problems, observed):
        obs = torch.as_tensor(obs, dtype=torch.float32, device=device)
        r = (p.receivers[:, :p.nrec] - obs).contiguous()
        total += float(0.5 * torch.sum(r ** 2))
        res.append(r)
    out = torch.empty(p0.slot, dtype=torch.float32, device=device)
    gp = (ctypes.c_void_p * n)(*[r.data_ptr() for r in res])
    _check(lib.simwave_gradient_backward_shots(
        arr, ctypes.c_size_t(n), ctypes.c_size_t(interval), ckp, gp,
        ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream)),
        "simwave_gradient_backward_shots")
    return total, p0.grid_view(out).contiguous()


def misfit_gradient(velocity, problems, observed, interval=None, workers=4, lockstep=True):
    """L2 misfit over shots and its velocity gradient.

    ``velocity``: the extended grid (float32 tensor on the device);
    ``problems``: one ``DeviceProblem`` per shot on that grid; ``observed``:
    one shot record per shot (tensor or array, same shape as the record).
    Shots of one layout, order and step range (``lockstep``) advance
    together, one launch per step for all of them. Otherwise shots are
    independent: up to ``workers`` of them run at once, each from its own
    host thread on its own CUDA stream (a shot's launches are short, so one
    host thread alone leaves the GPU idle between them). Returns
    ``(misfit, gradient)`` with the gradient on the extended grid.
    """
    if lockstep and _lockstep_ok(problems):
        return _misfit_gradient_lockstep(velocity, problems, observed, interval)
    import concurrent.futures
    v0 = velocity.detach()
    device = v0.device
    main = torch.cuda.current_stream(device)

    def one(args):
        prob, obs, stream = args
        stream.wait_stream(main)
        with torch.cuda.device(device), torch.cuda.stream(stream):
            v = v0.clone().requires_grad_(True)
            obs = torch.as_tensor(obs, dtype=torch.float32, device=device)
            rec = shot_record(v, prob, interval)
            loss = 0.5 * torch.sum((rec - obs) ** 2)
            (g,) = torch.autograd.grad(loss, v)
            done = torch.cuda.Event()
            done.record(stream)
        return float(loss.detach()), g, done

    n = max(1, min(int(workers), len(problems)))
    streams = [torch.cuda.Stream(device) for _ in range(n)]
    jobs = [(p, o, streams[i % n]) for i, (p, o) in enumerate(zip(problems, observed))]
    if n == 1:
        results = [one(j) for j in jobs]
    else:
        with concurrent.futures.ThreadPoolExecutor(max_workers=n) as pool:
            # shot i goes to stream i mod n; each worker thread takes whole
            # shots, so two shots never share a stream at the same time
            by_stream = [[j for j in jobs if j[2] is s] for s in streams]
            futs = [pool.submit(lambda js: [one(j) for j in js], js) for js in by_stream]
            results = [r for f in futs for r in f.result()]
    total = 0.0
    grad = torch.zeros_like(v0)
    for loss, g, done in results:
        main.wait_event(done)
        g.record_stream(main)  # made on a worker stream, read on this one
        grad += g
        total += loss
    return total, grad
