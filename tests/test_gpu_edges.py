"""Edge cases of the forward operator against the CPU oracle: no receivers,
an all-zero wavelet, a run resumed across two calls, source and receiver
windows that reach into the halo, and the largest radius on the smallest
grid the operator accepts (one interior point per axis)."""
import contextlib
import io

import numpy as np
import pytest

import oracle
import simwave_gb300 as sw
from _cases import random_problem, rel_l2

pytestmark = pytest.mark.gpu

BCS = ("null_neumann", "null_dirichlet", "none", "null_dirichlet",
       "null_neumann", "null_neumann")


def _host(kw):
    from simwave_gb300.backend.middleware import Middleware
    k = dict(kw, u_full=kw["u_full"].copy(), shot_record=kw["shot_record"].copy())
    with contextlib.redirect_stdout(io.StringIO()):
        Middleware().exec("forward", **k)
    return k["u_full"], k["shot_record"]


def _port(kw):
    k = dict(kw, u_full=kw["u_full"].copy(), shot_record=kw["shot_record"].copy())
    u, r, _ = oracle.forward("port", x_stride="layout", **k)
    return u, r


def _without_receivers(kw):
    kw = dict(kw)
    kw.update(rec_points_interval=np.zeros(0, np.uint64), rec_points_interval_size=0,
              rec_points_values=np.zeros(0, kw["velocity_model"].dtype),
              rec_points_values_size=0, rec_points_values_offset=np.zeros(1, np.uint64),
              num_receivers=0,
              shot_record=np.zeros((kw["end_timestep"], 0), kw["velocity_model"].dtype))
    return kw


@pytest.mark.parametrize("dim", [2, 3])
def test_no_receivers(dim):
    kw = random_problem(sw, dim, 8, dim == 3, "null_neumann", 2, n=28 if dim == 3 else 60,
                        tf=0.05, seed=3)
    kw = _without_receivers(kw)
    u, rec = _host(kw)
    ru, _ = _port(kw)
    assert rec.shape[1] == 0
    assert rel_l2(u, ru) <= 1e-4


@pytest.mark.parametrize("dim", [2, 3])
def test_zero_wavelet_gives_zero_fields(dim):
    kw = random_problem(sw, dim, 4, False, BCS[:2 * dim], 0, n=24 if dim == 3 else 50,
                        tf=0.05, seed=4)
    kw["wavelet"] = np.zeros_like(kw["wavelet"])
    u, rec = _host(kw)
    assert not u.any() and not rec.any()


@pytest.mark.parametrize("dim,vd", [(2, False), (2, True), (3, True)])
def test_run_resumed_across_two_calls(dim, vd):
    """Steps 1..k in one call, k+1..T in a second from the first call's
    slots and record, give the single call's results (stride 0)."""
    kw = random_problem(sw, dim, 8, vd, BCS[:2 * dim], 0, n=26 if dim == 3 else 70,
                        tf=0.06, seed=5, nrec=5)
    T = kw["end_timestep"]
    k = T // 2
    whole_u, whole_rec = _host(kw)
    first_u, first_rec = _host(dict(kw, end_timestep=k))
    second = dict(kw, begin_timestep=k + 1, u_full=first_u, shot_record=first_rec)
    u, rec = _host(second)
    assert np.array_equal(u, whole_u)
    assert np.array_equal(rec, whole_rec)
    ru, rrec = _port(second)
    assert rel_l2(u, ru) <= 1e-4 and rel_l2(rec, rrec) <= 1e-4


def _tiny(dim, order, extent, dtype=np.float32, stride=0, seed=0):
    """Middleware kwargs on a grid of `extent` points per axis with KWS
    windows covering the whole grid (halo included)."""
    from simwave_gb300.frontend.fd import half_coefficients
    rng = np.random.default_rng(seed)
    shape = (extent,) * dim
    T = 40
    nslots = 3 if stride == 0 else len(range(0, T, stride)) + 2

    def window(count):
        iv, vals, off = [], [], [0]
        for _ in range(count):
            for _a in range(dim):
                iv += [0, extent - 1]
            v = rng.uniform(0.1, 1.0, dim * extent)
            vals += list(v)
            off.append(off[-1] + len(v))
        return (np.array(iv, np.uint64), np.array(vals, dtype), np.array(off, np.uint64))

    siv, sval, soff = window(1)
    riv, rval, roff = window(3)
    h = 10.0
    return dict(
        u_full=np.zeros((nslots,) + shape, dtype),
        velocity_model=(1500.0 + 500.0 * rng.random(shape)).astype(dtype),
        density_model=None, damping_mask=np.full(shape, 1e-5, dtype),
        wavelet=rng.standard_normal(T).astype(dtype), wavelet_size=T, wavelet_count=1,
        second_order_fd_coefficients=np.asarray(half_coefficients(2, order), dtype),
        first_order_fd_coefficients=np.asarray(half_coefficients(1, order), dtype),
        boundary_condition=BCS[:2 * dim],
        src_points_interval=siv, src_points_interval_size=len(siv),
        src_points_values=sval, src_points_values_offset=soff,
        src_points_values_size=len(sval),
        rec_points_interval=riv, rec_points_interval_size=len(riv),
        rec_points_values=rval, rec_points_values_offset=roff,
        rec_points_values_size=len(rval),
        shot_record=np.zeros((T, 3), dtype), num_sources=1, num_receivers=3,
        grid_spacing=(dtype(h),) * dim, saving_stride=stride, dt=dtype(5e-4),
        begin_timestep=1, end_timestep=T, space_order=order, num_snapshots=nslots)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("order,extent", [(20, 21), (20, 24), (2, 3), (8, 12)])
def test_smallest_grids_and_halo_windows(dim, order, extent):
    """One (or a few) interior points per axis, every boundary kind, and
    source/receiver windows spanning the whole grid including the halo."""
    kw = _tiny(dim, order, extent, stride=3)
    u, rec = _host(kw)
    ru, rrec = _port(kw)
    assert rel_l2(u, ru) <= 1e-4
    assert rel_l2(rec, rrec) <= 1e-4


@pytest.mark.parametrize("dim, stride", [(2, 3), (3, 2), (3, 0)])
def test_nonzero_initial_slots(dim, stride):
    """Every wavefield slot starts with nonzero values, halo included: the
    host entry uploads a slot the steps write before they read only when its
    halo is not zero (else it clears the slot on the device), so both paths
    must keep the reference's result, which carries the initial halo values
    through the run."""
    shape = (40, 56) if dim == 2 else (30, 34, 34)
    kw = random_problem(sw, dim, 8, True, BCS[:2 * dim], stride, shape=shape, tf=0.05,
                        seed=7, nrec=4)
    rng = np.random.default_rng(11)
    u0 = rng.standard_normal(kw["u_full"].shape).astype(kw["u_full"].dtype)
    r = kw["space_order"] // 2
    # the last slot keeps a zero halo (cleared on the device), the others not
    last = u0[-1]
    inner = tuple(slice(r, n - r) for n in last.shape)
    keep = last[inner].copy()
    last[...] = 0
    last[inner] = keep
    kw = dict(kw, u_full=u0)
    u, rec = _host(kw)
    ru, rrec = _port(kw)
    assert rel_l2(u, ru) <= 1e-4 and rel_l2(rec, rrec) <= 1e-4
