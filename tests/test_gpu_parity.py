"""GPU parity: the sm_103a library against the CPU oracle.

Tolerances (relative L2 over the whole output array):
  float32: 1e-4 (the contract stated for this path), float64: 1e-9.
All GPU calls go through the C ABI (host-pointer drop-ins via the
Middleware, or simwave_forward_device via DeviceProblem).
"""
import copy

import numpy as np
import pytest

import oracle
import simwave_gb300 as sw
from simwave_gb300.backend.middleware import Middleware
from _cases import (CASE_FIXTURES, FIXTURES, fixture_kwargs, random_problem,
                    rel_l2)

pytestmark = pytest.mark.gpu

TOL = {np.dtype(np.float32): 1e-4, np.dtype(np.float64): 1e-9}


def gpu_forward(kw):
    kw = dict(kw)
    kw["u_full"] = kw["u_full"].copy()
    kw["shot_record"] = kw["shot_record"].copy()
    return Middleware().exec("forward", **kw)


def port_forward(kw, x_stride="layout"):
    kw = dict(kw)
    kw["u_full"] = kw["u_full"].copy()
    kw["shot_record"] = kw["shot_record"].copy()
    u, rec, _ = oracle.forward("port", x_stride=x_stride, **kw)
    return u, rec


def assert_close(got, want, dtype, what):
    tol = TOL[np.dtype(dtype)]
    err = rel_l2(got, want)
    assert np.all(np.isfinite(got)), what + " not finite"
    assert err <= tol, "{}: rel L2 {:.3e} > {:.1e}".format(what, err, tol)


@pytest.mark.parametrize("name", FIXTURES)
def test_fixture_parity(name):
    """GPU vs the outputs of the reference's own C path."""
    kw, expected_u, expected_rec, meta = fixture_kwargs(name)
    dtype = kw["velocity_model"].dtype
    u, rec = gpu_forward(kw)
    if name == "3d_vd_so6_noncube_s0_f32":
        # nx != ny: the reference's x first-derivative stride differs from the
        # layout's; compare with the oracle on the layout stride instead
        expected_u, expected_rec = port_forward(kw, x_stride="layout")
    if isinstance(expected_u, tuple):
        slot, expected_u = expected_u
        u = u[slot:slot + 1]
    assert_close(rec, expected_rec, dtype, "shot record")
    assert_close(u, expected_u, dtype, "wavefield")
    for s in range(u.shape[0]):
        if np.any(expected_u[s]):
            assert_close(u[s], expected_u[s], dtype, "slot %d" % s)


BCS = ["none", "null_dirichlet", "null_neumann"]


def _bc(rng, dim):
    return tuple(BCS[i] for i in rng.integers(0, 3, size=2 * dim))


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("vd", [False, True])
@pytest.mark.parametrize("order", range(2, 22, 2))
def test_random_parity_all_orders(dim, vd, order):
    rng = np.random.default_rng(1000 * dim + 10 * order + vd)
    bc = _bc(rng, dim)
    stride = int(rng.integers(0, 5))
    n = 44 if dim == 2 else 26
    shape = (n, n + 3) if dim == 2 else (n, n, n + 2 if not vd else n)
    kw = random_problem(sw, dim, order, vd, bc, stride, n=n, shape=shape,
                        tf=0.03, seed=order, nsrc=2, nrec=6,
                        src_radius=int(rng.integers(1, 6)),
                        rec_radius=int(rng.integers(1, 6)))
    u, rec = gpu_forward(kw)
    ru, rrec = port_forward(kw)
    assert_close(u, ru, np.float32, "wavefield bc=%s s=%d" % (bc, stride))
    assert_close(rec, rrec, np.float32, "shot record")


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("vd", [False, True])
@pytest.mark.parametrize("stride", [0, 1, 2, 3, 4])
def test_float64_parity(dim, vd, stride):
    bc = ("null_neumann", "null_dirichlet", "null_dirichlet", "null_neumann",
          "none", "null_neumann")[:2 * dim]
    n = 40 if dim == 2 else 20
    kw = random_problem(sw, dim, 8, vd, bc, stride, dtype=np.float64, n=n,
                        tf=0.04, seed=stride, nsrc=3, nrec=5)
    u, rec = gpu_forward(kw)
    ru, rrec = port_forward(kw)
    assert_close(u, ru, np.float64, "wavefield")
    assert_close(rec, rrec, np.float64, "shot record")


def test_multiwavelet_and_overlapping_sources():
    kw = random_problem(sw, 2, 4, True, "null_neumann", 0, n=40, tf=0.05,
                        seed=4, nsrc=6, nrec=9, multi=True, src_radius=6)
    u, rec = gpu_forward(kw)
    ru, rrec = port_forward(kw)
    assert_close(u, ru, np.float32, "wavefield")
    assert_close(rec, rrec, np.float32, "shot record")


def test_reference_parallel_config_2d():
    """The reference's backend-equivalence configuration
    (tests/test_parallel_solution.py:9-107), 2D, float64, atol 1e-8."""
    shape = (128, 128)
    vel = np.full(shape, 1500.0)
    vel[shape[0] // 2:] = 2000.0
    den = np.full(shape, 5.0)
    sm = sw.SpaceModel((0, 1280, 0, 1280), (10., 10.), vel, den,
                       space_order=4, dtype=np.float64)
    sm.config_boundary(damping_length=128, boundary_condition=(
        "null_neumann", "null_dirichlet", "null_neumann", "null_dirichlet"),
        damping_polynomial_degree=3, damping_alpha=0.001)
    tm = sw.TimeModel(space_model=sm, tf=0.4, saving_stride=0)
    src = sw.Source(sm, coordinates=[(10, i) for i in range(128, 1280, 128)],
                    window_radius=8)
    rec = sw.Receiver(sm, coordinates=[(10, i) for i in range(0, 1280, 10)],
                      window_radius=8)
    solver = sw.Solver(sm, tm, src, rec, sw.RickerWavelet(15.0, tm))
    kw = solver.forward_arguments()
    u, r = gpu_forward(kw)
    ru, rr = port_forward(kw)
    assert np.allclose(u, ru, atol=1e-8)
    assert np.allclose(r, rr, atol=1e-8)


def test_device_entry_matches_host_entry():
    from simwave_gb300.device import DeviceProblem
    import torch
    for stride in (0, 2, 3):
        kw = random_problem(sw, 3, 8, True, "null_neumann", stride, n=24,
                            tf=0.04, seed=7, nrec=7)
        hu, hrec = gpu_forward(kw)
        dp = DeviceProblem(kw)
        dp.run()
        torch.cuda.synchronize()
        assert np.array_equal(dp.u_full_numpy(), hu)
        assert np.array_equal(dp.shot_record_numpy(), hrec)


def test_repeated_calls_are_deterministic():
    kw = random_problem(sw, 3, 4, False, "null_dirichlet", 0, n=30, tf=0.04,
                        seed=2, nsrc=1, nrec=4)
    a = gpu_forward(kw)
    b = gpu_forward(kw)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


POLICIES = {"auto": 0, "scalar_tiled": 1, "vec_2cta": 2, "vec_1cta": 3,
            "vec_smemq": 4, "vec_2cta_rot": 5, "vec_1cta_rot": 6, "vec_packed": 7,
            "vec_packed_1cta": 8, "tmem": 9, "stage_release": 10}


@pytest.mark.parametrize("policy", list(POLICIES))
@pytest.mark.parametrize("order", [2, 4, 6, 8, 10, 16, 20])
@pytest.mark.parametrize("vd", [False, True])
def test_tiled_and_generic_kernels_agree(order, vd, policy):
    """Each tiled 3D kernel variant against the one-thread-per-point kernel
    and the oracle, on shapes that leave partial tiles in x and y."""
    from simwave_gb300.backend import _lib
    from simwave_gb300.device import DeviceProblem
    bc = ("null_neumann", "null_dirichlet", "none", "null_neumann",
          "null_dirichlet", "none")
    kw = random_problem(sw, 3, order, vd, bc, 0, shape=(30, 37, 45) if not vd
                        else (30, 41, 41), tf=0.03, seed=order, nrec=5)
    dp = DeviceProblem(kw)
    lib = _lib.load()
    assert lib.simwave_set_kernel_policy(POLICIES[policy]) == 0
    try:
        st = dp.run()
        dp.status()
    finally:
        lib.simwave_set_kernel_policy(0)
    assert st["stencil_variant"] == 1, "tiled kernel not selected"
    tiled_u, tiled_rec = dp.u_full_numpy(), dp.shot_record_numpy()
    dp.reset()
    st = dp.run(generic=True)
    dp.status()
    assert st["stencil_variant"] == 0
    gen_u, gen_rec = dp.u_full_numpy(), dp.shot_record_numpy()
    ru, rrec = port_forward(kw)
    assert_close(tiled_u, ru, np.float32, "tiled wavefield")
    assert_close(gen_u, ru, np.float32, "generic wavefield")
    assert_close(tiled_rec, rrec, np.float32, "tiled shot record")
    assert rel_l2(tiled_u, gen_u) < 2e-5


@pytest.mark.parametrize("order", [4, 8])
@pytest.mark.parametrize("vd", [False, True])
def test_stage_release_many_columns(order, vd):
    """The stage-release kernel (AUTO for order 8 with variable density) on
    a grid with more columns of 128 x 12 interior points than there are SMs
    (160 or 243 columns, so several waves of CTAs, each a chunk of planes),
    against the oracle."""
    from simwave_gb300.backend import _lib
    from simwave_gb300.device import DeviceProblem
    bc = ("null_neumann", "null_dirichlet", "none", "null_neumann",
          "null_dirichlet", "none")
    kw = random_problem(sw, 3, order, vd, bc, 3, shape=(14 - order, 958 - order, 254 - order),
                        tf=0.03, seed=order, nrec=7, nsrc=2)
    nz, nx, ny = kw["velocity_model"].shape
    assert ((ny - order + 127) // 128) * ((nx - order + 11) // 12) >= 160
    dp = DeviceProblem(kw)
    lib = _lib.load()
    assert lib.simwave_set_kernel_policy(POLICIES["stage_release"]) == 0
    try:
        st = dp.run()
        dp.status()
    finally:
        lib.simwave_set_kernel_policy(0)
    assert st["stencil_kernel"] == POLICIES["stage_release"]
    ru, rrec = port_forward(kw)
    assert_close(dp.u_full_numpy(), ru, np.float32, "stage-release wavefield")
    assert_close(dp.shot_record_numpy(), rrec, np.float32, "stage-release shot record")


@pytest.mark.parametrize("order", [2, 4, 8, 14, 20])
@pytest.mark.parametrize("vd", [False, True])
def test_tiled2d_and_generic_kernels_agree(order, vd):
    """The tiled 2D kernel against the one-thread-per-point kernel and the
    oracle (partial tiles in both axes)."""
    from simwave_gb300.device import DeviceProblem
    bc = ("null_neumann", "null_dirichlet", "null_dirichlet", "null_neumann")
    kw = random_problem(sw, 2, order, vd, bc, 3, shape=(77, 301), tf=0.04,
                        seed=order, nrec=6)
    dp = DeviceProblem(kw)
    # separate stencil, source, boundary and receiver kernels per step
    st = dp.run(time_kernels=True)
    dp.status()
    assert st["stencil_variant"] == 1, "tiled 2D kernel not selected"
    tiled_u, tiled_rec = dp.u_full_numpy(), dp.shot_record_numpy()
    # one launch per step (owner-computes sources and edges where the edge
    # tiles are wide enough), then all steps in one persistent launch
    for flags, variants in (({"step_launches": True}, (1, 3)), ({}, (2,))):
        dp.reset()
        st = dp.run(**flags)
        dp.status()
        assert st["stencil_variant"] in variants, st["stencil_variant"]
        assert np.array_equal(dp.u_full_numpy(), tiled_u)
        assert np.array_equal(dp.shot_record_numpy(), tiled_rec)
    dp.reset()
    st = dp.run(generic=True)
    assert st["stencil_variant"] == 0
    gen_u = dp.u_full_numpy()
    ru, rrec = port_forward(kw)
    assert_close(tiled_u, ru, np.float32, "tiled 2D wavefield")
    assert rel_l2(tiled_u, gen_u) < 2e-5


@pytest.mark.parametrize("order,vd", [(2, False), (4, True), (8, False), (12, True)])
def test_fused_step_sources_across_tiles(order, vd):
    """One launch per step with many wide source windows that straddle tile
    borders and the damping layer, against the oracle."""
    from simwave_gb300.device import DeviceProblem
    bc = ("null_dirichlet", "null_neumann", "null_neumann", "null_dirichlet")
    kw = random_problem(sw, 2, order, vd, bc, 0, shape=(126, 290), tf=0.05, seed=order,
                        nsrc=9, nrec=7, src_radius=10, rec_radius=10, multi=True)
    dp = DeviceProblem(kw)
    st = dp.run(step_launches=True)
    dp.status()
    assert st["stencil_variant"] == 3, "fused step kernel not selected"
    ru, rrec = port_forward(kw)
    assert_close(dp.u_full_numpy(), ru, np.float32, "fused-step wavefield")
    assert_close(dp.shot_record_numpy(), rrec, np.float32, "fused-step shot record")


@pytest.mark.parametrize("policy", ["tmem", "stage_release"])
@pytest.mark.parametrize("mask", ["perturbed_faces", "uniform", "none"])
def test_tmem_kernel_damping_masks(policy, mask):
    """The tensor-memory kernel takes the damping mask from per-axis tables
    where one axis is outside the zero box, checked on the device against
    the mask: a mask whose faces differ from its centre lines (read at every
    point instead), a uniform mask (no zero box) and no damping layer (the
    box is the whole grid) all match the oracle; so does the stage-release
    kernel (damping from Q) on the same masks."""
    from simwave_gb300.backend import _lib
    from simwave_gb300.device import DeviceProblem
    bc = ("null_dirichlet", "null_neumann", "none", "null_dirichlet",
          "null_neumann", "none")
    kw = random_problem(sw, 3, 8, True, bc, 0, shape=(34, 45, 47), tf=0.04, seed=3,
                        nrec=5, damping=0.0 if mask == "none" else 80.0)
    damp = kw["damping_mask"].copy()
    rng = np.random.default_rng(7)
    if mask == "perturbed_faces":
        # points of the z, x and y faces (layer 4..11 and the far side), of
        # an edge and of a corner differ from the centre lines
        for idx in ((5, 30, 30), (50, 20, 25), (30, 6, 30), (30, 60, 40), (25, 30, 6),
                    (25, 30, 62), (6, 6, 30), (5, 5, 5)):
            damp[idx] *= np.float32(1.0 + 0.5 * rng.random())
    elif mask == "uniform":
        damp[:] = np.float32(0.3)
    kw["damping_mask"] = damp
    dp = DeviceProblem(kw)
    lib = _lib.load()
    assert lib.simwave_set_kernel_policy(POLICIES[policy]) == 0
    try:
        st = dp.run()
        dp.status()
    finally:
        lib.simwave_set_kernel_policy(0)
    assert st["stencil_kernel"] == POLICIES[policy]
    ru, rrec = port_forward(kw)
    assert_close(dp.u_full_numpy(), ru, np.float32, "wavefield")
    assert_close(dp.shot_record_numpy(), rrec, np.float32, "shot record")
