"""The float64 adjoint-state gradient used as the oracle of the GPU
gradient: its forward is the C restatement's forward, and its gradient is
the derivative of that forward (central finite differences in float64),
for every boundary-condition mix, with waves that reach every edge."""
import numpy as np
import pytest

import adjoint_oracle
import oracle
from _cases import edge_problem, random_problem, rel_l2

BC_MIXES = [
    ("none",) * 4,
    ("null_dirichlet",) * 4,
    ("null_neumann",) * 4,
    ("null_neumann", "null_dirichlet", "none", "null_neumann"),
    ("null_dirichlet", "null_neumann", "null_neumann", "null_dirichlet"),
]


@pytest.mark.parametrize("bc", BC_MIXES)
@pytest.mark.parametrize("order", [2, 4, 8])
@pytest.mark.parametrize("density", [False, True])
def test_forward_matches_restatement(bc, order, density):
    kw = edge_problem(bc, order, nsrc=2, damping=2e-5, timesteps=120, density=density)
    p = adjoint_oracle.Problem2D(kw)
    levels, rec = p.forward()
    kk = dict(kw, u_full=kw["u_full"].copy(), shot_record=kw["shot_record"].copy())
    u, ref_rec, _ = oracle.forward("port", **kk)
    T = kw["end_timestep"]
    assert rel_l2(rec, ref_rec) < 1e-12
    assert rel_l2(levels[-1], u[(T + 1) % 3]) < 1e-12


def _functional(p, g, vel):
    return float(np.sum(g * p.with_velocity(vel).forward()[1]))


@pytest.mark.parametrize("bc", BC_MIXES)
@pytest.mark.parametrize("order", [4, 8])
@pytest.mark.parametrize("density", [False, True])
def test_gradient_matches_finite_differences(bc, order, density):
    kw = edge_problem(bc, order, nsrc=2, damping=2e-5, density=density)
    p = adjoint_oracle.Problem2D(kw)
    rng = np.random.default_rng(7)
    g = rng.standard_normal((kw["end_timestep"], kw["num_receivers"]))
    grad = p.gradient(g)
    dv = 20.0 * rng.standard_normal(p.vel.shape)
    eps = 1e-3
    fd = (_functional(p, g, p.vel + eps * dv) - _functional(p, g, p.vel - eps * dv)) / (2 * eps)
    assert abs(fd - np.sum(grad * dv)) <= 1e-6 * abs(fd)


@pytest.mark.parametrize("bc", [BC_MIXES[3], BC_MIXES[4]])
@pytest.mark.parametrize("density", [False, True])
def test_gradient_pointwise_at_edges(bc, density):
    """Single points on and next to the lines the boundary conditions act
    on, where the transposed boundary operations matter."""
    order = 4
    r = order // 2
    kw = edge_problem(bc, order, damping=2e-5, timesteps=120, density=density)
    p = adjoint_oracle.Problem2D(kw)
    rng = np.random.default_rng(3)
    g = rng.standard_normal((kw["end_timestep"], kw["num_receivers"]))
    grad = p.gradient(g)
    nz, nx = p.vel.shape
    points = [(r, nx // 2), (r + 1, nx // 2), (nz // 2, r), (nz // 2, r + 1),
              (nz - r - 1, nx // 2), (nz // 2, nx - r - 1), (r, r), (r + 1, r + 1),
              (nz // 2, nx // 2)]
    for (i, j) in points:
        dv = np.zeros_like(p.vel)
        dv[i, j] = 1.0
        eps = 1e-2
        fd = (_functional(p, g, p.vel + eps * dv) - _functional(p, g, p.vel - eps * dv)) / (2 * eps)
        assert abs(fd - grad[i, j]) <= 1e-6 * max(abs(fd), 1e-3 * np.abs(grad).max()), (i, j)


def test_gradient_zero_outside_interior():
    kw = edge_problem(BC_MIXES[2], 4, damping=2e-5, timesteps=60)
    p = adjoint_oracle.Problem2D(kw)
    g = np.ones((kw["end_timestep"], kw["num_receivers"]))
    grad = p.gradient(g)
    r = 2
    assert not grad[:r].any() and not grad[-r:].any()
    assert not grad[:, :r].any() and not grad[:, -r:].any()


@pytest.mark.parametrize("density", [False, True])
def test_front_end_problem_with_damping_layer(density):
    """A problem built by the front end (damping layer, Ricker wavelet, KWS
    windows of radius 4)."""
    import simwave_gb300 as sw
    kw = random_problem(sw, 2, 8, density, "null_neumann", 0, dtype=np.float64,
                        shape=(30, 34), tf=0.12, seed=5, nrec=6)
    p = adjoint_oracle.Problem2D(kw)
    rng = np.random.default_rng(2)
    g = rng.standard_normal((kw["end_timestep"], kw["num_receivers"]))
    grad = p.gradient(g)
    dv = 10.0 * rng.standard_normal(p.vel.shape)
    eps = 1e-3
    fd = (_functional(p, g, p.vel + eps * dv) - _functional(p, g, p.vel - eps * dv)) / (2 * eps)
    assert abs(fd - np.sum(grad * dv)) <= 1e-6 * abs(fd)
