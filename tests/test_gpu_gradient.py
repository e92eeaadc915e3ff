"""The GPU velocity gradient (hand-written adjoint behind torch.autograd)
against the float64 adjoint-state gradient and against finite differences
of the GPU forward, with constant and variable density; checkpoint
intervals give the same gradient; the differentiable shot record is the
plain forward's."""
import numpy as np
import pytest

import adjoint_oracle
import simwave_gb300 as sw
from _cases import edge_problem, random_problem, rel_l2

pytestmark = pytest.mark.gpu

BC_MIXES = [
    ("none",) * 4,
    ("null_dirichlet",) * 4,
    ("null_neumann",) * 4,
    ("null_neumann", "null_dirichlet", "none", "null_neumann"),
    ("null_dirichlet", "null_neumann", "null_neumann", "null_dirichlet"),
]

# float32 forward and adjoint against the float64 adjoint-state gradient:
# relative L2 over the grid (measured 1.5e-6 .. 2.9e-6 on these cases)
GRAD_TOL = 1e-4


def _problem(kw):
    from simwave_gb300.device import DeviceProblem
    return DeviceProblem(kw)


def _gpu_gradient(kw, g, interval=None, vel=None):
    import torch
    from simwave_gb300.gradient import shot_record
    p = _problem(kw)
    v = torch.tensor(kw["velocity_model"] if vel is None else vel, device="cuda",
                     dtype=torch.float32, requires_grad=True)
    rec = shot_record(v, p, interval)
    rec.backward(torch.tensor(g, dtype=torch.float32, device="cuda"))
    return rec.detach().cpu().numpy(), v.grad.cpu().numpy()


def _as64(kw):
    out = dict(kw)
    for k, v in kw.items():
        if isinstance(v, np.ndarray) and v.dtype == np.float32:
            out[k] = v.astype(np.float64)
    out["dt"] = np.float64(kw["dt"])
    out["grid_spacing"] = tuple(np.float64(h) for h in kw["grid_spacing"])
    return out


@pytest.mark.parametrize("bc", BC_MIXES)
@pytest.mark.parametrize("order", [4, 8, 16])
@pytest.mark.parametrize("density", [False, True])
def test_gradient_matches_float64_adjoint(bc, order, density):
    kw = edge_problem(bc, order, shape=(40, 44), timesteps=200, dtype=np.float32,
                      damping=2e-5, density=density)
    rng = np.random.default_rng(11)
    g = rng.standard_normal((kw["end_timestep"], kw["num_receivers"])).astype(np.float32)
    _, grad = _gpu_gradient(kw, g)
    ref = adjoint_oracle.gradient(_as64(kw), g.astype(np.float64))
    assert rel_l2(grad, ref) <= GRAD_TOL


@pytest.mark.parametrize("density", [False, True])
def test_front_end_problem_gradient(density):
    """Damping layer, Ricker wavelet, radius-4 KWS windows, Neumann edges."""
    kw = random_problem(sw, 2, 8, density, "null_neumann", 0, shape=(60, 70), tf=0.25,
                        seed=4, nrec=12)
    rng = np.random.default_rng(5)
    g = rng.standard_normal((kw["end_timestep"], kw["num_receivers"])).astype(np.float32)
    _, grad = _gpu_gradient(kw, g)
    ref = adjoint_oracle.gradient(_as64(kw), g.astype(np.float64))
    assert rel_l2(grad, ref) <= GRAD_TOL


def test_record_equals_plain_forward():
    kw = random_problem(sw, 2, 8, False, "null_neumann", 0, shape=(60, 70), tf=0.2,
                        seed=2, nrec=9)
    p = _problem(kw)
    p.run()
    p.status()
    plain = p.shot_record_numpy()
    g = np.zeros((kw["end_timestep"], kw["num_receivers"]), dtype=np.float32)
    rec, _ = _gpu_gradient(kw, g)
    assert np.array_equal(rec, plain)


@pytest.mark.parametrize("bc", [BC_MIXES[3], BC_MIXES[4]])
@pytest.mark.parametrize("density", [False, True])
def test_checkpoint_interval_does_not_change_gradient(bc, density):
    kw = edge_problem(bc, 8, shape=(40, 44), timesteps=150, dtype=np.float32,
                      damping=2e-5, nsrc=1, density=density)
    rng = np.random.default_rng(1)
    g = rng.standard_normal((150, kw["num_receivers"])).astype(np.float32)
    grads = [_gpu_gradient(kw, g, interval)[1] for interval in (1, 7, 13, 150, 1000)]
    for other in grads[1:]:
        assert np.array_equal(grads[0], other)


@pytest.mark.parametrize("density", [False, True])
def test_gradient_matches_finite_differences(density):
    """Directional derivative of J = sum(g * rec) by central differences of
    the GPU forward (float32 records summed in float64)."""
    import torch
    from simwave_gb300.gradient import shot_record
    kw = edge_problem(BC_MIXES[3], 8, shape=(40, 44), timesteps=200, dtype=np.float32,
                      damping=2e-5, density=density)
    if density:
        # a smooth density (a point-random one makes the float32 difference
        # quotient too noisy for this bar; the float64 oracle, itself checked
        # by central differences, covers rough densities)
        z = np.linspace(0.0, 1.0, 40)[:, None]
        x = np.linspace(0.0, 1.0, 44)[None, :]
        kw["density_model"] = (1800.0 + 400.0 * np.sin(3.0 * z + 1.0) *
                               np.cos(2.0 * x)).astype(np.float32)
    rng = np.random.default_rng(3)
    g = rng.standard_normal((200, kw["num_receivers"]))
    _, grad = _gpu_gradient(kw, g.astype(np.float32))
    # perturbations of about 10 m/s: large enough that the difference of two
    # float32 records stands well above their rounding, small enough that
    # the central difference's O(eps^2) term stays below 1e-4
    dv = 20.0 * rng.standard_normal(kw["velocity_model"].shape)
    eps = 0.5
    p = _problem(kw)
    vel = kw["velocity_model"].astype(np.float64)

    def J(v):
        t = torch.tensor(v.astype(np.float32), device="cuda")
        with torch.no_grad():
            rec = shot_record(t, p).cpu().numpy().astype(np.float64)
        return float(np.sum(g * rec))

    fd = (J(vel + eps * dv) - J(vel - eps * dv)) / (2 * eps)
    ad = float(np.sum(grad.astype(np.float64) * dv))
    assert abs(fd - ad) <= 1e-2 * abs(fd)


def test_misfit_gradient_two_shots():
    import torch
    from simwave_gb300.gradient import misfit_gradient
    kws = [edge_problem(BC_MIXES[2], 8, shape=(40, 44), timesteps=160, dtype=np.float32,
                        damping=2e-5, seed=s) for s in (0, 1)]
    # one velocity for both shots; observed data from a perturbed model
    for k in kws[1:]:
        k["velocity_model"] = kws[0]["velocity_model"]
    vel = kws[0]["velocity_model"]
    true = vel * np.float32(1.02)
    observed = [adjoint_oracle.shot_record(_as64(k), vel=true.astype(np.float64)) for k in kws]
    probs = [_problem(k) for k in kws]
    loss, grad = misfit_gradient(torch.tensor(vel, device="cuda"), probs, observed)
    ref = np.zeros(vel.shape)
    ref_loss = 0.0
    for k, obs in zip(kws, observed):
        p64 = adjoint_oracle.Problem2D(_as64(k))
        levels, rec = p64.forward()
        res = rec - obs
        ref_loss += 0.5 * float(np.sum(res ** 2))
        ref += p64.gradient(res, levels)
    assert abs(loss - ref_loss) <= 1e-4 * ref_loss
    assert rel_l2(grad.cpu().numpy(), ref) <= GRAD_TOL


def test_gradient_refuses_halo_windows_and_3d():
    import torch
    from simwave_gb300.gradient import shot_record
    kw = edge_problem(BC_MIXES[0], 4, dtype=np.float32)
    iv = kw["rec_points_interval"].copy()
    iv[0] = 1  # first receiver window starts in the halo (r = 2)
    kw["rec_points_interval"] = iv
    p = _problem(kw)
    v = torch.tensor(kw["velocity_model"], device="cuda", requires_grad=True)
    with pytest.raises(RuntimeError, match="halo"):
        shot_record(v, p)
    kw3 = random_problem(sw, 3, 4, False, "none", 0, n=20, tf=0.02)
    p3 = _problem(kw3)
    with pytest.raises(ValueError, match="2D"):
        shot_record(torch.tensor(kw3["velocity_model"], device="cuda"), p3)


@pytest.mark.parametrize("order,shape,bc", [(8, (40, 44), BC_MIXES[3]),
                                            (4, (46, 150), BC_MIXES[4]),
                                            (20, (55, 60), BC_MIXES[1])])
def test_lockstep_shots_match_one_by_one(order, shape, bc):
    """Several shots of one grid in lockstep (one launch per step for all;
    the order-20 shape has no tiling offset that gives both edge tiles r + 1
    rows, so it runs one shot after another) give the misfit and the summed
    gradient of the shots run one by one."""
    import torch
    from simwave_gb300.gradient import misfit_gradient
    kws = [edge_problem(bc, order, shape=shape, timesteps=120, dtype=np.float32,
                        damping=2e-5, seed=s, nsrc=1 + s % 2) for s in range(3)]
    for k in kws[1:]:
        k["velocity_model"] = kws[0]["velocity_model"]
    vel = kws[0]["velocity_model"]
    observed = [adjoint_oracle.shot_record(_as64(k), vel=(vel * np.float32(1.01)).astype(np.float64))
                for k in kws]
    out = {}
    for lockstep in (True, False):
        probs = [_problem(k) for k in kws]
        out[lockstep] = misfit_gradient(torch.tensor(vel, device="cuda"), probs, observed,
                                        interval=7, lockstep=lockstep)
    # overlapping source windows are added with float32 atomics (their order
    # varies from run to run), and the residual against data of a model 1 %
    # away cancels most of the record's digits: last-bit differences of the
    # records show up near 1e-5 in the misfit
    assert abs(out[True][0] - out[False][0]) <= 1e-4 * abs(out[False][0])
    assert rel_l2(out[True][1].cpu().numpy(), out[False][1].cpu().numpy()) <= 1e-4
