"""The batch engine against the CPU oracle and the single-shot entry: mixed
orders, densities, grid sizes, boundary sets and saving strides advanced
together give each shot's own result."""
import numpy as np
import pytest

import oracle
import simwave_gb300 as sw
from _cases import random_problem, rel_l2

pytestmark = pytest.mark.gpu


def _shots(seed=0, count=7):
    rng = np.random.default_rng(seed)
    bcs = ["none", "null_dirichlet", "null_neumann"]
    kws = []
    for i in range(count):
        order = int(rng.choice([2, 4, 8, 12, 16, 20]))
        vd = bool(rng.integers(0, 2))
        nz, nx = (int(v) for v in rng.integers(36, 150, size=2))
        bc = tuple(bcs[j] for j in rng.integers(0, 3, size=4))
        stride = int(rng.integers(0, 4))
        kws.append(random_problem(sw, 2, order, vd, bc, stride, shape=(nz, nx),
                                  tf=float(rng.uniform(0.03, 0.08)), seed=seed + i,
                                  nsrc=int(rng.integers(1, 3)),
                                  nrec=int(rng.integers(3, 12))))
    return kws


def test_batch_matches_oracle():
    from simwave_gb300.batch import run_batch
    from simwave_gb300.device import DeviceProblem
    kws = _shots(seed=3)
    probs = run_batch([DeviceProblem(k) for k in kws], chunk=40)
    for k, p in zip(kws, probs):
        kk = dict(k, u_full=k["u_full"].copy(), shot_record=k["shot_record"].copy())
        ru, rrec, _ = oracle.forward("port", **kk)
        assert rel_l2(p.u_full_numpy(), ru) <= 1e-4
        assert rel_l2(p.shot_record_numpy(), rrec) <= 1e-4


@pytest.mark.parametrize("rows", [8, 16, 32, 64, 128, 256])
def test_batch_tile_heights_agree(rows):
    from simwave_gb300.batch import BatchEngine, run_batch
    from simwave_gb300.device import DeviceProblem
    kws = _shots(seed=11, count=5)
    eng = BatchEngine()
    for order in (2, 4, 8, 12, 16, 20):
        eng.set_tile_rows(order, rows)
    probs = run_batch([DeviceProblem(k) for k in kws], engine=eng)
    single = []
    for k in kws:
        d = DeviceProblem(k)
        d.run()
        d.status()
        single.append(d)
    for p, s in zip(probs, single):
        assert rel_l2(p.u_full_numpy(), s.u_full_numpy()) <= 1e-5
        assert rel_l2(p.shot_record_numpy(), s.shot_record_numpy()) <= 1e-5
    eng.close()


@pytest.mark.parametrize("rows", [64, 128, 256])
def test_streamed_tiles_bitwise_equal_staged_tiles(rows):
    """Tall tiles streamed through a ring of rows give the 16-row staged
    tiles' results bit for bit (the same per-point arithmetic), on shots of
    every order with and without density, taller and wider than one tile."""
    from simwave_gb300.batch import BatchEngine, run_batch
    from simwave_gb300.device import DeviceProblem
    rng = np.random.default_rng(21)
    kws = []
    for i, order in enumerate((2, 4, 8, 12, 16, 20)):
        nz, nx = (int(v) for v in rng.integers(150, 330, size=2))
        kws.append(random_problem(sw, 2, order, bool(i % 2), ("null_neumann", "none",
                                  "null_dirichlet", "null_neumann"), 2, shape=(nz, nx),
                                  tf=0.05, seed=30 + i, nsrc=2, nrec=9))
    out = {}
    for h in (16, rows):
        eng = BatchEngine()
        for order in (2, 4, 8, 12, 16, 20):
            eng.set_tile_rows(order, h)
        probs = run_batch([DeviceProblem(k) for k in kws], engine=eng)
        out[h] = [(p.u_full_numpy(), p.shot_record_numpy()) for p in probs]
        eng.close()
    for (u1, r1), (u2, r2) in zip(out[16], out[rows]):
        assert np.array_equal(u1, u2) and np.array_equal(r1, r2)


def test_batch_admits_while_running():
    """Shots added after others started still give their own results."""
    from simwave_gb300.batch import BatchEngine
    from simwave_gb300.device import DeviceProblem
    kws = _shots(seed=5, count=4)
    probs = [DeviceProblem(k) for k in kws]
    eng = BatchEngine()
    ids = [eng.add(probs[0]), eng.add(probs[1])]
    eng.run(7)
    ids += [eng.add(probs[2])]
    eng.run(20)
    ids += [eng.add(probs[3])]
    while any(eng.remaining(i) > 0 for i in ids):
        eng.run(50)
    for i in ids:
        eng.release(i)
    eng.close()
    for k, p in zip(kws, probs):
        kk = dict(k, u_full=k["u_full"].copy(), shot_record=k["shot_record"].copy())
        ru, rrec, _ = oracle.forward("port", **kk)
        assert rel_l2(p.u_full_numpy(), ru) <= 1e-4
        assert rel_l2(p.shot_record_numpy(), rrec) <= 1e-4


def test_batch_rejects_3d_and_unchecked_windows():
    from simwave_gb300.batch import BatchEngine
    from simwave_gb300.device import DeviceProblem
    kw3 = random_problem(sw, 3, 4, False, "none", 0, n=20, tf=0.02)
    eng = BatchEngine()
    with pytest.raises(RuntimeError, match="2D float32"):
        eng.add(DeviceProblem(kw3))
    eng.close()


def _cd_shots(seed, count):
    """Constant-density shots with several time-blocked tiles per axis,
    every boundary kind and saving stride (sources off the halo)."""
    rng = np.random.default_rng(seed)
    bcs = ["none", "null_dirichlet", "null_neumann"]
    kws = []
    for i in range(count):
        order = int(rng.choice([2, 4, 6, 8, 12, 16, 20]))
        nz, nx = (int(v) for v in rng.integers(60, 300, size=2))
        bc = tuple(bcs[j] for j in rng.integers(0, 3, size=4))
        stride = int(rng.integers(0, 5))
        kws.append(random_problem(sw, 2, order, False, bc, stride, shape=(nz, nx),
                                  tf=float(rng.uniform(0.04, 0.1)), seed=seed + i,
                                  nsrc=int(rng.integers(1, 4)),
                                  nrec=int(rng.integers(3, 40)), multi=bool(i % 2)))
    return kws


@pytest.mark.parametrize("depth", [2, 3, 4])
def test_time_blocked_batch_matches_oracle(depth):
    """Each time-blocked shot against the oracle and the per-step batch,
    advanced in chunks that end inside time blocks."""
    from simwave_gb300.batch import BatchEngine
    from simwave_gb300.device import DeviceProblem
    kws = _cd_shots(seed=20 + depth, count=6)
    eng = BatchEngine()
    for order in range(2, 22, 2):
        try:
            eng.set_depth(order, depth)
        except RuntimeError:
            pass  # depth too large for this order: the shot keeps depth 1
    probs = [DeviceProblem(k) for k in kws]
    ids = [eng.add(p) for p in probs]
    blocked = [eng.depth(i) for i in ids]
    assert max(blocked) == depth
    while any(eng.remaining(i) > 0 for i in ids):
        eng.run(13)
    for i in ids:
        eng.release(i)
    eng.close()
    ref = BatchEngine()
    plain = [DeviceProblem(k) for k in kws]
    pids = [ref.add(p) for p in plain]
    assert all(ref.depth(i) == 1 for i in pids)
    while any(ref.remaining(i) > 0 for i in pids):
        ref.run(64)
    for i in pids:
        ref.release(i)
    ref.close()
    for k, p, q in zip(kws, probs, plain):
        assert rel_l2(p.u_full_numpy(), q.u_full_numpy()) <= 1e-5
        assert rel_l2(p.shot_record_numpy(), q.shot_record_numpy()) <= 1e-5
        kk = dict(k, u_full=k["u_full"].copy(), shot_record=k["shot_record"].copy())
        ru, rrec, _ = oracle.forward("port", **kk)
        assert rel_l2(p.u_full_numpy(), ru) <= 1e-4
        assert rel_l2(p.shot_record_numpy(), rrec) <= 1e-4


def test_time_blocking_skips_what_it_cannot_run():
    """Variable density and source windows reaching into the halo keep the
    per-step kernels (and still match the oracle)."""
    from simwave_gb300.batch import BatchEngine
    from simwave_gb300.device import DeviceProblem
    vd = random_problem(sw, 2, 4, True, "null_neumann", 0, shape=(120, 140), tf=0.05, seed=1)
    halo = random_problem(sw, 2, 4, False, "null_neumann", 0, shape=(120, 140), tf=0.05,
                          seed=2, damping=0.0)
    # move the source window onto the first rows (inside the halo)
    iv = halo["src_points_interval"].copy()
    iv[1] = iv[1] - iv[0]
    iv[0] = 0
    halo["src_points_interval"] = iv
    cd = random_problem(sw, 2, 4, False, "null_neumann", 0, shape=(120, 140), tf=0.05, seed=3)
    eng = BatchEngine()
    eng.set_depth(4, 3)
    probs = [DeviceProblem(k) for k in (vd, halo, cd)]
    ids = [eng.add(p) for p in probs]
    assert [eng.depth(i) for i in ids] == [1, 1, 3]
    while any(eng.remaining(i) > 0 for i in ids):
        eng.run(50)
    for i in ids:
        eng.release(i)
    eng.close()
    for k, p in zip((vd, halo, cd), probs):
        kk = dict(k, u_full=k["u_full"].copy(), shot_record=k["shot_record"].copy())
        ru, rrec, _ = oracle.forward("port", **kk)
        assert rel_l2(p.u_full_numpy(), ru) <= 1e-4
        assert rel_l2(p.shot_record_numpy(), rrec) <= 1e-4


def test_depth_settings_are_checked():
    from simwave_gb300.batch import BatchEngine
    eng = BatchEngine()
    with pytest.raises(RuntimeError):
        eng.set_depth(20, 4)  # 4 x 10 rows of margin leave too few owned rows
    with pytest.raises(RuntimeError):
        eng.set_depth(8, 5)
    eng.set_depth(8, 4)
    eng.set_depth(8, 1)
    eng.close()


@pytest.mark.parametrize("depth", [2, 4])
def test_time_blocked_keeps_nonzero_halos(depth):
    """Slots whose halos hold values (a run resumed from another code's
    state): 'none' and Dirichlet halos keep each slot's own values, as the
    per-step kernels leave them."""
    from simwave_gb300.batch import BatchEngine
    from simwave_gb300.device import DeviceProblem
    bc = ("none", "null_neumann", "null_dirichlet", "none")
    kw = random_problem(sw, 2, 4, False, bc, 0, shape=(150, 260), tf=0.08, seed=9, nrec=20)
    rng = np.random.default_rng(4)
    u = kw["u_full"]
    r = 2
    mask = np.ones(u.shape[1:], bool)
    mask[r:-r, r:-r] = False
    for s in range(u.shape[0]):
        u[s][mask] = rng.standard_normal(mask.sum()).astype(np.float32)
    outs = []
    for d in (1, depth):
        eng = BatchEngine()
        eng.set_depth(4, d)
        p = DeviceProblem(kw)
        i = eng.add(p)
        assert eng.depth(i) == d
        while eng.remaining(i) > 0:
            eng.run(17)
        eng.release(i)
        eng.close()
        outs.append((p.u_full_numpy(), p.shot_record_numpy()))
    assert rel_l2(outs[1][0], outs[0][0]) <= 1e-5
    assert rel_l2(outs[1][1], outs[0][1]) <= 1e-5
    kk = dict(kw, u_full=kw["u_full"].copy(), shot_record=kw["shot_record"].copy())
    ru, rrec, _ = oracle.forward("port", **kk)
    assert rel_l2(outs[1][0], ru) <= 1e-4
    assert rel_l2(outs[1][1], rrec) <= 1e-4


def test_time_blocked_shot_released_early_resumes():
    """A time-blocked shot released part way leaves its current levels in
    its slots: a second engine (per step) finishes it as if uninterrupted."""
    from simwave_gb300.batch import BatchEngine
    from simwave_gb300.device import DeviceProblem
    kw = random_problem(sw, 2, 8, False, "null_neumann", 0, shape=(140, 200), tf=0.08,
                        seed=12, nrec=9)
    p = DeviceProblem(kw)
    eng = BatchEngine()
    eng.set_depth(8, 3)
    i = eng.add(p)
    assert eng.depth(i) == 3
    eng.run(22)
    left = eng.remaining(i)
    assert 0 < left
    eng.release(i)
    eng.close()
    # continue the same device problem from step 23 with per-step kernels
    eng = BatchEngine()
    p.problem.begin_timestep = int(kw["end_timestep"]) - left + 1
    i = eng.add(p)
    while eng.remaining(i) > 0:
        eng.run(50)
    eng.release(i)
    eng.close()
    kk = dict(kw, u_full=kw["u_full"].copy(), shot_record=kw["shot_record"].copy())
    ru, rrec, _ = oracle.forward("port", **kk)
    assert rel_l2(p.u_full_numpy(), ru) <= 1e-4
    assert rel_l2(p.shot_record_numpy(), rrec) <= 1e-4


def test_autotune_returns_a_valid_setting():
    from simwave_gb300.batch import BatchEngine, autotune, run_batch
    from simwave_gb300.device import DeviceProblem
    kws = _cd_shots(seed=40, count=4)
    probs = [DeviceProblem(k) for k in kws]
    tuning = autotune(probs, steps=16)
    assert set(tuning) == {int(k["space_order"]) for k in kws}
    for t in tuning.values():
        assert t["rows"] in (8, 16, 32, 64, 128, 256) and 1 <= t["depth"] <= 4
    eng = BatchEngine()
    eng.apply(tuning)
    run_batch(probs, engine=eng)
    eng.close()
    for k, p in zip(kws, probs):
        kk = dict(k, u_full=k["u_full"].copy(), shot_record=k["shot_record"].copy())
        ru, rrec, _ = oracle.forward("port", **kk)
        assert rel_l2(p.u_full_numpy(), ru) <= 1e-4
        assert rel_l2(p.shot_record_numpy(), rrec) <= 1e-4
