"""The batch engine against the CPU checker and the single-shot entry: mixed
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


def test_batch_matches_checker():
    from simwave_gb300.batch import run_batch
    from simwave_gb300.device import DeviceProblem
    kws = _shots(seed=3)
    probs = run_batch([DeviceProblem(k) for k in kws], chunk=40)
    for k, p in zip(kws, probs):
        kk = dict(k, u_full=k["u_full"].copy(), shot_record=k["shot_record"].copy())
        ru, rrec, _ = oracle.forward("port", **kk)
        assert rel_l2(p.u_full_numpy(), ru) <= 1e-4
        assert rel_l2(p.shot_record_numpy(), rrec) <= 1e-4


@pytest.mark.parametrize("rows", [8, 16, 32])
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
