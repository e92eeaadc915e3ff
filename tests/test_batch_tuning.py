"""The batch autotuner's choices (host logic only; timings are faked): tile
rows per order from the order's shots alone, then a time-blocking depth per
order kept only when the whole shot set runs at least the margin faster."""
import types

import pytest

torch = pytest.importorskip("torch")
from simwave_gb300 import batch  # noqa: E402


def _shot(order):
    prob = types.SimpleNamespace(space_order=order)
    return types.SimpleNamespace(problem=prob, device="cpu", reset=lambda: None)


def _tuning_with(monkeypatch, shots, timing, candidates):
    monkeypatch.setattr(batch, "_time_engine",
                        lambda probs, tuning, steps: timing(probs, tuning))
    monkeypatch.setattr(batch, "_candidates",
                        lambda order, rows, depths, device: candidates[order])
    return batch.autotune(shots, steps=8)


def test_rows_from_each_order_and_depth_only_with_margin(monkeypatch):
    shots = [_shot(4), _shot(4), _shot(8)]
    candidates = {4: [(8, 1), (16, 1), (32, 1), (16, 2), (16, 4)],
                  8: [(8, 1), (16, 1), (32, 1), (16, 2)]}

    def timing(probs, tuning):
        orders = {int(p.problem.space_order) for p in probs}
        if len(probs) < len(shots):  # one order alone: rows only
            (o,) = orders
            return {8: 3.0, 16: 1.0, 32: 2.0, 64: 1.5, 128: 2.5, 256: 2.5}[tuning[o]["rows"]] \
                if o == 4 else {8: 1.0, 16: 2.0, 32: 3.0, 64: 4.0, 128: 5.0,
                                256: 5.0}[tuning[o]["rows"]]
        t = 10.0
        t -= {1: 0.0, 2: 0.5, 4: 1.0}[tuning[4]["depth"]]   # 5 % and 10 % faster
        t -= {1: 0.0, 2: 0.1}[tuning[8]["depth"]]           # 1 %: below the margin
        return t

    got = _tuning_with(monkeypatch, shots, timing, candidates)
    assert got == {4: {"rows": 16, "depth": 4}, 8: {"rows": 8, "depth": 1}}


def test_depth_never_kept_when_slower(monkeypatch):
    shots = [_shot(12)]
    candidates = {12: [(8, 1), (16, 1), (32, 1), (16, 2), (16, 3)]}

    def timing(probs, tuning):
        return 1.0 if tuning[12]["depth"] == 1 else 1.2

    got = _tuning_with(monkeypatch, shots, timing, candidates)
    assert got[12]["depth"] == 1
