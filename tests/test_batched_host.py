"""Host logic of the lock-step batch driver (eigenfns_gb300.batched) on the CPU: solves
of different lengths advance together, one shared transfer per step, failures and a
tensor-core timeout are reported per solve."""
from __future__ import annotations

import pytest

torch = pytest.importorskip("torch")


class _Stream:
    def __init__(self, log):
        self.log = log

    def synchronize(self):
        self.log.append("sync")


@pytest.fixture()
def driver(monkeypatch):
    from eigenfns_gb300 import batched, blas
    log = []
    flag = {"tc": 0}
    monkeypatch.setattr(torch.cuda, "current_stream", lambda d=None: _Stream(log))
    monkeypatch.setattr(batched, "_request_to_host", lambda req: req)
    monkeypatch.setattr(blas, "tc_error", lambda: flag["tc"])
    return batched, log, flag


def _solve(name, n, log, fail_at=None):
    acc = 0
    for i in range(n):
        log.append(f"{name}{i}")
        h = yield torch.tensor([float(i)])
        if fail_at == i:
            raise ValueError(f"{name} failed")
        acc += int(h[0])
    return name, acc


def test_lock_step_shares_one_sync_per_step(driver):
    batched, log, _ = driver
    d = batched.BatchedSolves(streams=1)
    for name, n in (("a", 3), ("b", 1), ("c", 2)):
        d.add(name, _solve(name, n, log))
    out = d.run()
    assert out == {"a": ("a", 3), "b": ("b", 0), "c": ("c", 1)}
    assert d.steps == 3 and log.count("sync") == 3
    # every solve queued its step-k work before the step-k synchronisation
    assert log[:4] == ["a0", "b0", "c0", "sync"]


def test_failures_are_per_solve_and_timeouts_fail_all(driver):
    batched, log, flag = driver
    d = batched.BatchedSolves(streams=1)
    d.add("ok", _solve("ok", 2, log))
    d.add("bad", _solve("bad", 3, log, fail_at=0))
    out = d.run()
    assert out["ok"] == ("ok", 1) and isinstance(out["bad"], ValueError)
    d = batched.BatchedSolves(streams=1)
    d.add("x", _solve("x", 3, log))
    d.add("y", _solve("y", 3, log))
    flag["tc"] = 1
    out = d.step()
    assert set(out) == {"x", "y"} and all(isinstance(v, RuntimeError) for v in out.values())
    assert len(d) == 0
