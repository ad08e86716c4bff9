"""Host logic of the pipelined batch driver (eigenfns_gb300.batched) on the CPU: solves
of different lengths advance round robin, each step waits for each solve's own request
only, failures are reported per solve and a tensor-core timeout fails every solve in
flight."""
from __future__ import annotations

import pytest

torch = pytest.importorskip("torch")


@pytest.fixture()
def driver(monkeypatch):
    from eigenfns_gb300 import batched, blas
    log = []
    flag = {"tc": 0, "cleared": 0}

    class _Event:
        def __init__(self, tag):
            self.tag = tag

    def clear():
        flag["cleared"] += 1
        v, flag["tc"] = flag["tc"], 0
        return v

    monkeypatch.setattr(batched, "_request_to_host", lambda req: req)
    monkeypatch.setattr(batched, "_new_flag", lambda: {"v": 0})
    monkeypatch.setattr(batched, "_queue_flag", lambda f: f.__setitem__("v", flag["tc"]))
    monkeypatch.setattr(batched, "_flag_value", lambda f: f["v"])
    monkeypatch.setattr(batched, "_record_event", lambda: _Event(len(log)))
    monkeypatch.setattr(batched, "_wait", lambda ev: log.append("wait"))
    monkeypatch.setattr(blas, "tc_error", clear)
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


def test_round_robin_waits_per_solve(driver):
    batched, log, _ = driver
    d = batched.BatchedSolves()
    for name, n in (("a", 3), ("b", 1), ("c", 2)):
        d.add(name, _solve(name, n, log))
    out = d.run()
    assert out == {"a": ("a", 3), "b": ("b", 0), "c": ("c", 1)}
    assert d.steps == 3
    # every solve queued its first request on joining; a step waits for one solve's own
    # request, resumes it (which queues its next work) and only then waits for the next
    assert log[:3] == ["a0", "b0", "c0"]
    assert log[3:9] == ["wait", "a1", "wait", "wait", "c1", "wait"]
    assert log.count("wait") == 3 + 2 + 1


def test_failures_are_per_solve_and_timeouts_fail_all(driver):
    batched, log, flag = driver
    d = batched.BatchedSolves()
    d.add("ok", _solve("ok", 2, log))
    d.add("bad", _solve("bad", 3, log, fail_at=0))
    out = d.run()
    assert out["ok"] == ("ok", 1) and isinstance(out["bad"], ValueError)
    d = batched.BatchedSolves()
    d.add("x", _solve("x", 3, log))
    flag["tc"] = 1                          # a timeout before y's request was copied
    d.add("y", _solve("y", 3, log))
    out = d.step()
    assert set(out) == {"x", "y"} and all(isinstance(v, RuntimeError) for v in out.values())
    assert len(d) == 0 and flag["cleared"] == 1 and flag["tc"] == 0


def _group(names, lengths, log):
    """A stand-in grouped solve: members finish after their own number of steps and are
    reported through GroupResults at the step they finish."""
    from eigenfns_gb300.grouped import GroupResults
    left = dict(zip(names, lengths))
    step = 0
    while True:
        log.append(f"g{step}")
        yield torch.tensor([float(step)])
        step += 1
        done = {k: (k, step) for k, n in left.items() if n == step}
        for k in done:
            del left[k]
        if not left:
            return GroupResults(done)
        if done:
            yield GroupResults(done)


def test_group_members_report_as_they_finish(driver):
    batched, log, _ = driver
    d = batched.BatchedSolves()
    d.add(("group", 0), _group(["p", "q", "r"], [1, 3, 2], log))
    d.add("solo", _solve("solo", 2, log))
    seen = []
    while len(d):
        seen.append(sorted(map(str, d.step())))
    assert seen == [["p"], ["r", "solo"], ["q"]]


def test_group_by_shape_keeps_order_and_caps_size():
    from eigenfns_gb300.batched import group_by_shape

    class _Op:
        def __init__(self, g):
            self.grid_size, self.device = g, "cuda:0"

    ops = [_Op(g) for g in (32, 48, 32, 32, 48, 32)]
    ms = [16, 32, 16, 16, 32, 8]
    groups = group_by_shape(ops, ms, [4] * 6, max_group=2)
    assert groups == [[0, 2], [3], [1, 4], [5]]


def test_combined_host_reads_and_stacked_eigh():
    """A HostMany request comes back as the list of its parts' results: numpy copies for
    tensors and (w, V) for HostEigh, stacked for a stack of matrices (one LAPACK call per
    problem, the same numbers as for the matrix alone)."""
    import numpy as np
    from eigenfns_gb300.solver import HostEigh, HostMany, run_steps

    rng = np.random.default_rng(3)
    A = rng.standard_normal((3, 50, 50)) + 1j * rng.standard_normal((3, 50, 50))
    A = A + A.conj().transpose(0, 2, 1)

    def gen():
        t, (w, V) = yield HostMany([torch.arange(4.0), HostEigh(torch.from_numpy(A))])
        w1, V1 = yield HostEigh(torch.from_numpy(A[1]))
        return t, w, V, w1, V1

    t, w, V, w1, V1 = run_steps(gen())
    assert np.array_equal(t, np.arange(4.0)) and w.shape == (3, 50) and V.shape == (3, 50, 50)
    assert np.array_equal(w[1], w1) and np.array_equal(V[1], V1)
    for i in range(3):
        assert np.allclose(A[i] @ V[i], V[i] * w[i][None, :], atol=1e-10)


def test_host_copy_requests_are_read_without_a_second_copy():
    """A HostEigh of a HostCopy (the copy queued before more device work) reaches the
    eigendecomposition from its own pinned buffer, after its own event, in both drivers."""
    import numpy as np
    from eigenfns_gb300 import batched, solver

    class _Event:
        def __init__(self):
            self.waited = False

        def synchronize(self):
            self.waited = True

    hc = solver.HostCopy.__new__(solver.HostCopy)
    hc.host = torch.diag(torch.tensor([3.0, 1.0, 2.0], dtype=torch.float64)).to(torch.complex128)
    hc.event = _Event()
    req = solver.HostEigh(hc)
    assert batched._request_to_host(req).A is hc.host
    w, V = solver._to_host(req)
    assert hc.event.waited and np.allclose(w, [1.0, 2.0, 3.0]) and V.shape == (3, 3)
