"""Host logic of the request server on the CPU: admission by device-memory footprint,
the concurrency cap, arrival order, error surfacing and the same results served as
plain. The solve itself is replaced by a deterministic stand-in (the real one runs in
tests/test_gpu_serve.py)."""
from __future__ import annotations

import contextlib
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")


class _Stream:
    def synchronize(self):
        pass


@pytest.fixture()
def fake_server(monkeypatch):
    """The server with its solves replaced by step generators that yield CPU tensors a
    few times and return made-up eigenvalues (the batch driver's host transfer becomes a
    no-op), so admission, batching and result order are exercised without a GPU."""
    from eigenfns_gb300 import batched, blas, serve
    monkeypatch.setattr(torch.cuda, "device", lambda d: contextlib.nullcontext())
    monkeypatch.setattr(torch.cuda, "synchronize", lambda d=None: None)
    monkeypatch.setattr(torch.cuda, "current_stream", lambda d=None: _Stream())
    monkeypatch.setattr(batched, "_request_to_host", lambda req: req)
    monkeypatch.setattr(batched, "_new_flag", lambda: [0])
    monkeypatch.setattr(batched, "_queue_flag", lambda f: None)
    monkeypatch.setattr(batched, "_record_event", lambda: None)
    monkeypatch.setattr(batched, "_wait", lambda ev: None)
    monkeypatch.setattr(blas, "tc_error", lambda: 0)
    state = {"running": 0, "peak": 0}

    class _Stats:
        def __init__(self, req):
            self.rounds = [{"max_res_locked": 1e-5}]
            self.theta_applications = 10 * req.nev
            self.iterations = req.nev

    def fake_steps(req, op, check_tc):
        state["running"] += 1
        state["peak"] = max(state["peak"], state["running"])
        try:
            for _ in range(2 + req.nev % 3):
                time.sleep(0.003)                   # device work of one step
                h = yield torch.zeros(2)
                assert h.shape == (2,)
                if req.seed < 0:
                    raise RuntimeError("planted failure")
            time.sleep(0.002)
            vals = np.sort(np.random.default_rng(req.seed).random(req.nev)) + req.grid
            return vals, None, _Stats(req)
        finally:
            state["running"] -= 1

    def fake_solve(req, device):
        from eigenfns_gb300.solver import run_steps
        monkeypatch.setattr("eigenfns_gb300.solver._to_host", lambda r: r.numpy())
        vals, _, st = run_steps(fake_steps(req, None, True))
        return vals, st

    def fake_group(reqs, ops):
        """Members advance in lock step on one shared host read; each is reported as
        it finishes, as the grouped solver does."""
        from eigenfns_gb300.grouped import GroupResults
        gens, done = {}, {}
        for r in reqs:
            g = fake_steps(r, None, False)
            try:
                next(g)
                gens[r.rid] = g
            except StopIteration as stop:
                done[r.rid] = stop.value
        while gens:
            h = yield torch.zeros(2)
            finished = {}
            for rid, g in list(gens.items()):
                try:
                    g.send(h)
                except StopIteration as stop:
                    finished[rid] = stop.value
                    del gens[rid]
                except Exception as exc:
                    finished[rid] = exc
                    del gens[rid]
            done.update(finished)
            if finished and gens:
                yield GroupResults(finished)
                done = {}
        return GroupResults(done)

    monkeypatch.setattr(serve, "_operator", lambda req, device: None)
    monkeypatch.setattr(serve, "_steps", fake_steps)
    monkeypatch.setattr(serve, "_group_steps", fake_group)
    monkeypatch.setattr(serve, "_solve_one", fake_solve)
    return serve, state


def _requests(serve, n=12):
    return [serve.SolveRequest(rid=i, nodes=64, grid=32 if i % 3 else 48, seed=100 + i,
                               nev=8 + (i % 5), arrival=0.005 * i) for i in range(n)]


def test_admission_respects_budget_and_concurrency(fake_server):
    serve, state = fake_server
    reqs = [serve.SolveRequest(rid=i, nodes=64, grid=32, seed=100 + i, nev=12, arrival=0.002 * i)
            for i in range(10)]
    fp = serve.footprint_bytes(reqs[0])
    srv = serve.EigenServer(budget_bytes=2.5 * fp, max_concurrent=4, device="cpu")
    res = srv.run(reqs, realtime=True)           # memory admits two at a time
    assert [r.rid for r in res] == list(range(len(reqs)))
    assert srv.peak_used <= 2.5 * fp and srv.peak_concurrent == 2 and state["peak"] <= 2
    assert all(r.start >= r.arrival - 1e-6 and r.end >= r.start for r in res)
    state["peak"] = 0
    mixed = _requests(serve)
    srv = serve.EigenServer(budget_bytes=1e15, max_concurrent=3, device="cpu")
    res = srv.run(mixed, realtime=False)         # the slot cap binds
    assert len(res) == len(mixed) and srv.peak_concurrent <= 3 and state["peak"] <= 3


def test_served_results_equal_plain(fake_server):
    serve, _ = fake_server
    reqs = _requests(serve, 8)
    served = serve.EigenServer(budget_bytes=1e15, max_concurrent=8, device="cpu").run(reqs,
                                                                                      realtime=False)
    plain = serve.run_plain(reqs, device="cpu")
    for a, b in zip(served, plain):
        assert a.rid == b.rid and np.array_equal(a.vals, b.vals)
    s = serve.summarize(served, 1.0)
    assert s["modes"] == sum(r.nev for r in reqs) and s["p99_latency_s"] >= s["p50_latency_s"]


def test_oversized_request_and_failures_are_reported(fake_server):
    serve, _ = fake_server
    reqs = _requests(serve, 4)
    with pytest.raises(ValueError):
        serve.EigenServer(budget_bytes=1.0, device="cpu").run(reqs)
    reqs[2].seed = -1                        # planted failure inside one solve
    with pytest.raises(RuntimeError, match="1 request"):
        serve.EigenServer(budget_bytes=1e15, device="cpu").run(reqs, realtime=False)


def test_request_stream_is_seeded():
    from eigenfns_gb300 import serve
    a = serve.poisson_requests(20, seed=5, rate_hz=40.0)
    b = serve.poisson_requests(20, seed=5, rate_hz=40.0)
    assert [(r.grid, r.nev, r.k_frac, r.arrival) for r in a] == \
           [(r.grid, r.nev, r.k_frac, r.arrival) for r in b]
    assert all(a[i].arrival < a[i + 1].arrival for i in range(19))
    assert all(-0.5 <= x < 0.5 for r in a for x in r.k_frac)
    assert all(8 <= r.nev <= 48 and r.grid in (32, 48, 64) for r in a)


def test_waiting_requests_start_as_groups(fake_server):
    serve, _ = fake_server
    reqs = [serve.SolveRequest(rid=i, nodes=64, grid=32 if i < 6 else 48, seed=100 + i,
                               nev=12 if i % 2 else 30, arrival=0.0,
                               block_size=8 if i in (0, 6) else 16) for i in range(10)]
    srv = serve.EigenServer(budget_bytes=1e15, max_concurrent=16, device="cpu")
    res = srv.run(reqs, realtime=False)
    # one group per (grid, block) shape: 32^3 x {8, 16} and 48^3 x {8, 16}
    assert len(res) == 10 and srv.groups == 4 and srv.peak_concurrent == 10


def test_full_shape_request_stream():
    """bench_serve.py's stream: seeded, N paired with its grid (N = 1000 on 96^3 or 128^3),
    8-120 bands, increasing arrivals, and every request fits the 160 GB admission budget."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench_serve
    from eigenfns_gb300 import serve
    a = bench_serve.requests(64, seed=3, rate_hz=2.0, tol=1e-4)
    b = bench_serve.requests(64, seed=3, rate_hz=2.0, tol=1e-4)
    assert [(r.nodes, r.grid, r.nev, r.k_frac, r.arrival) for r in a] == \
           [(r.nodes, r.grid, r.nev, r.k_frac, r.arrival) for r in b]
    assert all((r.nodes, r.grid) in bench_serve.KINDS for r in a)
    assert {r.grid for r in a} == {32, 48, 64, 96, 128}
    assert all(8 <= r.nev <= 120 and r.tol == 1e-4 for r in a)
    assert all(a[i].arrival < a[i + 1].arrival for i in range(63))
    assert max(serve.footprint_bytes(r) for r in a) < 160e9


def test_large_grid_requests_run_alone_without_blocking_small_ones(fake_server):
    """Requests on grids >= exclusive_grid run one at a time and by themselves; lighter
    requests behind a waiting large one are admitted while it waits."""
    serve, state = fake_server
    big = [serve.SolveRequest(rid=i, nodes=1000, grid=128, seed=10 + i, nev=20, arrival=0.0)
           for i in range(3)]
    small = [serve.SolveRequest(rid=3 + i, nodes=64, grid=32, seed=20 + i, nev=9, arrival=0.001)
             for i in range(4)]
    srv = serve.EigenServer(budget_bytes=1e15, max_concurrent=16, device="cpu", group_wait=0.0,
                            min_group=1)
    res = {r.rid: r for r in srv.run(big + small, realtime=True)}
    assert len(res) == 7
    spans = sorted((res[i].start, res[i].end) for i in range(3))
    assert all(spans[j][1] <= spans[j + 1][0] + 1e-6 for j in range(2))   # one at a time
    assert all(res[3 + i].start < spans[1][0] for i in range(4))            # not held back
    srv = serve.EigenServer(budget_bytes=1e15, max_concurrent=16, device="cpu", group_wait=0.0,
                            min_group=1, exclusive_grid=1 << 30)
    res = srv.run(big, realtime=False)
    assert len({r.start for r in res}) == 1                                  # one group otherwise
