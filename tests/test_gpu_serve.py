"""The request server: concurrent solves give the same results as solving alone.

Requests of one shape run as one grouped solve, whose members run the same
deterministic kernels and host arithmetic as their solves alone, so the eigenvalues
served in a mix must equal those of the plain one-at-a-time path (compared at 1e-12
relative; they agree bit for bit).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _requests():
    from eigenfns_gb300.serve import SolveRequest
    return [SolveRequest(0, 64, 32, 11, 8, (0.1, -0.2, 0.3)),
            SolveRequest(1, 64, 32, 12, 12, (0.0, 0.0, 0.0)),
            SolveRequest(2, 216, 48, 13, 10, (0.25, 0.1, -0.4)),
            SolveRequest(3, 64, 32, 14, 16, (-0.3, 0.45, 0.05), arrival=0.05)]


def test_served_results_equal_solving_alone():
    from eigenfns_gb300.serve import EigenServer, run_plain
    reqs = _requests()
    alone = run_plain(reqs)
    srv = EigenServer(budget_bytes=40e9, max_concurrent=4)
    served = srv.run(reqs, realtime=True)
    assert srv.peak_concurrent >= 2
    for a, b in zip(alone, served):
        assert a.rid == b.rid and len(a.vals) == len(b.vals)
        assert np.abs(a.vals - b.vals).max() <= 1e-12 * np.abs(a.vals).max()
        assert b.max_res < 1e-4


def test_admission_respects_the_budget():
    from eigenfns_gb300.serve import EigenServer, footprint_bytes
    reqs = _requests()[:3]
    fps = [footprint_bytes(r) for r in reqs]
    budget = max(fps) * 1.01
    srv = EigenServer(budget_bytes=budget, max_concurrent=8)
    res = srv.run(reqs, realtime=False)
    assert len(res) == 3 and srv.peak_used <= budget
    # two requests whose footprints do not fit together run one at a time
    pair = _requests()[:2]
    tight = max(footprint_bytes(r) for r in pair) * 1.01
    assert tight < sum(footprint_bytes(r) for r in pair)
    srv = EigenServer(budget_bytes=tight, max_concurrent=8)
    assert len(srv.run(pair, realtime=False)) == 2 and srv.peak_concurrent == 1
    with pytest.raises(ValueError):
        EigenServer(budget_bytes=max(fps) / 4).run(reqs, realtime=False)


def test_footprint_covers_measured_device_memory():
    """The admission footprint of a request is at least the device memory its solve
    allocates through torch (the peak above the level before the request), which holds
    the blocks, the locked set, the slabs and the scratch; the operator's own tables,
    allocated by the library, are the footprint's 20 B per voxel on top."""
    from eigenfns_gb300 import blas
    from eigenfns_gb300.serve import SolveRequest, _solve_one, footprint_bytes
    for req in (SolveRequest(0, 64, 32, 21, 16, (0.1, 0.2, 0.3)),
                SolveRequest(1, 216, 48, 22, 24, (0.0, 0.0, 0.0))):
        blas.release_workspaces()
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        base = torch.cuda.memory_allocated()
        torch.cuda.reset_peak_memory_stats()
        _solve_one(req, torch.device("cuda", 0))
        torch.cuda.synchronize()
        used = torch.cuda.max_memory_allocated() - base
        assert used <= footprint_bytes(req), (used, footprint_bytes(req))


def test_group_footprint_covers_measured_device_memory():
    """A grouped solve's device memory (stacked slabs, locked sets, temporaries) stays
    within the sum of its members' admission footprints."""
    from eigenfns_gb300 import blas
    from eigenfns_gb300.grouped import run_group
    from eigenfns_gb300.serve import SolveRequest, _group_steps, _operator, footprint_bytes
    reqs = [SolveRequest(i, 216, 48, 30 + i, 24, (0.1 * i, 0.0, -0.1)) for i in range(3)]
    dev = torch.device("cuda", 0)
    ops = [_operator(r, dev) for r in reqs]
    blas.release_workspaces()
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    base = torch.cuda.memory_allocated()
    torch.cuda.reset_peak_memory_stats()
    res = run_group(_group_steps(reqs, ops))
    torch.cuda.synchronize()
    used = torch.cuda.max_memory_allocated() - base
    assert sorted(res) == [0, 1, 2] and not any(isinstance(v, Exception) for v in res.values())
    assert used <= sum(footprint_bytes(r) for r in reqs), (used, [footprint_bytes(r) for r in reqs])
