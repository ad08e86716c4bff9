"""A continuously batched eigensolve server on one GPU.

Requests (structure seed and size, grid, Bloch k, number of bands, tolerance)
arrive over time. The server admits a waiting request as soon as a slot is free
and its device-memory footprint fits the budget, and adds its solve to the running
batch: the admitted solves advance round robin (eigenfns_gb300.batched), each one
request ahead of the host, so the host's work on one solve overlaps the device work
the others queued, and a request that arrives while others run joins at the next step.
Solver state (blocks, locked set, operator tables, scratch) stays on the device for
the life of the request and is released when it finishes. Each solve is the plain
deflated block LOBPCG of eigenfns_gb300.solver with the same kernels in the same
order as alone, so its result is the same alone and in the mix.

`run_plain` processes the same requests one at a time (the plain path) for the
served-vs-plain comparison.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np
import torch



@dataclass
class SolveRequest:
    rid: int
    nodes: int
    grid: int
    seed: int
    nev: int
    k_frac: tuple = (0.0, 0.0, 0.0)
    tol: float = 1e-4
    arrival: float = 0.0          # seconds after the start of the run

    def block(self) -> tuple:
        """LOBPCG block and guard for this request: about nev/2 per block, 8..32."""
        m = int(min(32, max(8, 2 * math.ceil(self.nev / 4))))
        guard = max(2, m // 4)
        return m, guard


@dataclass
class SolveResult:
    rid: int
    vals: np.ndarray
    max_res: float
    arrival: float
    start: float
    end: float
    theta_applications: int
    iterations: int

    @property
    def latency(self) -> float:
        return self.end - self.arrival


def footprint_bytes(req: SolveRequest) -> int:
    """Device memory a request holds while it runs (vectors, locked set, tables, scratch)."""
    G = req.grid
    N = G ** 3
    vec = 2 * N * 8
    m, guard = req.block()
    cap = int(math.ceil(req.nev / max(m - guard, 1))) * (m - guard) + m
    slabs = 9 * m                       # two [P; X; W] slabs and [ΘP; ΘX; ΘW]
    extra = 4 * m                       # carries, index copies, Gram/rotation temporaries
    theta_ws = min(96 << 20, 3 * N * 8 * m) + (64 << 20)
    tables = 20 * N                     # eps copies, switch bits, structure scratch
    return int((cap + slabs + extra) * vec + theta_ws + tables)


def _operator(req: SolveRequest, device: torch.device):
    from .operator import MaxwellOperator
    from .structure import make_structure
    eps, L, _ = make_structure(req.nodes, req.grid, seed=req.seed)
    return MaxwellOperator(eps, L, k_frac=req.k_frac, device=device)


def _steps(req: SolveRequest, op, check_tc: bool):
    from .solver import lobpcg_steps
    m, guard = req.block()
    return lobpcg_steps(op, req.nev, m=m, guard=guard, tol=req.tol, seed=req.seed,
                        verbose=False, check_tc=check_tc)


def _solve_one(req: SolveRequest, device: torch.device):
    from .solver import run_steps
    op = _operator(req, device)
    vals, vecs, st = run_steps(_steps(req, op, True))
    del vecs, op
    return vals, st


class EigenServer:
    """Admission by device-memory footprint; admitted solves run in one pipelined batch."""

    def __init__(self, budget_bytes: float = 160e9, max_concurrent: int = 16, device=None):
        self.budget = float(budget_bytes)
        self.max_concurrent = int(max_concurrent)
        self.device = torch.device(device) if device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        self._used = 0.0
        self.peak_concurrent = 0
        self.peak_used = 0.0
        self.errors: list = []
        self.steps = 0

    def run(self, requests, realtime: bool = True) -> list:
        """Serve `requests` (arrival times honoured when `realtime`); returns results."""
        from .batched import BatchedSolves
        pending = sorted(requests, key=lambda r: r.arrival)
        for r in pending:
            if footprint_bytes(r) > self.budget:
                raise ValueError(f"request {r.rid} needs {footprint_bytes(r) / 1e9:.1f} GB, "
                                 f"above the {self.budget / 1e9:.1f} GB budget")
        results: list = []
        batch = BatchedSolves()
        running: dict = {}            # rid -> (request, footprint, start, operator)
        t0 = time.perf_counter()

        def finish(done: dict):
            for rid, res in done.items():
                req, fp, start, _ = running.pop(rid)
                self._used -= fp
                if isinstance(res, Exception):
                    self.errors.append((rid, repr(res)))
                    continue
                vals, vecs, st = res
                del vecs
                results.append(SolveResult(rid, vals, max(r["max_res_locked"] for r in st.rounds),
                                           req.arrival, start, time.perf_counter() - t0,
                                           st.theta_applications, st.iterations))

        with torch.cuda.device(self.device):
            while pending or len(batch):
                now = time.perf_counter() - t0
                while pending:
                    head = pending[0]
                    fp = footprint_bytes(head)
                    arrived = (not realtime) or head.arrival <= now
                    if not (arrived and len(running) < self.max_concurrent
                            and self._used + fp <= self.budget):
                        break
                    pending.pop(0)
                    self._used += fp
                    start = time.perf_counter() - t0
                    op = _operator(head, self.device)
                    running[head.rid] = (head, fp, start, op)
                    self.peak_concurrent = max(self.peak_concurrent, len(running))
                    self.peak_used = max(self.peak_used, self._used)
                    finish(batch.add(head.rid, _steps(head, op, False)))
                if len(batch):
                    finish(batch.step())
                elif pending and realtime:
                    time.sleep(max(min(pending[0].arrival - (time.perf_counter() - t0), 0.05), 1e-4))
            self.steps = batch.steps
            torch.cuda.synchronize(self.device)
        if self.errors:
            raise RuntimeError(f"{len(self.errors)} request(s) failed: {self.errors[:3]}")
        return sorted(results, key=lambda r: r.rid)


def run_plain(requests, device=None) -> list:
    """The plain path: the same requests solved one after another, on one stream."""
    device = torch.device(device) if device is not None else torch.device(
        "cuda", torch.cuda.current_device())
    results = []
    t0 = time.perf_counter()
    for req in sorted(requests, key=lambda r: r.arrival):
        start = time.perf_counter() - t0
        vals, st = _solve_one(req, device)
        torch.cuda.synchronize(device)
        end = time.perf_counter() - t0
        results.append(SolveResult(req.rid, vals, max(r["max_res_locked"] for r in st.rounds),
                                   req.arrival, start, end, st.theta_applications, st.iterations))
    return sorted(results, key=lambda r: r.rid)


def poisson_requests(n: int, seed: int, rate_hz: float, nodes=(64, 216, 512), grids=(32, 48, 64),
                     nev_range=(8, 48)) -> list:
    """A seeded request stream: Poisson arrivals, node count with its grid, random k and bands."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate_hz)
        j = int(rng.integers(len(nodes)))
        k = tuple(float(x) for x in rng.random(3) - 0.5)
        out.append(SolveRequest(rid=i, nodes=int(nodes[j]), grid=int(grids[j]),
                                seed=int(rng.integers(1 << 30)), k_frac=k,
                                nev=int(rng.integers(nev_range[0], nev_range[1] + 1)), arrival=t))
    return out


def summarize(results, wall: float) -> dict:
    lat = np.asarray([r.latency for r in results])
    modes = int(sum(len(r.vals) for r in results))
    return {"requests": len(results), "modes": modes, "wall_s": wall, "modes_per_s": modes / wall,
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "max_res": float(max(r.max_res for r in results))}
