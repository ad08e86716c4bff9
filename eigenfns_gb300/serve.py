"""A continuously batched eigensolve server on one GPU.

Requests (structure seed and size, grid, Bloch k, number of bands, tolerance)
arrive over time. The server admits waiting requests when slots are free and their
device-memory footprints fit the budget. Admitted requests of one shape (grid edge and
LOBPCG block) start together as one grouped solve (eigenfns_gb300.grouped: one launch
sequence per iteration for the whole group, their projected problems on parallel host
threads); all running groups advance round robin in the pipelined batch driver
(eigenfns_gb300.batched), so the host's work on one group overlaps the device work of
the others. While the GPU is busy, newly arrived requests wait up to `group_wait`
seconds (or until `min_group` of them are waiting) so that they start as a group rather
than one by one. A request's result is reported when its own bands are locked; a
group's device memory is released when its last member finishes. Each member computes
exactly what its solve computes alone (grouped solves are bit-for-bit the single
solves), so a request's result is the same served and plain.

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

    block_size: int = 16          # LOBPCG block; the guard is a quarter of it

    def block(self) -> tuple:
        """LOBPCG block and guard: one block size for every request by default, so that
        requests on one grid share a shape and can run as one grouped solve."""
        return int(self.block_size), int(self.block_size) // 4


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


def _shape(req: SolveRequest) -> tuple:
    return (req.grid,) + req.block() + (req.tol,)


def _group_steps(reqs: list, ops: list):
    """One grouped solve for requests of one shape (members keyed by request id)."""
    from .grouped import lobpcg_group_steps
    m, guard = reqs[0].block()
    return lobpcg_group_steps(ops, [r.nev for r in reqs], keys=[r.rid for r in reqs], m=m,
                              guard=guard, tol=reqs[0].tol, seeds=[r.seed for r in reqs])


def _solve_one(req: SolveRequest, device: torch.device):
    from .solver import run_steps
    op = _operator(req, device)
    vals, vecs, st = run_steps(_steps(req, op, True))
    del vecs, op
    return vals, st


class EigenServer:
    """Admission by device-memory footprint; admitted requests of one shape start as one
    grouped solve; the running groups advance in one pipelined batch."""

    def __init__(self, budget_bytes: float = 160e9, max_concurrent: int = 16, device=None,
                 group_wait: float = 0.5, min_group: int = 12, max_group: int = 32,
                 exclusive_grid: int = 96):
        """`exclusive_grid`: requests on grids of this edge or larger keep the device busy
        alone (their kernels fill every SM), so interleaving two of them gains nothing
        and lengthens both latencies: at most one such request runs at a time, by
        itself, and lighter requests are admitted around it (a large request waiting
        for the running one does not hold back the lighter requests behind it)."""
        self.budget = float(budget_bytes)
        self.exclusive_grid = int(exclusive_grid)
        self.max_concurrent = int(max_concurrent)
        self.group_wait = float(group_wait)
        self.min_group = int(min_group)
        self.max_group = int(max_group)
        self.device = torch.device(device) if device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        self._used = 0.0
        self.peak_concurrent = 0
        self.peak_used = 0.0
        self.errors: list = []
        self.steps = 0
        self.groups = 0

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
        running: dict = {}            # rid -> (request, start, group key)
        groups: dict = {}             # group key -> [members still running, bytes held]
        t0 = time.perf_counter()

        def record(rid, res):
            req, start, gk = running.pop(rid)
            if isinstance(res, Exception):
                self.errors.append((rid, repr(res)))
            else:
                vals, vecs, st = res
                del vecs
                results.append(SolveResult(rid, vals, max(r["max_res_locked"] for r in st.rounds),
                                           req.arrival, start, time.perf_counter() - t0,
                                           st.theta_applications, st.iterations))
            g = groups[gk]
            g[0] -= 1
            if g[0] == 0:                 # the group's stacked arrays are gone
                self._used -= g[1]
                del groups[gk]

        def finish(done: dict):
            for key, res in done.items():
                if key in groups:         # the grouped solve failed as a whole
                    for rid in [r for r, v in running.items() if v[2] == key]:
                        record(rid, res)
                elif key in running:
                    record(key, res)

        def admit(now):
            """Take arrived requests that fit (slots, memory) and start them as groups."""
            take = []
            heavy_busy = any(self._heavy(v[0]) for v in running.values())
            i = 0
            while i < len(pending):
                head = pending[i]
                if realtime and head.arrival > now:
                    break
                if self._heavy(head) and heavy_busy:
                    i += 1                    # waits for the running large solve
                    continue
                fp = footprint_bytes(head)
                if not (len(running) + len(take) < self.max_concurrent and self._used + fp <= self.budget):
                    break
                pending.pop(i)
                self._used += fp
                take.append((head, fp))
                heavy_busy = heavy_busy or self._heavy(head)
            by_shape: dict = {}
            for req, fp in take:
                by_shape.setdefault(_shape(req), []).append((req, fp))
            for members in by_shape.values():
                for c in range(0, len(members), self.max_group):
                    chunk = members[c:c + self.max_group]
                    gk = ("group", self.groups)
                    self.groups += 1
                    start = time.perf_counter() - t0
                    reqs = [r for r, _ in chunk]
                    ops = [_operator(r, self.device) for r in reqs]
                    groups[gk] = [len(reqs), float(sum(fp for _, fp in chunk))]
                    for r in reqs:
                        running[r.rid] = (r, start, gk)
                    finish(batch.add(gk, _group_steps(reqs, ops)))
            self.peak_concurrent = max(self.peak_concurrent, len(running))
            self.peak_used = max(self.peak_used, self._used)

        with torch.cuda.device(self.device):
            while pending or len(batch):
                now = time.perf_counter() - t0
                heavy_busy = any(self._heavy(v[0]) for v in running.values())
                waiting = []                  # arrived requests that could start now
                for r in pending:
                    if len(waiting) >= self.min_group or (realtime and r.arrival > now):
                        break
                    if not (heavy_busy and self._heavy(r)):
                        waiting.append(r)
                if waiting and (not running or len(waiting) >= self.min_group
                                or now - waiting[0].arrival >= self.group_wait):
                    admit(now)
                if len(batch):
                    finish(batch.step())
                elif pending and realtime:
                    time.sleep(max(min(pending[0].arrival - (time.perf_counter() - t0), 0.05), 1e-4))
            self.steps = batch.steps
            torch.cuda.synchronize(self.device)
        if self.errors:
            raise RuntimeError(f"{len(self.errors)} request(s) failed: {self.errors[:3]}")
        return sorted(results, key=lambda r: r.rid)


    def _heavy(self, req: SolveRequest) -> bool:
        return req.grid >= self.exclusive_grid


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
