"""Served against plain on a request stream of the full serving shape, on one GPU.

    python bench_serve.py [--requests 32 --rate 2.0 --seed 2026 --tol 1e-4]

Requests: Poisson arrivals at --rate per second (seeded); each draws a rod network
with N in {64, 216, 512, 1000} nodes and its grid (32^3, 48^3, 64^3, and 96^3 or 128^3
for N = 1000, either with equal odds), a Bloch k-point uniform in the first Brillouin
zone, and 8-120 lowest bands. The served run admits them by device-memory footprint
under a 160 GB budget (eigenfns_gb300.serve.EigenServer: requests of one shape start
as grouped solves, groups advance in the pipelined batch driver); the plain run
solves the same requests one at a time in arrival order. Both build each request's
structure and operator. Prints one JSON line: throughput, p50/p99 latency per arm,
and the largest eigenvalue difference between the two arms.

The reference's serving stand-in is its detached chain scripts, one solve per process
(scripts/exp/chain_i6resume.sh); it has no served path to time.
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

KINDS = ((64, 32), (216, 48), (512, 64), (1000, 96), (1000, 128))   # (nodes, grid)


def requests(n: int, seed: int, rate_hz: float, tol: float) -> list:
    from eigenfns_gb300.serve import SolveRequest
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    for i in range(n):
        t += rng.exponential(1.0 / rate_hz)
        nodes, grid = KINDS[int(rng.integers(len(KINDS)))]
        k = tuple(float(x) for x in rng.random(3) - 0.5)
        out.append(SolveRequest(rid=i, nodes=nodes, grid=grid, seed=int(rng.integers(1 << 30)),
                                k_frac=k, nev=int(rng.integers(8, 121)), tol=tol, arrival=t))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=32)
    ap.add_argument("--rate", type=float, default=2.0, help="arrivals per second")
    ap.add_argument("--seed", type=int, default=2026)
    ap.add_argument("--tol", type=float, default=1e-4)
    a = ap.parse_args()
    import torch
    from eigenfns_gb300.serve import EigenServer, run_plain, summarize
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    reqs = requests(a.requests, a.seed, a.rate, a.tol)
    run_plain([r for r in reqs if r.grid <= 48][:2], device=dev)      # warm the small-grid kernels
    t0 = time.perf_counter()
    srv = EigenServer(budget_bytes=160e9, max_concurrent=32, device=dev)
    res_s = srv.run(reqs, realtime=True)
    wall_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    res_p = run_plain(reqs, device=dev)
    wall_p = time.perf_counter() - t0
    ss, sp = summarize(res_s, wall_s), summarize(res_p, wall_p)
    diff = max(float(np.abs(x.vals - y.vals).max() / np.abs(y.vals).max()) for x, y in zip(res_s, res_p))
    grids = {g: sum(1 for r in reqs if r.grid == g) for _, g in KINDS}
    print(json.dumps({
        "workload": (f"{len(reqs)} Poisson requests ({a.rate}/s, seed {a.seed}): N in (64, 216, 512, 1000) "
                     f"on 32^3/48^3/64^3/(96^3 or 128^3), random k, 8-120 bands, tol {a.tol}; "
                     "160 GB admission budget, 32 slots"),
        "requests_per_grid": grids, "bands": int(sum(r.nev for r in reqs)),
        "served": ss, "plain": sp, "speedup": ss["modes_per_s"] / sp["modes_per_s"],
        "peak_concurrent": srv.peak_concurrent, "groups": srv.groups,
        "max_rel_diff_served_vs_plain": diff}))


if __name__ == "__main__":
    main()
