"""Small, self-contained kernel workloads for profiling (ncu) and quick timing.

    python profile_kernels.py theta --grid 128 --m 2
    python profile_kernels.py gram --ma 32 --mb 32 --grid 128
    python profile_kernels.py gram_tc --ma 32 --mb 32 --grid 128
    python profile_kernels.py rotate --ma 96 --mb 64 --grid 128
    python profile_kernels.py cheb --grid 192 --m 8 --steps 8
    python profile_kernels.py kpm --grid 256 --m 4 --steps 8
    python profile_kernels.py rowstats --ma 32 --mb 32 --grid 128
    python profile_kernels.py rownorms --ma 64 --grid 128
    python profile_kernels.py batched --seeds 16

`batched` runs the 48-instance grouped LOBPCG workload of bench.py (N in 64/216/512 x
--seeds seeds on 32^3/48^3/64^3) twice untimed, once timed, and once under
torch.profiler (CUPTI kernel records, not ncu), and prints the device time per kernel
against the wall time.

Each runs 3 warm-up calls and then --reps timed calls (default 1; CUDA events on
the current stream), printing the mean time; under ncu, skip the warm-up launches
with -s.
Inputs are seeded random blocks and a seeded binary eps grid.
"""
from __future__ import annotations

import argparse

import numpy as np
import torch


def _op(G: int):
    from eigenfns_gb300.operator import MaxwellOperator
    rng = np.random.default_rng(0)
    eps = np.asarray(1.0 + 7.41 * (rng.random((G, G, G)) > 0.78), np.float32)
    return MaxwellOperator(eps, 5.0)


REPS = 1


def _timed(fn, warm: int = 3) -> float:
    """Mean milliseconds per call over REPS calls after `warm` untimed ones."""
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(REPS):
        fn()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / REPS


def _batched(seeds: int) -> None:
    import collections
    import time

    from torch.profiler import ProfilerActivity, profile

    import bench
    from eigenfns_gb300.batched import lobpcg_batched
    from eigenfns_gb300.operator import MaxwellOperator
    from eigenfns_gb300.solver import lobpcg_blocks
    from eigenfns_gb300.structure import bz_kpoint, make_structure
    dev = torch.device("cuda", torch.cuda.current_device())
    inst = []
    for nodes, grid, nev, m, guard in bench.BATCHED_KINDS:
        for j in range(seeds):
            seed = 1000 * nodes + j
            eps, L, _ = make_structure(nodes, grid, seed=seed)
            inst.append((MaxwellOperator(eps, L, k_frac=bz_kpoint(seed), device=dev), nev, m, guard, seed))
    for k in range(len(bench.BATCHED_KINDS)):
        op, nev, m, g, s = inst[k * seeds]
        lobpcg_blocks(op, nev, m=m, guard=g, tol=1e-4, seed=s, verbose=False)

    def run():
        return lobpcg_batched([i[0] for i in inst], [i[1] for i in inst], m=[i[2] for i in inst],
                              guard=[i[3] for i in inst], tol=1e-4, seeds=[i[4] for i in inst])
    run()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    run()
    torch.cuda.synchronize()
    print(f"batched wall {time.perf_counter() - t0:.3f} s")
    with profile(activities=[ProfilerActivity.CPU, ProfilerActivity.CUDA]) as prof:
        t0 = time.perf_counter()
        run()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    agg = collections.defaultdict(lambda: [0, 0.0])
    for e in prof.events():
        if e.device_type == torch.autograd.DeviceType.CUDA:
            a = agg[e.name[:90]]
            a[0] += 1
            a[1] += e.device_time_total
    tot = sum(v[1] for v in agg.values())
    print(f"profiled wall {wall * 1e3:.1f} ms, kernels {tot / 1e3:.1f} ms, "
          f"launches {sum(v[0] for v in agg.values())}")
    for k, v in sorted(agg.items(), key=lambda x: -x[1][1])[:30]:
        print(f"{v[1] / 1e3:9.1f} ms {v[0]:7d} {v[1] / max(v[0], 1):8.1f} us  {k}")
    print(prof.key_averages().table(sort_by="self_cpu_time_total", row_limit=12))


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("kernel", choices=["theta", "precond", "gram", "gram_tc", "rotate", "cheb", "kpm",
                                       "rowstats", "rownorms", "residual", "batched"])
    ap.add_argument("--grid", type=int, default=128)
    ap.add_argument("--m", type=int, default=2)
    ap.add_argument("--ma", type=int, default=32)
    ap.add_argument("--mb", type=int, default=32)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--reps", type=int, default=1, help="timed calls (mean reported)")
    ap.add_argument("--seeds", type=int, default=16, help="batched: seeds per node count")
    a = ap.parse_args(argv)
    if a.kernel == "batched":
        _batched(a.seeds)
        return
    global REPS
    REPS = max(1, a.reps)
    g = torch.Generator(device="cuda").manual_seed(1)
    G = a.grid
    if a.kernel in ("theta", "precond", "cheb", "kpm"):
        op = _op(G)
        X = torch.randn((a.m, 2, G, G, G), dtype=torch.complex64, device="cuda", generator=g)
        Y = torch.empty_like(X)
        if a.kernel == "theta":
            ms = _timed(lambda: op.theta(X, out=Y))
        elif a.kernel == "precond":
            ms = _timed(lambda: op.precondition(X, out=Y))
        elif a.kernel == "cheb":
            from eigenfns_gb300.interior import _apply_cheb_poly
            coef = np.linspace(1.0, 0.1, a.steps + 1)
            ms = _timed(lambda: _apply_cheb_poly(op, X, coef, 4.0e4))
        else:
            from eigenfns_gb300.kpm import kpm_moments
            ms = _timed(lambda: kpm_moments(op, 4.0e4, 2 * a.steps, a.m, Z=X))
        us = 1e3 * ms / a.m
        gbs = (32.0 * G ** 3 * a.m + 4.0 * G ** 3) / (ms * 1e-3) / 1e9
        print(f"{a.kernel} grid {G} m {a.m}: {ms:.3f} ms  ({us:.1f} us/vector, "
              f"{gbs:.0f} GB/s of compulsory operator bytes)")
    else:
        from eigenfns_gb300 import blas
        K = 2 * G ** 3
        A = torch.randn((a.ma, K), dtype=torch.complex64, device="cuda", generator=g)
        B = torch.randn((a.mb, K), dtype=torch.complex64, device="cuda", generator=g)
        if a.kernel == "rowstats":
            ms = _timed(lambda: blas.rowstats(A, B[: a.ma]))
        elif a.kernel == "rownorms":                # rowstats of a block with itself
            ms = _timed(lambda: blas.rowstats(A, A))
        elif a.kernel == "residual":
            lam = torch.rand(a.ma, dtype=torch.float64, device="cuda")
            R = torch.empty_like(A)
            ms = _timed(lambda: blas.residual_norms(B[: a.ma], A, lam, R))
        elif a.kernel == "gram":
            ms = _timed(lambda: blas.gram(A, B))
        elif a.kernel == "gram_tc":
            ms = _timed(lambda: blas.gram_tc(A, B))
        else:
            C = np.random.default_rng(2).standard_normal((a.ma, a.mb)).astype(np.complex64)
            ms = _timed(lambda: blas.rotate(C, A, B))
        rows = {"gram": a.ma + a.mb, "gram_tc": a.ma + a.mb, "rowstats": 2 * a.ma, "rownorms": a.ma,
                "residual": 3 * a.ma}.get(a.kernel, a.ma + a.mb)
        print(f"{a.kernel} {a.ma}x{a.mb} K={K}: {ms:.3f} ms  ({8.0 * K * rows / (ms * 1e-3) / 1e9:.0f} GB/s "
              f"of {rows} rows read or written)")


if __name__ == "__main__":
    main()
