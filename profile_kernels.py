"""Small, self-contained kernel workloads for profiling (ncu) and quick timing.

    python profile_kernels.py theta --grid 128 --m 2
    python profile_kernels.py gram --ma 32 --mb 32 --grid 128
    python profile_kernels.py gram_tc --ma 32 --mb 32 --grid 128
    python profile_kernels.py rotate --ma 96 --mb 64 --grid 128
    python profile_kernels.py cheb --grid 192 --m 8 --steps 8
    python profile_kernels.py kpm --grid 256 --m 4 --steps 8
    python profile_kernels.py rowstats --ma 32 --mb 32 --grid 128
    python profile_kernels.py rownorms --ma 64 --grid 128

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


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("kernel", choices=["theta", "precond", "gram", "gram_tc", "rotate", "cheb", "kpm",
                                       "rowstats", "rownorms", "residual"])
    ap.add_argument("--grid", type=int, default=128)
    ap.add_argument("--m", type=int, default=2)
    ap.add_argument("--ma", type=int, default=32)
    ap.add_argument("--mb", type=int, default=32)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--reps", type=int, default=1, help="timed calls (mean reported)")
    a = ap.parse_args(argv)
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
