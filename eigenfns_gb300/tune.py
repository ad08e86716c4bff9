"""Autotuner for the operator pipeline and the Gram schedules, timed on the running GPU.

What it chooses
  operator  per (grid edge G, block size m): the three-pass pipeline (z / xy-plane / z,
            for the grid edges that have a plan) with a sub-batch workspace of 1, 2, 4, 8
            or 16 vectors, or the five-pass pencil pipeline; applied with
            MaxwellOperator.configure (ef_op_configure).
  Gram      per (ma, mb) at a vector length K: the tensor-core kernel with 1, 2, 3 or 4
            K-chunks per SM, or the CUDA-core split-K kernel; registered with
            ef_tune_gram, which ef_gram consults at every call.

Each candidate runs `warmup` untimed calls and then `reps` timed calls (CUDA events on
the current stream); the lowest mean wins. Choices are stored in a JSON file keyed by
the GPU name, the library version and the shape ($EIGENFNS_GB300_TUNE_CACHE, else
~/.cache/eigenfns_gb300/tune.json), and later processes re-apply them without timing.
The solvers (single and grouped LOBPCG) apply a stored operator choice to their
operators by default (apply_cached), so an operator built after a tuning run gets the
tuned pipeline; autotune=False leaves operators as they are.
The choice of units does not change the Gram's arithmetic; the kernel choice selects
between the mixed-precision (3xTF32) and the plain fp32 Gram, both fp32-class.
"""
from __future__ import annotations

import json
import os
import threading
from pathlib import Path

import torch

from . import blas
from ._lib import call, load

_LOCK = threading.Lock()
GRAM_CANDIDATES = ((1, 1), (1, 2), (1, 3), (1, 4), (2, 0))   # (kernel, units per SM)


def cache_path() -> Path:
    p = os.environ.get("EIGENFNS_GB300_TUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "eigenfns_gb300" / "tune.json"


def _load_cache() -> dict:
    try:
        return json.loads(cache_path().read_text())
    except (OSError, ValueError):
        return {}


def _store(key: str, value: dict) -> None:
    with _LOCK:
        data = _load_cache()
        data[key] = value
        path = cache_path()
        path.parent.mkdir(parents=True, exist_ok=True)
        tmp = path.with_suffix(f".{os.getpid()}.tmp")
        tmp.write_text(json.dumps(data, indent=1, sort_keys=True))
        tmp.replace(path)


def _prefix(device) -> str:
    return f"{torch.cuda.get_device_name(device)}|{load().ef_version().decode()}"


def _time_ms(fn, warmup: int, reps: int) -> float:
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def operator_candidates(op) -> list:
    """(passes, sub-batch bytes) pairs worth timing for this operator."""
    per_vec = 3 * 8 * op.grid_size ** 3
    out = [(5, 0)]
    try:
        op.configure(3, 0)
        out = [(3, k * per_vec + 1) for k in (1, 2, 4, 8, 16)] + out
    except ValueError:
        pass                      # no three-pass plan for this grid edge
    finally:
        op.configure(0, 0)
    return out


def tune_operator(op, m: int, warmup: int = 2, reps: int = 3, use_cache: bool = True) -> dict:
    """Pick and apply the fastest operator pipeline for blocks of m vectors."""
    key = f"{_prefix(op.device)}|op|G={op.grid_size}|m={m}"
    if use_cache:
        hit = _load_cache().get(key)
        if hit is not None:
            op.configure(hit["passes"], hit["subbatch_bytes"])
            return dict(hit, cached=True)
    X = torch.randn(op.vec_shape(m), dtype=torch.complex64, device=op.device)
    Y = torch.empty_like(X)
    timings = []
    for passes, sb in operator_candidates(op):
        op.configure(passes, sb)
        timings.append((_time_ms(lambda: op.theta(X, out=Y), warmup, reps), passes, sb))
    del X, Y
    ms, passes, sb = min(timings)
    op.configure(passes, sb)
    res = {"passes": passes, "subbatch_bytes": sb, "ms": ms,
           "candidates": [[p, b, t] for t, p, b in timings]}
    _store(key, res)
    return dict(res, cached=False)


def apply_cached(op, m: int) -> bool:
    """Apply the operator pipeline an earlier tuning chose for this GPU, grid edge and
    block size, without timing anything; False (the operator left as it is) when the
    cache holds no choice for it."""
    if not hasattr(op, "configure"):
        return False
    hit = _load_cache().get(f"{_prefix(op.device)}|op|G={op.grid_size}|m={m}")
    if hit is None:
        return False
    op.configure(hit["passes"], hit["subbatch_bytes"])
    return True


def apply_gram(ma: int, mb: int, kernel: int, units: int) -> None:
    call("ef_tune_gram", int(ma), int(mb), int(kernel), int(units))


def tune_gram(shapes, K: int, device=None, warmup: int = 2, reps: int = 5,
              use_cache: bool = True) -> dict:
    """Pick and register the fastest Gram schedule for each (ma, mb) at vector length K."""
    device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    out = {}
    cache = _load_cache() if use_cache else {}
    todo = []
    for ma, mb in dict.fromkeys((int(a), int(b)) for a, b in shapes):
        key = f"{_prefix(device)}|gram|{ma}x{mb}|K={K}"
        hit = cache.get(key)
        if hit is not None:
            apply_gram(ma, mb, hit["kernel"], hit["units"])
            out[(ma, mb)] = dict(hit, cached=True)
        else:
            todo.append((ma, mb, key))
    if not todo:
        return out
    mmax = max(max(a, b) for a, b, _ in todo)
    pool = torch.randn((2 * mmax, K), dtype=torch.complex64, device=device)
    for ma, mb, key in todo:
        A, B = pool[:ma], pool[mmax:mmax + mb]
        timings = []
        for kernel, units in GRAM_CANDIDATES:
            apply_gram(ma, mb, kernel, units)
            timings.append((_time_ms(lambda: blas.gram(A, B), warmup, reps), kernel, units))
        ms, kernel, units = min(timings)
        apply_gram(ma, mb, kernel, units)
        res = {"kernel": kernel, "units": units, "ms": ms,
               "candidates": [[k, u, t] for t, k, u in timings]}
        _store(key, res)
        out[(ma, mb)] = dict(res, cached=False)
    del pool
    return out


def lobpcg_gram_shapes(m: int) -> list:
    """The Gram shapes one LOBPCG iteration with block m issues (besides deflation)."""
    return [(m, m), (2 * m, m), (m, 2 * m), (m, 3 * m)]


def autotune(op, m: int, use_cache: bool = True) -> dict:
    """Tune the operator pipeline and LOBPCG's Gram shapes for this operator and block."""
    K = 2 * op.grid_size ** 3
    return {"operator": tune_operator(op, m, use_cache=use_cache),
            "gram": {f"{a}x{b}": v for (a, b), v in
                     tune_gram(lobpcg_gram_shapes(m), K, op.device, use_cache=use_cache).items()}}


def enabled(flag=None) -> bool:
    """Autotuning on request (flag True) or, when flag is None, with EF_AUTOTUNE=1."""
    if flag is not None:
        return bool(flag)
    return os.environ.get("EF_AUTOTUNE", "0") not in ("", "0")
