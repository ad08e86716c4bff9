"""Many eigensolves in lock step on one GPU (the batched path).

Each solve is the deflated block LOBPCG of eigenfns_gb300.solver written as a step
generator (solver.lobpcg_steps): the algorithm runs until it needs device data on the
host (residual norms, an SVQB Gram, the Rayleigh-Ritz matrix) and yields those device
tensors, or a request for the fp64 eigendecomposition of one. The driver here advances
every active solve to its next such point, which queues that solve's kernels on the
shared stream, then copies all the requested tensors to pinned host memory and
synchronizes once for the whole batch, runs the step's eigendecompositions side by
side on host threads, and resumes each solve with its data. Per step the host
therefore waits once for all instances instead of once per instance, the GPU runs the
instances' kernels back to back, and the instances' fp64 eigh calls share the host
cores. Solves may join and leave between steps (continuous batching, see
eigenfns_gb300.serve). A solve's kernels and their order are exactly those of the solve
run alone, so its results are identical alone and in the batch.

Reference: the per-instance algorithm is eigenfns/solver.py:136-382; the reference has
no batched path (its multi-instance runs are separate processes, e.g.
scripts/exp/chain_i6resume.sh).
"""
from __future__ import annotations

import contextlib
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import torch

from . import blas
from .solver import HostEigh, lobpcg_steps

_POOL = None


def _pool() -> ThreadPoolExecutor:
    """Host threads for the solves' fp64 eigh calls (LAPACK releases the GIL)."""
    global _POOL
    if _POOL is None:
        _POOL = ThreadPoolExecutor(max_workers=max(1, min(32, os.cpu_count() or 1)))
    return _POOL


class _EighOnHost:
    __slots__ = ("A",)

    def __init__(self, A):
        self.A = A


def _pinned_copy(t: torch.Tensor) -> torch.Tensor:
    h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    h.copy_(t, non_blocking=True)
    return h


def _request_to_host(req):
    if isinstance(req, HostEigh):
        return _EighOnHost(_pinned_copy(req.A))
    if isinstance(req, tuple):
        return tuple(_pinned_copy(t) for t in req)
    return _pinned_copy(req)


def _numpy(h):
    if isinstance(h, tuple):
        return tuple(x.numpy() for x in h)
    return h.numpy()


class BatchedSolves:
    """Lock-step driver of step generators.

    Each solve is bound to one of `streams` CUDA streams (round robin as solves join), so
    the small kernels of different solves can run side by side on the device while each
    solve's own kernels keep their order (its scratch buffers are per stream); a step
    ends with one device synchronisation."""

    def __init__(self, streams: int = 8):
        self._active: dict = {}     # key -> (generator, pending request)
        self._stream_of: dict = {}
        self._streams = [torch.cuda.Stream() for _ in range(max(1, streams))] if streams > 1 else None
        self._next = 0
        self.steps = 0

    def __len__(self) -> int:
        return len(self._active)

    def keys(self):
        return list(self._active)

    def _ctx(self, key):
        if self._streams is None:
            return contextlib.nullcontext()
        return torch.cuda.stream(self._stream_of[key])

    def add(self, key, gen) -> dict:
        """Start a solve (runs it up to its first host read). Returns {key: result} if it
        finished without reading anything (never for LOBPCG)."""
        if self._streams is not None:
            self._stream_of[key] = self._streams[self._next % len(self._streams)]
            self._next += 1
            # the solve's inputs were made on the caller's stream
            self._stream_of[key].wait_stream(torch.cuda.current_stream())
        try:
            with self._ctx(key):
                self._active[key] = (gen, next(gen))
        except StopIteration as stop:
            self._stream_of.pop(key, None)
            return {key: stop.value}
        return {}

    def step(self) -> dict:
        """One shared host transfer and one resume of every active solve; returns the
        solves that finished in this step as {key: result or the exception raised}."""
        if not self._active:
            return {}
        hosts = {}
        for k, (_, req) in self._active.items():
            with self._ctx(k):
                hosts[k] = _request_to_host(req)
        if self._streams is None:
            torch.cuda.current_stream().synchronize()
        else:
            torch.cuda.synchronize()
        self.steps += 1
        # the step's eigenproblems run side by side on the host threads
        eigh = {k: _pool().submit(np.linalg.eigh, h.A.numpy()) for k, h in hosts.items()
                if isinstance(h, _EighOnHost)}
        if blas.tc_error():
            # a tensor-core pipeline wait ran out in some solve since the last step: every
            # solve in flight may hold invalid data, so all of them fail
            err = RuntimeError("a tensor-core kernel timed out waiting on its pipeline; results invalid")
            done = {k: err for k in self._active}
            for g, _ in self._active.values():
                g.close()
            self._active.clear()
            self._stream_of.clear()
            return done
        finished = {}
        for k in list(self._active):
            gen, _ = self._active[k]
            try:
                data = eigh[k].result() if k in eigh else _numpy(hosts[k])
                with self._ctx(k):
                    self._active[k] = (gen, gen.send(data))
            except StopIteration as stop:
                finished[k] = stop.value
                del self._active[k]
            except Exception as exc:            # surfaced to the caller per solve
                finished[k] = exc
                del self._active[k]
        for k in finished:
            s = self._stream_of.pop(k, None)
            if s is not None:                   # results are used on the caller's stream
                torch.cuda.current_stream().wait_stream(s)
        return finished

    def run(self) -> dict:
        """Step until every solve has finished; returns {key: result}."""
        out = {}
        while self._active:
            out.update(self.step())
        return out


def lobpcg_batched(ops, nevs, m: int = 32, guard: int = 8, tol: float = 1e-4, maxit: int = 400,
                   seeds=None, streams: int = 8, **kw) -> list:
    """Solve several operators' lowest eigenpairs in lock step.

    `ops` are MaxwellOperators (any mix of grids and k-points), `nevs` the bands wanted
    from each (an int applies to all); `m`/`guard` may also be per-instance lists.
    Returns [(eigenvalues, locked vectors, SolveStats)] in the order of `ops`, each equal
    to lobpcg_blocks(op, nev, ...) run alone; raises the first failure after the batch.
    `streams` CUDA streams are shared round robin by the solves (1: the current stream).
    """
    n = len(ops)
    per = lambda v: list(v) if isinstance(v, (list, tuple)) else [v] * n
    nevs, ms, guards = per(nevs), per(m), per(guard)
    seeds = per(0 if seeds is None else seeds)
    drv = BatchedSolves(streams)
    out = {}
    for i, op in enumerate(ops):
        out.update(drv.add(i, lobpcg_steps(op, nevs[i], m=ms[i], guard=guards[i], tol=tol,
                                           maxit=maxit, seed=seeds[i], verbose=False,
                                           check_tc=False, **kw)))
    out.update(drv.run())
    res = [out[i] for i in range(n)]
    for r in res:
        if isinstance(r, Exception):
            raise r
    return res
