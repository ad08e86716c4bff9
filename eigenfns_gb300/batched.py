"""Many eigensolves interleaved on one GPU (the batched path).

Each solve is the deflated block LOBPCG of eigenfns_gb300.solver written as a step
generator (solver.lobpcg_steps): the algorithm runs until it needs device data on the
host (residual norms, an SVQB Gram, the Rayleigh-Ritz matrix) and yields those device
tensors, or a request for the fp64 eigendecomposition of one.

The driver here keeps every active solve one request ahead of the host. When a solve
yields, its request is copied to pinned host memory on the solve's stream right away,
followed by a copy of the tensor-core error flag and an event. A step then visits the
solves in order: it waits for that solve's event only, runs the eigendecomposition on
the host if one was asked for, and resumes the solve, which queues its next kernels and
its next request before the driver moves on. While the host works on one solve the GPU
runs what the others queued, so host and device time overlap and no step waits for the
whole device. Solves may join and leave between steps (continuous batching, see
eigenfns_gb300.serve). A solve's kernels and their order are exactly those of the solve
run alone and its host arithmetic is the same, so its results are identical alone and
in the batch.

Reference: the per-instance algorithm is eigenfns/solver.py:136-382; the reference has
no batched path (its multi-instance runs are separate processes, e.g.
scripts/exp/chain_i6resume.sh).
"""
from __future__ import annotations

import contextlib

import numpy as np
import torch

from . import blas
from .solver import HostEigh, lobpcg_steps


class _EighOnHost:
    __slots__ = ("A",)

    def __init__(self, A):
        self.A = A


def _pinned_copy(t: torch.Tensor) -> torch.Tensor:
    h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    h.copy_(t, non_blocking=True)
    return h


def _request_to_host(req):
    """Queue the copy of a request's device tensors to pinned host memory."""
    if isinstance(req, HostEigh):
        return _EighOnHost(_pinned_copy(req.A))
    if isinstance(req, tuple):
        return tuple(_pinned_copy(t) for t in req)
    return _pinned_copy(req)


def _host_data(h):
    """What the solve is sent back: numpy copies, or the fp64 eigh it asked for."""
    if isinstance(h, _EighOnHost):
        return np.linalg.eigh(h.A.numpy())
    if isinstance(h, tuple):
        return tuple(x.numpy() for x in h)
    return h.numpy()


def _new_flag():
    return torch.zeros((1,), dtype=torch.int32, pin_memory=True)


def _queue_flag(flag) -> None:
    blas.tc_error_async(flag)


def _flag_value(flag) -> int:
    return int(flag[0])


def _record_event():
    ev = torch.cuda.Event()
    ev.record()
    return ev


def _wait(ev) -> None:
    ev.synchronize()


class _Pending:
    __slots__ = ("gen", "host", "event", "flag")

    def __init__(self, gen, host, event, flag):
        self.gen, self.host, self.event, self.flag = gen, host, event, flag


class BatchedSolves:
    """Pipelined round-robin driver of step generators.

    `streams` > 1 binds each solve to one of that many CUDA streams (round robin as solves
    join), so that the small kernels of different solves may also run side by side on
    the device; each solve's own kernels keep their order and its scratch buffers are
    per stream. With 1 (the default) every solve queues on the caller's stream."""

    def __init__(self, streams: int = 1):
        self._active: dict = {}     # key -> _Pending
        self._stream_of: dict = {}
        self._flags: dict = {}
        self._streams = [torch.cuda.Stream() for _ in range(streams)] if streams > 1 else None
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

    def _queue(self, key, gen, req) -> None:
        """Copy the request, then the error flag, to the host behind the solve's work."""
        with self._ctx(key):
            host = _request_to_host(req)
            flag = self._flags[key]
            _queue_flag(flag)
            ev = _record_event()
        self._active[key] = _Pending(gen, host, ev, flag)

    def _drop(self, key) -> None:
        self._active.pop(key, None)
        self._flags.pop(key, None)
        s = self._stream_of.pop(key, None)
        if s is not None:                       # results are used on the caller's stream
            torch.cuda.current_stream().wait_stream(s)

    def add(self, key, gen) -> dict:
        """Start a solve (runs it up to its first host read). Returns {key: result} if it
        finished without reading anything (never for LOBPCG)."""
        if self._streams is not None:
            self._stream_of[key] = self._streams[self._next % len(self._streams)]
            self._next += 1
            # the solve's inputs were made on the caller's stream
            self._stream_of[key].wait_stream(torch.cuda.current_stream())
        self._flags[key] = _new_flag()
        try:
            with self._ctx(key):
                req = next(gen)
        except StopIteration as stop:
            self._drop(key)
            return {key: stop.value}
        self._queue(key, gen, req)
        return {}

    def _fail_all(self, finished: dict) -> None:
        # a tensor-core pipeline wait ran out: every solve in flight may hold invalid data
        blas.tc_error()                         # clears the flag (synchronises)
        err = RuntimeError("a tensor-core kernel timed out waiting on its pipeline; results invalid")
        for k in list(self._active):
            self._active[k].gen.close()
            finished[k] = err
            self._drop(k)

    def step(self) -> dict:
        """Resume every active solve once, each as soon as its own request has reached the
        host; returns the solves that finished as {key: result or the exception raised}."""
        finished: dict = {}
        for k in list(self._active):
            p = self._active.get(k)
            if p is None:
                continue
            _wait(p.event)
            if _flag_value(p.flag):
                self._fail_all(finished)
                break
            try:
                data = _host_data(p.host)
                with self._ctx(k):
                    req = p.gen.send(data)
                self._queue(k, p.gen, req)
            except StopIteration as stop:
                finished[k] = stop.value
                self._drop(k)
            except Exception as exc:            # surfaced to the caller per solve
                finished[k] = exc
                self._drop(k)
        self.steps += 1
        return finished

    def run(self) -> dict:
        """Step until every solve has finished; returns {key: result}."""
        out = {}
        while self._active:
            out.update(self.step())
        return out


def lobpcg_batched(ops, nevs, m: int = 32, guard: int = 8, tol: float = 1e-4, maxit: int = 400,
                   seeds=None, streams: int = 1, **kw) -> list:
    """Solve several operators' lowest eigenpairs, interleaved.

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
