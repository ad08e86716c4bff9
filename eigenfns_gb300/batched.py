"""Many eigensolves interleaved on one GPU (the batched path).

Each solve is the deflated block LOBPCG of eigenfns_gb300.solver written as a step
generator (solver.lobpcg_steps): the algorithm runs until it needs device data on the
host (residual norms, an SVQB Gram, the Rayleigh-Ritz matrix) and yields those device
tensors, or a request for the fp64 eigendecomposition of one.

The driver here keeps every active solve one request ahead of the host. When a solve
yields, its request is copied to pinned host memory on the stream right away,
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

import numpy as np
import torch

from . import blas, hosteig
from .grouped import GroupResults
from .solver import HostCopy, HostEigh, HostMany, lobpcg_steps


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
    if isinstance(req, HostMany):
        return [_request_to_host(r) for r in req.items]
    if isinstance(req, HostEigh):
        return _EighOnHost(req.A.host if isinstance(req.A, HostCopy) else _pinned_copy(req.A))
    if isinstance(req, tuple):
        return tuple(_pinned_copy(t) for t in req)
    return _pinned_copy(req)


def _host_data(h):
    """What the solve is sent back: numpy copies, or the fp64 eigh it asked for."""
    if isinstance(h, list):
        return [_host_data(x) for x in h]
    if isinstance(h, _EighOnHost):
        A = h.A.numpy()
        return hosteig.eigh_many(A) if A.ndim == 3 else hosteig.eigh(A)
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

    Every solve queues on the caller's stream, so the device runs the solves' work in
    the order the host issued it. (Binding solves to separate streams let small kernels
    of different solves overlap, 7 % faster on the 24-solve mix, but changed some solves'
    iteration counts against the solve run alone, so it is not offered.)"""

    def __init__(self):
        self._active: dict = {}     # key -> _Pending
        self._flags: dict = {}
        self.steps = 0

    def __len__(self) -> int:
        return len(self._active)

    def keys(self):
        return list(self._active)

    def _queue(self, key, gen, req) -> None:
        """Copy the request, then the error flag, to the host behind the solve's work."""
        host = _request_to_host(req)
        flag = self._flags[key]
        _queue_flag(flag)
        self._active[key] = _Pending(gen, host, _record_event(), flag)

    def _drop(self, key) -> None:
        self._active.pop(key, None)
        self._flags.pop(key, None)

    def _advance(self, key, gen, data, finished: dict, first: bool = False) -> None:
        """Resume a solve with `data` up to its next host read and queue that read; results
        of group members reported on the way go to `finished`."""
        try:
            req = next(gen) if first else gen.send(data)
            while isinstance(req, GroupResults):
                finished.update(req.results)
                req = gen.send(None)
        except StopIteration as stop:
            if isinstance(stop.value, GroupResults):
                finished.update(stop.value.results)
            else:
                finished[key] = stop.value
            self._drop(key)
            return
        except Exception as exc:            # surfaced to the caller per solve (or group)
            finished[key] = exc
            self._drop(key)
            return
        self._queue(key, gen, req)

    def add(self, key, gen) -> dict:
        """Start a solve (runs it up to its first host read). Returns what finished without
        reading anything ({key: result}; never for LOBPCG)."""
        self._flags[key] = _new_flag()
        finished: dict = {}
        self._advance(key, gen, None, finished, first=True)
        return finished

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
            self._advance(k, p.gen, _host_data(p.host), finished)
        self.steps += 1
        return finished

    def run(self) -> dict:
        """Step until every solve has finished; returns {key: result}."""
        out = {}
        while self._active:
            out.update(self.step())
        return out


def group_by_shape(ops, ms, guards, max_group: int = 64) -> list:
    """Instances that can share a group (same grid edge, device, block and guard), in
    input order, split into groups of at most max_group: [[instance index, ...], ...]."""
    groups: dict = {}
    for i, op in enumerate(ops):
        groups.setdefault((op.grid_size, str(op.device), int(ms[i]), int(guards[i])), []).append(i)
    out = []
    for members in groups.values():
        out.extend(members[s:s + max_group] for s in range(0, len(members), max_group))
    return out


def lobpcg_batched(ops, nevs, m: int = 32, guard: int = 8, tol: float = 1e-4, maxit: int = 400,
                   seeds=None, grouped: bool = True, max_group: int = 64, **kw) -> list:
    """Solve several operators' lowest eigenpairs together.

    `ops` are MaxwellOperators (any mix of grids and k-points), `nevs` the bands wanted
    from each (an int applies to all); `m`/`guard` may also be per-instance lists.
    With `grouped` (the default) the instances of one shape run as grouped solves
    (eigenfns_gb300.grouped: one launch sequence per iteration for the whole group), the
    groups interleaved by the pipelined driver; otherwise every instance is its own
    interleaved solve. Returns [(eigenvalues, locked vectors, SolveStats)] in the order
    of `ops`, each equal to lobpcg_blocks(op, nev, ...) run alone; raises the first
    failure after the batch.
    """
    from .grouped import lobpcg_group_steps
    n = len(ops)
    per = lambda v: list(v) if isinstance(v, (list, tuple)) else [v] * n
    nevs, ms, guards = per(nevs), per(m), per(guard)
    seeds = per(0 if seeds is None else seeds)
    drv = BatchedSolves()
    out: dict = {}
    members: dict = {}
    if grouped:
        for g, idx in enumerate(group_by_shape(ops, ms, guards, max_group)):
            members[("group", g)] = idx
            i0 = idx[0]
            out.update(drv.add(("group", g), lobpcg_group_steps(
                [ops[i] for i in idx], [nevs[i] for i in idx], keys=idx, m=ms[i0], guard=guards[i0],
                tol=tol, maxit=maxit, seeds=[seeds[i] for i in idx], **kw)))
    else:
        for i, op in enumerate(ops):
            out.update(drv.add(i, lobpcg_steps(op, nevs[i], m=ms[i], guard=guards[i], tol=tol,
                                               maxit=maxit, seed=seeds[i], verbose=False,
                                               check_tc=False, **kw)))
    out.update(drv.run())
    for gk, idx in members.items():          # a group that failed as a whole
        if gk in out:
            for i in idx:
                out.setdefault(i, out[gk])
    res = [out[i] for i in range(n)]
    for r in res:
        if isinstance(r, Exception):
            raise r
    return res
