"""CUDA-event timing of the operator pipeline, for the benchmark's roofline.

Inside `with theta_timer() as t:` every MaxwellOperator.theta call records a
pair of CUDA events on the stream it launches on (torch's current stream) and
its vector count, so the average duration of the fused Θ pipeline can be read
after the timed region without synchronising inside it.
"""
from __future__ import annotations

from contextlib import contextmanager

import torch

_ACTIVE = None


class ThetaTimer:
    def __init__(self):
        self.records = []   # (start_event, end_event, m, grid)

    def begin(self):
        ev = torch.cuda.Event(enable_timing=True)
        ev.record(torch.cuda.current_stream())
        return ev

    def end(self, start, m: int, grid: int):
        ev = torch.cuda.Event(enable_timing=True)
        ev.record(torch.cuda.current_stream())
        self.records.append((start, ev, int(m), int(grid)))

    def summary(self):
        torch.cuda.synchronize()
        ms = [s.elapsed_time(e) for s, e, _, _ in self.records]
        vecs = [m for _, _, m, _ in self.records]
        return {"calls": len(ms), "total_ms": float(sum(ms)), "vectors": int(sum(vecs)),
                "mean_ms_per_call": float(sum(ms) / max(len(ms), 1)),
                "mean_vectors_per_call": float(sum(vecs) / max(len(vecs), 1))}


def active():
    return _ACTIVE


@contextmanager
def theta_timer():
    global _ACTIVE
    prev = _ACTIVE
    _ACTIVE = ThetaTimer()
    try:
        yield _ACTIVE
    finally:
        _ACTIVE = prev
