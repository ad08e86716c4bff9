"""CUDA-event timing of the library's kernels, for the benchmark's roofline.

Inside `with op_timer() as t:` every Θ / preconditioner application, Gram and
rotation records a pair of CUDA events on the stream it launches on (torch's
current stream) together with its algorithmic bytes and flops, so per-kernel
average durations can be read after the timed region without synchronising
inside it. `theta_timer` is the same recorder (kept for the Θ-only view).
"""
from __future__ import annotations

from collections import defaultdict
from contextlib import contextmanager

import torch

_ACTIVE = None


class OpTimer:
    def __init__(self):
        self.records = defaultdict(list)   # name -> [(start, end, bytes, flops, vectors)]

    def begin(self):
        ev = torch.cuda.Event(enable_timing=True)
        ev.record(torch.cuda.current_stream())
        return ev

    def end(self, name: str, start, nbytes: float, flops: float = 0.0, vectors: int = 0):
        ev = torch.cuda.Event(enable_timing=True)
        ev.record(torch.cuda.current_stream())
        self.records[name].append((start, ev, float(nbytes), float(flops), int(vectors)))

    def summary(self) -> dict:
        torch.cuda.synchronize()
        out = {}
        for name, recs in self.records.items():
            ms = [s.elapsed_time(e) for s, e, _, _, _ in recs]
            nbytes = sum(r[2] for r in recs)
            flops = sum(r[3] for r in recs)
            vecs = sum(r[4] for r in recs)
            tot = sum(ms)
            out[name] = {"calls": len(ms), "total_ms": tot, "bytes": nbytes, "flops": flops,
                         "vectors": vecs, "mean_ms_per_call": tot / max(len(ms), 1),
                         "gbs": nbytes / max(tot, 1e-12) / 1e6,
                         "tflops": flops / max(tot, 1e-12) / 1e9}
        return out


ThetaTimer = OpTimer


def active():
    return _ACTIVE


@contextmanager
def op_timer():
    global _ACTIVE
    prev = _ACTIVE
    _ACTIVE = OpTimer()
    try:
        yield _ACTIVE
    finally:
        _ACTIVE = prev


theta_timer = op_timer
