"""Autotuner on the GPU: every candidate it may pick gives the same results, and a
second call reuses the cached choice."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_operator_pipelines_agree_and_tuning_caches(tmp_path, monkeypatch):
    from eigenfns_gb300 import tune
    from eigenfns_gb300.operator import MaxwellOperator
    from eigenfns_gb300.structure import make_structure
    monkeypatch.setenv("EIGENFNS_GB300_TUNE_CACHE", str(tmp_path / "t.json"))
    eps, L, _ = make_structure(64, 32, seed=2)
    op = MaxwellOperator(eps, L, k_frac=(0.1, 0.2, -0.3))
    X = torch.randn(op.vec_shape(6), dtype=torch.complex64, device=op.device)
    outs = []
    for passes, sb in tune.operator_candidates(op):
        op.configure(passes, sb)
        assert op.pipeline == passes
        outs.append(op.theta(X).cpu().numpy())
    ref = outs[-1]
    for o in outs[:-1]:
        assert np.abs(o - ref).max() <= 2e-5 * np.abs(ref).max()
    first = tune.tune_operator(op, 6, reps=1)
    second = tune.tune_operator(op, 6, reps=1)
    assert not first["cached"] and second["cached"]
    assert second["passes"] == first["passes"] and op.pipeline == first["passes"]
    with pytest.raises(ValueError):
        MaxwellOperator(np.ones((6, 6, 6), np.float32), 1.0).configure(3, 0)


def test_gram_schedules_agree(tmp_path, monkeypatch):
    from eigenfns_gb300 import blas, tune
    from eigenfns_gb300._lib import call
    monkeypatch.setenv("EIGENFNS_GB300_TUNE_CACHE", str(tmp_path / "t.json"))
    K = 2 * 48 ** 3
    g = torch.Generator(device="cuda").manual_seed(3)
    A = torch.randn((32, K), dtype=torch.complex64, device="cuda", generator=g)
    B = torch.randn((64, K), dtype=torch.complex64, device="cuda", generator=g)
    ref = (A.to(torch.complex128).conj() @ B.to(torch.complex128).T).cpu().numpy()
    try:
        for kernel, units in tune.GRAM_CANDIDATES:
            tune.apply_gram(32, 64, kernel, units)
            got = blas.gram(A, B).cpu().numpy()
            assert np.abs(got - ref).max() <= 2e-6 * np.abs(ref).max(), (kernel, units)
        res = tune.tune_gram([(32, 64)], K, reps=1)
        assert (32, 64) in res and res[(32, 64)]["kernel"] in (1, 2)
    finally:
        call("ef_tune_reset")
