"""Every public driver that runs the tensor-core Gram or rotation reports a timed-out
pipeline wait as RuntimeError instead of returning its (invalid) results.

The device flag cannot be raised without breaking a kernel, so the host read of
it (eigenfns_gb300.blas.tc_error) is replaced by one that reports a timeout; each
driver then runs a tiny 8^3 problem and must raise.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def op8():
    from eigenfns_gb300.operator import MaxwellOperator
    rng = np.random.default_rng(3)
    eps = np.asarray(1.0 + 7.57 * (rng.random((8, 8, 8)) > 0.7), np.float32)
    return MaxwellOperator(eps, 1.0)


def _block(op, m):
    from eigenfns_gb300.chebyshev import random_block
    return random_block(op, m, 11, 0)


DRIVERS = {
    "lobpcg_blocks": lambda op: __import__("eigenfns_gb300.solver", fromlist=["x"]).lobpcg_blocks(
        op, 4, m=6, guard=2, tol=1e-3, maxit=5, verbose=False),
    "rr_extract": lambda op: __import__("eigenfns_gb300.interior", fromlist=["x"]).rr_extract(
        op, _block(op, 6)),
    "bandpass_subspace": lambda op: __import__("eigenfns_gb300.interior", fromlist=["x"]).bandpass_subspace(
        op, 10.0, 20.0, 400.0, m=6, degree=20, max_outer=1, verbose=False),
    "two_stage": lambda op: __import__("eigenfns_gb300.run_interior", fromlist=["x"]).two_stage(
        op, 10.0, 20.0, 6, lam_max=400.0, build_degree=20, build_outers=1, polish_degree=20,
        polish_outers=1),
    "chebsi_bottom_up": lambda op: __import__("eigenfns_gb300.chebyshev", fromlist=["x"]).chebsi_bottom_up(
        op, 3, guard=3, degree=10, max_outer=1, lam_max=400.0, verbose=False),
    "kpm_count_below": lambda op: __import__("eigenfns_gb300.chebyshev", fromlist=["x"]).kpm_count_below(
        op, 15.0, 400.0, degree=10, n_probe=3),
    "folded_subspace": lambda op: __import__("eigenfns_gb300.interior", fromlist=["x"]).folded_subspace(
        op, 15.0, 2, m=6, guard=2, maxit=3, verbose=False),
    "shift_invert_subspace": lambda op: __import__("eigenfns_gb300.interior", fromlist=["x"]).shift_invert_subspace(
        op, 15.0, m=6, max_outer=1, inner_maxit=5, verbose=False),
    "polish_subspace": lambda op: __import__("eigenfns_gb300.interior", fromlist=["x"]).polish_subspace(
        op, _block(op, 6), 10.0, 20.0, 400.0, max_sweeps=1, strip_degree=10, verbose=False),
}


@pytest.mark.parametrize("name", sorted(DRIVERS))
def test_driver_raises_on_tensor_core_timeout(op8, name, monkeypatch):
    from eigenfns_gb300 import blas
    monkeypatch.setattr(blas, "tc_error", lambda: 1)
    with pytest.raises(RuntimeError, match="tensor-core"):
        DRIVERS[name](op8)
