"""Host logic of the bake-off methods on the CPU: the batched MINRES recurrence
(interior.py:618-687) on diagonal stand-in operators, with the library's per-vector
inner product replaced by a torch one, and the folded diagonal preconditioner's
formula (interior.py:258-269). The GPU runs are in tests/test_gpu_bakeoff.py."""
from __future__ import annotations

from types import SimpleNamespace

import numpy as np
import pytest

torch = pytest.importorskip("torch")

G = 8


def _re_dot_cpu(P, Q):
    return (P.reshape(P.shape[0], -1).conj() * Q.reshape(Q.shape[0], -1)).real.sum(1).to(torch.float64)


class _DiagOp:
    """Θ = diag(D) on (m, 2, G, G, G) blocks; the preconditioner a fixed SPD diagonal."""

    def __init__(self, D, P):
        self.D, self.P = D, P

    def _as_block(self, X):
        return X.contiguous()

    def theta(self, X, out=None):
        return X * self.D

    def precondition(self, X, out=None):
        return X * self.P


def _ops(gapped: bool):
    rng = np.random.default_rng(0)
    D = rng.uniform(0.5, 10.0, (2, G, G, G))
    if gapped:
        D[rng.random(D.shape) > 0.5] += 30.0      # nothing within 10 of the shift 20
    P = 1.0 / (D * rng.uniform(0.8, 1.2, D.shape))
    return _DiagOp(torch.from_numpy(D.astype(np.float32)), torch.from_numpy(P.astype(np.float32)))


def _unit_rhs(m=2, seed=1):
    g = torch.Generator().manual_seed(seed)
    B = torch.randn((m, 2, G, G, G), dtype=torch.complex64, generator=g)
    return B / torch.linalg.vector_norm(B.reshape(m, -1), dim=1)[:, None, None, None, None]


@pytest.mark.parametrize("sigma,gapped,use_precond,tol,bound",
                         [(0.0, False, True, 1e-5, 1e-5), (0.0, False, False, 1e-5, 1e-4),
                          (20.0, True, True, 1e-6, 1e-4), (20.0, True, False, 1e-6, 1e-5)])
def test_minres_recurrence_converges(monkeypatch, sigma, gapped, use_precond, tol, bound):
    from eigenfns_gb300 import bakeoff
    monkeypatch.setattr(bakeoff, "_re_dot", _re_dot_cpu)
    op = _ops(gapped)
    B = _unit_rhs()
    Y, it, nt = bakeoff.minres_batched(op, B, sigma, tol=tol, maxit=400, use_precond=use_precond)
    R = op.theta(Y) - sigma * Y - B
    rel = torch.linalg.vector_norm(R.reshape(2, -1), dim=1).max().item()
    assert rel < bound and it < 400 and it % 4 == 0 and nt >= 2 * it


def test_minres_residual_falls_with_iterations(monkeypatch):
    from eigenfns_gb300 import bakeoff
    monkeypatch.setattr(bakeoff, "_re_dot", _re_dot_cpu)
    op = _ops(True)
    B = _unit_rhs(seed=2)
    rels = []
    for maxit in (4, 12, 40):
        Y, _, _ = bakeoff.minres_batched(op, B, 20.0, tol=1e-12, maxit=maxit, use_precond=False)
        rels.append(torch.linalg.vector_norm((op.theta(Y) - 20.0 * Y - B).reshape(2, -1)).item())
    assert rels[0] > rels[1] > rels[2]


def test_folded_preconditioner_formula():
    """Wang-Zunger folded diagonal 1 / ((kn^2 <1/eps> - σ)^2 + a^2), a^2 = σ^2 by default."""
    from eigenfns_gb300.bakeoff import FoldedOperator
    rng = np.random.default_rng(4)
    kn = torch.from_numpy(rng.uniform(0.0, 9.0, (G, G, G)).astype(np.float32))
    base = SimpleNamespace(basis=SimpleNamespace(kn=kn), grid_size=G, box_size=1.0,
                           dtype=np.complex64, device=torch.device("cpu"), eps_mean_inv=0.4,
                           kn_floor=0.5, _as_block=lambda X: X.contiguous())
    sigma = 3.0
    fop = FoldedOperator(base, sigma)
    kin = kn.double() ** 2 * 0.4
    ref = (1.0 / ((kin - sigma) ** 2 + sigma ** 2)).float()
    assert torch.allclose(fop._fold_diag, ref, rtol=1e-6)
    R = _unit_rhs(3)
    assert torch.equal(fop.precondition(R), R * ref)
    out = torch.empty_like(R)
    assert fop.precondition(R, out=out) is out and torch.equal(out, R * ref)
    assert FoldedOperator(base, sigma, precond_reg=2.0).precond_reg == 2.0
