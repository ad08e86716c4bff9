"""Device fp64 small dense problems against numpy: Cholesky-QR coefficients and the
Hermitian eigendecomposition (the host LAPACK calls of eigenfns/solver.py:46-66,
113-126, 281-301)."""
from __future__ import annotations

import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _herm(rng, b, n):
    M = rng.standard_normal((b, n, n)) + 1j * rng.standard_normal((b, n, n))
    return M + np.conj(np.swapaxes(M, 1, 2))


@pytest.mark.parametrize("n,b", [(1, 1), (7, 3), (32, 4), (48, 2), (96, 1)])
def test_eigh_matches_numpy(n, b):
    from eigenfns_gb300 import dense
    rng = np.random.default_rng(n)
    H = _herm(rng, b, n)
    w, V, st = dense.eigh(torch.from_numpy(H).cuda())
    w, V = w.cpu().numpy(), V.cpu().numpy()
    assert (st.cpu().numpy() == 0).all()
    for i in range(b):
        w0 = np.linalg.eigvalsh(H[i])
        scale = np.abs(w0).max()
        assert np.abs(w[i] - w0).max() <= 1e-12 * scale
        R = np.conj(V[i].T) @ H[i] @ V[i]
        assert np.abs(R - np.diag(w[i])).max() <= 1e-11 * scale
        assert np.abs(np.conj(V[i].T) @ V[i] - np.eye(n)).max() <= 1e-12


def test_eigh_projected_problem_of_a_solve_matches_numpy():
    """A Rayleigh-Ritz matrix as the solver builds it (Gram of a block against Θ)."""
    from eigenfns_gb300 import blas, dense
    from eigenfns_gb300.chebyshev import random_block
    from eigenfns_gb300.operator import MaxwellOperator
    from eigenfns_gb300.structure import make_structure
    eps, L, _ = make_structure(64, 16, seed=4, sub=2)
    op = MaxwellOperator(eps, L)
    X = random_block(op, 24, 5, 0)
    A = blas.gram(X, op.theta(X))
    A = 0.5 * (A + A.conj().T)
    w, V, st = dense.eigh(A)
    w0 = np.linalg.eigvalsh(A.cpu().numpy())
    assert int(st) == 0 and np.abs(w.cpu().numpy() - w0).max() <= 1e-12 * np.abs(w0).max()


def test_cholqr_orthonormalises_and_keeps_the_span(golden):
    from eigenfns_gb300 import blas, dense
    B = torch.from_numpy(golden["la_B"]).cuda()          # the SVQB fixture's input block
    ref = golden["la_ortho"].reshape(B.shape[0], -1)      # the reference's ortho_block(B)
    C, st = dense.cholqr_coeffs(blas.gram(B, B))
    Q = blas.rotate(C, B)
    Qh = Q.reshape(Q.shape[0], -1).to(torch.complex128)
    assert int(st) == 0
    assert (Qh.conj() @ Qh.T - torch.eye(Q.shape[0], device=Q.device)).abs().max() <= 1e-5
    # the same span as the reference's SVQB result: principal angles ~ 0
    qa = np.linalg.qr(Qh.cpu().numpy().T)[0]
    qb = np.linalg.qr(ref.T.astype(np.complex128))[0]
    s = np.linalg.svd(np.conj(qa.T) @ qb, compute_uv=False)
    assert s.min() >= 1 - 1e-5


def test_cholqr_dead_directions_become_zero_rows(golden):
    """A near-dependent row (the SVQB drop fixture's block) and a zero row are dead
    directions: zero rows, the rest orthonormal, as ortho_block's drop at 1e-5
    (solver.py:113-126)."""
    from eigenfns_gb300 import blas, dense
    B = torch.from_numpy(golden["la_Bdep"]).cuda()
    B[4] = 0
    C, st = dense.cholqr_coeffs(blas.gram(B, B), tol=1e-5)
    Q = blas.rotate(C, B)
    norms = blas.row_norms(Q).cpu().numpy()
    assert int(st) >= 2 and norms[4] == 0.0 and norms[3] == 0.0
    live = np.where(norms > 0.5)[0]
    Qh = Q[torch.from_numpy(live).cuda()].reshape(len(live), -1).to(torch.complex128)
    assert (Qh.conj() @ Qh.T - torch.eye(len(live), device=Q.device)).abs().max() <= 1e-4


def test_timing_report():
    """Times the device routines against numpy on the host (printed, not asserted)."""
    from eigenfns_gb300 import dense
    rng = np.random.default_rng(1)
    for n, b in ((96, 1), (32, 1), (48, 48)):
        H = torch.from_numpy(_herm(rng, b, n)).cuda()
        dense.eigh(H)
        torch.cuda.synchronize()
        t = time.perf_counter()
        dense.eigh(H)
        torch.cuda.synchronize()
        dev = time.perf_counter() - t
        Hh = H.cpu().numpy()
        t = time.perf_counter()
        for i in range(b):
            np.linalg.eigh(Hh[i])
        host = time.perf_counter() - t
        print(f"eigh n={n} batch={b}: device {dev * 1e3:.2f} ms, host numpy {host * 1e3:.2f} ms")
