"""Small dense fp64 problems on the GPU (Cholesky-QR coefficients, Hermitian eigh).

The reference solves these on the host with numpy's LAPACK (SVQB and Rayleigh-Ritz,
eigenfns/solver.py:46-66, 113-126, 281-301). Here they can stay on the device, batched
one CTA per problem (ef_cholqr_f64, ef_eigh_f64), which removes a device-to-host round
trip per call and solves many small problems side by side. GB300's fp64 rate is about
1/64 of its fp32 rate, so a single large eigenproblem (n near 96) is still faster on the
host; the solver uses the device Cholesky-QR for the second, well-conditioned SVQB pass.
"""
from __future__ import annotations

import torch

from . import blas
from ._lib import call, load

MAX_N = 96


def _batched(A: torch.Tensor):
    if A.dtype != torch.complex128 or not A.is_cuda:
        raise ValueError("expected a complex128 CUDA tensor")
    if A.dim() == 2:
        A = A[None]
    if A.dim() != 3 or A.shape[1] != A.shape[2]:
        raise ValueError(f"expected (n, n) or (batch, n, n), got {tuple(A.shape)}")
    n = int(A.shape[1])
    if not 1 <= n <= MAX_N:
        raise ValueError(f"n = {n} outside 1..{MAX_N}")
    return A.contiguous(), n


def cholqr_coeffs(G: torch.Tensor, tol: float = 1e-10):
    """(C, status): complex64 C = R^-1 with G = R^H R for each Gram matrix in the batch.
    Pivots at or below tol * max diag are dead directions (zero rows and columns of C,
    so the rotated row is zero, as SVQB's drop); status counts them."""
    squeeze = G.dim() == 2
    G, n = _batched(G)
    b = int(G.shape[0])
    C = torch.empty((b, n, n), dtype=torch.complex64, device=G.device)
    status = torch.empty((b,), dtype=torch.int32, device=G.device)
    call("ef_cholqr_f64", G.data_ptr(), n, b, C.data_ptr(), status.data_ptr(), float(tol),
         blas._stream())
    return (C[0], status[0]) if squeeze else (C, status)


def eigh(A: torch.Tensor):
    """(w, V, status) for each Hermitian matrix of the batch: w ascending, V's columns the
    eigenvectors (the numpy.linalg.eigh convention); status 1 = not converged."""
    squeeze = A.dim() == 2
    A, n = _batched(A)
    b = int(A.shape[0])
    w = torch.empty((b, n), dtype=torch.float64, device=A.device)
    V = torch.empty((b, n, n), dtype=torch.complex128, device=A.device)
    status = torch.empty((b,), dtype=torch.int32, device=A.device)
    ws = blas.workspace(load().ef_eigh_f64_workspace_bytes(n, b), A.device, "eigh")
    call("ef_eigh_f64", A.data_ptr(), n, b, w.data_ptr(), V.data_ptr(), ws.data_ptr(), ws.numel(),
         status.data_ptr(), blas._stream())
    return (w[0], V[0], status[0]) if squeeze else (w, V, status)
