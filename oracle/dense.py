"""Dense Θ by columns and dense reference spectra.

TEST INFRASTRUCTURE ONLY.

`dense_theta` follows tests/test_operator.py:16-24 of the reference (apply Θ
to each unit vector); columns are applied in batches instead of one by one.
"""
from __future__ import annotations

import numpy as np


def dense_theta(op, batch: int = 256) -> np.ndarray:
    G = op.grid_size
    n = 2 * G ** 3
    M = np.zeros((n, n), op.dtype)
    for s in range(0, n, batch):
        e = min(batch, n - s)
        I = np.zeros((e, n), op.dtype)
        I[np.arange(e), s + np.arange(e)] = 1.0
        M[:, s:s + e] = op.theta(I.reshape(e, 2, G, G, G)).reshape(e, n).T
    return M


def dense_spectrum(op) -> np.ndarray:
    """Sorted eigenvalues of the Hermitian part, the two Γ zero slots included."""
    M = dense_theta(op).astype(np.complex128)
    return np.sort(np.linalg.eigvalsh((M + M.conj().T) / 2))


def dense_eigh(op):
    M = dense_theta(op).astype(np.complex128)
    w, V = np.linalg.eigh((M + M.conj().T) / 2)
    return w, V
