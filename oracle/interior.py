"""Oracle restatement of the interior-window (bandpass ChebSI) machinery.

TEST INFRASTRUCTURE ONLY (the checker, never the shipped path).

Follows eigenfns/interior.py of the reference:
  rr_extract          :37-88   SVQB, chunk-assembled X^H Θ X, dead rows +1e8,
                               eigh, rotate, NORMALIZED Rayleigh quotient and
                               relative residual |Θx - λx| / |Θx|
  _jackson            :312-316
  _step_coeffs        :319-325
  bandpass_coeffs     :328-333
  _apply_cheb_poly    :336-354 Y = sum_k c_k T_k(B) X, B = 2Θ/λ_max - 1,
                               fp32 coefficients, unit rows at the end
  bandpass_subspace   :357-427 filter -> rr_extract -> in-window counts
  gram_chunked        :432-441
  ortho_block_lowmem  :444-466
"""
from __future__ import annotations

import time

import numpy as np

from .rng import complex_normal
from .solver import _flat, _SVQB_DROP, combine, gram, ortho_block, row_norms, svqb_coeffs, rotate


def gram_chunked(A, B, rows: int = 8):
    m = int(A.shape[0])
    out = np.zeros((m, int(B.shape[0])), np.complex128)
    for s in range(0, m, rows):
        out[s:s + min(rows, m - s)] = gram(A[s:s + rows], B)
    return out


def ortho_block_lowmem(X, passes: int = 2, rows: int = 8):
    for _ in range(passes):
        C, _ = svqb_coeffs(gram_chunked(X, X, rows), _SVQB_DROP)
        X = rotate(C.astype(X.dtype), X)
    return X


def rr_extract(op, X, theta_chunk: int = 8):
    m = int(X.shape[0])
    X = ortho_block_lowmem(X) if m >= 48 else ortho_block(X)
    A = np.zeros((m, m), np.complex128)
    for s in range(0, m, theta_chunk):
        Hc = op.theta(X[s:s + theta_chunk])
        A[:, s:s + Hc.shape[0]] = gram_chunked(X, Hc)
    A = (A + A.conj().T) / 2
    dead = row_norms(X) < 0.5
    A[np.diag_indices_from(A)] += np.where(dead, 1e8, 0.0)
    wA, VA = np.linalg.eigh(A)
    Xr = combine(VA.astype(op.dtype), X)
    lam = np.empty(m)
    rn = np.empty(m)
    for s in range(0, m, theta_chunk):
        Xc = Xr[s:s + theta_chunk]
        Hc = op.theta(Xc)
        xn2 = np.real(np.sum(np.abs(_flat(Xc)) ** 2, axis=1))
        lc = np.real(np.sum(_flat(Xc).conj() * _flat(Hc), axis=1)) / np.maximum(xn2, 1e-30)
        Rc = Hc - lc.astype(op.rdtype)[:, None, None, None, None] * Xc
        lam[s:s + Xc.shape[0]] = lc
        rn[s:s + Xc.shape[0]] = row_norms(Rc) / np.maximum(row_norms(Hc), 1e-30)
    bad = row_norms(Xr) < 0.5
    lam = np.where(bad, np.inf, lam)
    rn = np.where(bad, np.inf, rn)
    return lam, Xr, rn


def _jackson(p: int) -> np.ndarray:
    k = np.arange(p + 1)
    g = ((p - k + 1) * np.cos(np.pi * k / (p + 1))
         + np.sin(np.pi * k / (p + 1)) / np.tan(np.pi / (p + 1)))
    return g / (p + 1)


def _step_coeffs(xb: float, p: int) -> np.ndarray:
    k = np.arange(1, p + 1)
    tb = np.arccos(np.clip(xb, -1.0, 1.0))
    c = np.empty(p + 1)
    c[0] = 1 - tb / np.pi
    c[1:] = -2 * np.sin(k * tb) / (k * np.pi)
    return c


def bandpass_coeffs(lam_lo: float, lam_hi: float, lam_max: float, degree: int) -> np.ndarray:
    x_lo = 2 * lam_lo / lam_max - 1
    x_hi = 2 * lam_hi / lam_max - 1
    return _jackson(degree) * (_step_coeffs(x_hi, degree) - _step_coeffs(x_lo, degree))


def _apply_cheb_poly(op, X, coef, lam_max: float):
    inv_l = 2.0 / lam_max
    c = np.asarray(coef, np.float32)

    def Bx(V):
        return (inv_l * op.theta(V) - V).astype(op.dtype)

    T0 = X
    T1 = Bx(X)
    Y = (c[0] * T0 + c[1] * T1).astype(op.dtype)
    for k in range(2, len(c)):
        T2 = (2.0 * Bx(T1) - T0).astype(op.dtype)
        Y = (Y + c[k] * T2).astype(op.dtype)
        T0, T1 = T1, T2
    ns = 1.0 / np.maximum(row_norms(Y), 1e-30)
    return (Y * ns.astype(op.rdtype)[:, None, None, None, None]).astype(op.dtype)


def random_block(op, m: int, seed: int, stream: int = 0x425031):
    G = op.grid_size
    return (complex_normal(seed, stream, (m, 2, G, G, G)).astype(op.dtype)
            * op.mask[None, None]).astype(op.dtype)


def bandpass_subspace(op, lam_lo: float, lam_hi: float, lam_max: float, m: int = 64,
                      degree: int = 2000, max_outer: int = 8, res_tol: float = 1e-4,
                      target_count: int | None = None, chunk: int = 16,
                      theta_chunk: int = 8, seed: int = 0, X0=None):
    if X0 is not None:
        X = np.asarray(X0, op.dtype)
        m = int(X.shape[0])
    else:
        X = random_block(op, m, seed)
    coef = bandpass_coeffs(lam_lo, lam_hi, lam_max, degree)
    n_theta = 0
    t0 = time.perf_counter()
    hist = []
    best = -1
    lam = Xr = rn = None
    for outer in range(max_outer):
        outs = []
        for s in range(0, X.shape[0], chunk):
            outs.append(_apply_cheb_poly(op, X[s:s + chunk], coef, lam_max))
            n_theta += degree * int(X[s:s + chunk].shape[0])
        X = np.concatenate(outs, axis=0)
        lam, Xr, rn = rr_extract(op, X, theta_chunk)
        n_theta += m + m
        inwin = (lam >= lam_lo) & (lam <= lam_hi) & np.isfinite(lam)
        conv = inwin & (rn < res_tol)
        hist.append({"outer": outer, "in_window": int(inwin.sum()),
                     "converged": int(conv.sum()),
                     "median_res_inwin": float(np.median(rn[inwin])) if inwin.any() else np.nan})
        if target_count is not None and conv.sum() >= target_count:
            break
        if int(conv.sum()) <= best and outer >= 2:
            break
        best = max(best, int(conv.sum()))
        X = Xr
    return Xr, {"method": "bandpass", "degree": degree, "m": m,
                "lam_window": (lam_lo, lam_hi), "theta_applications": n_theta,
                "wall_seconds": time.perf_counter() - t0, "outer_stats": hist,
                "lam": lam, "res": rn}
