"""Oracle restatement of the KPM moment recurrence and its CPU analysis.

TEST INFRASTRUCTURE ONLY (the checker, never the shipped path).

Follows the reference's
  scripts/exp/exp_kpm_dos.py:125-163   probes z masked at |k+G| > 0, T_0 = z,
      T_1 = Bz with B = 2Θ/λ_max - 1; then for k = 1..p/2:
      T_{k+1} = 2 B T_k - T_{k-1},
      μ_2k = 2<T_k,T_k> - μ_0,  μ_2k+1 = 2<T_{k+1},T_k> - μ_1
  scripts/exp/exp_kpm_analyze.py:22-70 jackson, step_coeffs, counting,
      dos_curve, smearing_width
"""
from __future__ import annotations

import numpy as np

from .rng import rademacher


def _dots(A, B):
    fa = A.reshape(A.shape[0], -1)
    fb = B.reshape(B.shape[0], -1)
    return np.real(np.sum(fa.conj().astype(np.complex128) * fb, axis=1))


def kpm_moments(op, lam_max: float, degree: int, probes: int, seed: int = 7,
                chunk: int | None = None, probe_kind: str = "real", Z=None) -> np.ndarray:
    """Per-probe moments (probes, 2*(degree//2)+2) in fp64."""
    G = op.grid_size
    half = degree // 2
    n_mom = 2 * half + 2
    mom = np.zeros((probes, n_mom), np.float64)
    chunk = chunk or probes
    inv_l = 2.0 / lam_max

    def Bx(V):
        return (inv_l * op.theta(V) - V).astype(op.dtype)

    for s in range(0, probes, chunk):
        c = min(chunk, probes - s)
        Zc = rademacher(seed, s, (c, 2, G, G, G), probe_kind) if Z is None else Z[s:s + c]
        Zc = (np.asarray(Zc).astype(op.dtype) * op.mask[None, None]).astype(op.dtype)
        t0v, t1v = Zc, Bx(Zc)
        mu0 = _dots(t0v, t0v)
        mu1 = _dots(t0v, t1v)
        mom[s:s + c, 0], mom[s:s + c, 1] = mu0, mu1
        for k in range(1, half + 1):
            t2v = (2.0 * Bx(t1v) - t0v).astype(op.dtype)
            mom[s:s + c, 2 * k] = 2.0 * _dots(t1v, t1v) - mu0
            mom[s:s + c, 2 * k + 1] = 2.0 * _dots(t2v, t1v) - mu1
            t0v, t1v = t1v, t2v
    return mom


def jackson(p):
    k = np.arange(p + 1)
    g = ((p - k + 1) * np.cos(np.pi * k / (p + 1))
         + np.sin(np.pi * k / (p + 1)) / np.tan(np.pi / (p + 1)))
    return g / (p + 1)


def step_coeffs(xb, p):
    k = np.arange(1, p + 1)
    tb = np.arccos(np.clip(xb, -1.0, 1.0))
    c = np.empty(p + 1)
    c[0] = 1 - tb / np.pi
    c[1:] = -2 * np.sin(k * tb) / (k * np.pi)
    return c


def counting(mom, lam_max, lams, degree=None):
    p = (mom.shape[1] - 1) if degree is None else degree
    g = jackson(p)
    xs = (2.0 * np.asarray(lams) - lam_max) / lam_max
    est = np.empty((mom.shape[0], len(xs)))
    for j, xb in enumerate(xs):
        est[:, j] = mom[:, :p + 1] @ (step_coeffs(xb, p) * g)
    return est.mean(0), est.std(0, ddof=1) / np.sqrt(mom.shape[0]), est


def dos_curve(mom, lam_max, n_pts=4000, degree=None):
    p = (mom.shape[1] - 1) if degree is None else degree
    g = jackson(p)
    mu = mom.mean(0)[:p + 1] * g
    theta = (np.arange(n_pts) + 0.5) * np.pi / n_pts
    x = np.cos(theta)
    T = np.cos(np.outer(np.arange(p + 1), theta))
    rho_x = (mu[0] + 2 * (mu[1:] @ T[1:])) / (np.pi * np.sin(theta))
    lam = (x + 1) * lam_max / 2
    rho_lam = rho_x * 2 / lam_max
    order = np.argsort(lam)
    return lam[order], rho_lam[order]


def smearing_width(lam, lam_max, degree):
    x = np.clip(2 * lam / lam_max - 1, -1 + 1e-12, 1 - 1e-12)
    return np.pi / degree * np.sqrt(1 - x ** 2) * lam_max / 2
