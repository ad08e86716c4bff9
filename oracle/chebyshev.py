"""Oracle restatement of Lanczos λ_max, bottom-up ChebSI and the KPM count.

TEST INFRASTRUCTURE ONLY (the checker, never the shipped path).

Follows eigenfns/chebyshev.py of the reference:
  lanczos_lambda_max  :28-64   max over seeds of theta_max + beta_last
  _cheb_filter_chunk  :67-92   [λ_c, λ_max]-damping recurrence, rescale every 32
  chebsi_bottom_up    :103-210 filter, deflate, SVQB, RR, lock converged prefix
  kpm_count_below     :213-267 Jackson-damped step trace with ±1 probes
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from .rng import complex_normal, rademacher
from .solver import (_flat, combine, deflate, deflate_chunk_rows, gram,
                     ortho_block, row_norms)


def lanczos_lambda_max(op, iters: int = 24, seed: int = 0, n_seeds: int = 2,
                       v0=None) -> float:
    if n_seeds > 1:
        return max(lanczos_lambda_max(op, iters, seed + 1000 * s, n_seeds=1)
                   for s in range(n_seeds))
    G = op.grid_size
    if v0 is None:
        v0 = complex_normal(seed, 0x4C414E, (1, 2, G, G, G))
    v = np.asarray(v0).astype(op.dtype) * op.mask[None, None]
    v = (v / np.linalg.norm(_flat(v))).astype(op.dtype)
    alphas, betas = [], []
    v_prev = None
    beta = 0.0
    for _ in range(iters):
        w = op.theta(v)
        alpha = float(np.real(np.sum(_flat(v).conj() * _flat(w))))
        w = w - alpha * v - (beta * v_prev if v_prev is not None else 0.0)
        w = w.astype(op.dtype)
        beta_new = float(np.linalg.norm(_flat(w)))
        alphas.append(alpha)
        betas.append(beta_new)
        if beta_new < 1e-20:
            break
        v_prev = v
        v = (w / beta_new).astype(op.dtype)
        beta = beta_new
    T = np.diag(alphas) + np.diag(betas[:-1], 1) + np.diag(betas[:-1], -1)
    theta = np.linalg.eigvalsh(T)
    return float(theta[-1] + betas[-1])


def _cheb_filter_chunk(op, X, degree: int, lam_c: float, lam_max: float):
    e = (lam_max - lam_c) / 2.0
    c = (lam_max + lam_c) / 2.0
    Y = ((op.theta(X) - c * X) / e).astype(op.dtype)
    Xk_prev, Xk = X, Y
    for j in range(degree - 1):
        Xn = ((op.theta(Xk) - c * Xk) * (2.0 / e) - Xk_prev).astype(op.dtype)
        Xk_prev, Xk = Xk, Xn
        if (j + 1) % 32 == 0:
            s = np.max(np.abs(_flat(Xk)), axis=1)
            sc = np.where(s > 1e30, 1.0 / np.maximum(s, 1e-30), 1.0)
            scale = sc.astype(op.rdtype)[:, None, None, None, None]
            Xk = (Xk * scale).astype(op.dtype)
            Xk_prev = (Xk_prev * scale).astype(op.dtype)
    ns = 1.0 / np.maximum(row_norms(Xk), 1e-30)
    return (Xk * ns.astype(op.rdtype)[:, None, None, None, None]).astype(op.dtype)


@dataclass
class ChebStats:
    theta_applications: int = 0
    outer: list = field(default_factory=list)
    lambda_max: float = 0.0
    wall_seconds: float = 0.0


def chebsi_bottom_up(op, nev: int, guard: int = 48, degree: int = 200, tol: float = 1e-4,
                     max_outer: int = 30, chunk: int = 64, seed: int = 0,
                     lam_max: float | None = None, verbose: bool = False):
    t0 = time.perf_counter()
    m = nev + guard
    G = op.grid_size
    stats = ChebStats()
    if lam_max is None:
        lam_max = 1.05 * lanczos_lambda_max(op)
        stats.theta_applications += 24
    stats.lambda_max = lam_max
    X = (complex_normal(seed, 0x434845, (m, 2, G, G, G)).astype(op.dtype)
         * op.mask[None, None]).astype(op.dtype)
    X = ortho_block(X)
    n_locked = 0
    locked_vals = np.empty((0,))
    lam = None
    for outer in range(max_outer):
        if lam is None:
            lam_c = lam_max / 50.0
        else:
            hi = lam[min(m - 1, nev + guard // 2 - 1)]
            lam_c = float(min(hi * 1.1, lam_max / 4))
        act = X[n_locked:]
        outs = []
        for s in range(0, act.shape[0], chunk):
            piece = act[s:s + chunk]
            outs.append(_cheb_filter_chunk(op, piece, degree, lam_c, lam_max))
            stats.theta_applications += degree * piece.shape[0]
        act = np.concatenate(outs, axis=0)
        if n_locked:
            act = deflate(act, X[:n_locked])
            act = deflate(act, X[:n_locked])
        act = ortho_block(act)
        Hact = np.concatenate([op.theta(act[s:s + chunk]) for s in range(0, act.shape[0], chunk)])
        stats.theta_applications += act.shape[0]
        A = np.asarray(gram(act, Hact)).astype(np.complex128)
        A = (A + A.conj().T) / 2
        dead = row_norms(act) < 0.5
        A[np.diag_indices_from(A)] += np.where(dead, 1e4, 0.0)
        wA, VA = np.linalg.eigh(A)
        C = VA.astype(op.dtype)
        act = combine(C, act)
        Hact = combine(C, Hact)
        lam_act = wA
        R = Hact - lam_act.astype(op.rdtype)[:, None, None, None, None] * act
        rn = row_norms(R) / np.maximum(row_norms(Hact), 1e-30)
        want = nev - n_locked
        conv_prefix = 0
        for i in range(min(want, len(rn))):
            if rn[i] < tol:
                conv_prefix += 1
            else:
                break
        X = np.concatenate([X[:n_locked], act], axis=0)
        lam_full = np.concatenate([locked_vals, lam_act])
        if conv_prefix:
            locked_vals = lam_full[:n_locked + conv_prefix]
            n_locked += conv_prefix
        lam = lam_full
        stats.outer.append({"outer": outer, "locked": n_locked, "lam_c": lam_c,
                            "median_res": float(np.median(rn))})
        if n_locked >= nev:
            break
    stats.wall_seconds = time.perf_counter() - t0
    return lam[:nev], X[:nev], stats


def step_jackson_coeffs(lam_b: float, lam_max: float, degree: int) -> np.ndarray:
    """Jackson-damped Chebyshev coefficients of 1_{λ<λ_b} (chebyshev.py:232-242)."""
    xb = (2 * lam_b - lam_max) / lam_max
    ks = np.arange(degree + 1)
    tb = np.arccos(np.clip(xb, -1, 1))
    mu = np.empty(degree + 1)
    mu[0] = 1 - tb / np.pi
    mu[1:] = -2 * np.sin(ks[1:] * tb) / (ks[1:] * np.pi)
    g = ((degree - ks + 1) * np.cos(np.pi * ks / (degree + 1))
         + np.sin(np.pi * ks / (degree + 1)) / np.tan(np.pi / (degree + 1)))
    g /= (degree + 1)
    return mu * g


def kpm_count_below(op, lam_b: float, lam_max: float, degree: int = 500,
                    n_probe: int = 30, seed: int = 1, locked=None,
                    probe_kind: str = "real", Z=None):
    G = op.grid_size
    coef = step_jackson_coeffs(lam_b, lam_max, degree).astype(np.float32)
    if Z is None:
        Z = rademacher(seed, 0x4B504D, (n_probe, 2, G, G, G), probe_kind)
    n_probe = Z.shape[0]
    Z = (np.asarray(Z).astype(op.dtype) * op.mask[None, None]).astype(op.dtype)
    if locked is not None:
        cr = deflate_chunk_rows(G)
        Z = deflate(Z, locked, cr)
        Z = deflate(Z, locked, cr)

    def Bx(V):
        return ((2.0 / lam_max) * op.theta(V) - V).astype(op.dtype)

    T0, T1 = Z, Bx(Z)
    zf = _flat(Z)
    est = coef[0] * np.real(np.sum(zf.conj() * _flat(T0), axis=1))
    est = est + coef[1] * np.real(np.sum(zf.conj() * _flat(T1), axis=1))
    for k in range(2, degree + 1):
        T2 = (2.0 * Bx(T1) - T0).astype(op.dtype)
        est = est + coef[k] * np.real(np.sum(zf.conj() * _flat(T2), axis=1))
        T0, T1 = T1, T2
    per_probe = np.asarray(est, np.float64)
    return float(per_probe.mean()), float(per_probe.std(ddof=1) / np.sqrt(n_probe))
