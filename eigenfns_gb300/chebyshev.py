"""Lanczos λ_max, bottom-up ChebSI and the KPM count on the GPU.

A drop-in for eigenfns/chebyshev.py of the reference:
  lanczos_lambda_max  :28-64   max over seeds of theta_max + beta_last
  chebsi_bottom_up    :103-210 bottom-up filtered subspace iteration with locking
  kpm_count_below     :213-267 Jackson-damped step trace; the recurrence and the
                               <z, T_k z> reductions run fused in the operator's
                               last FFT pass (ef_kpm_count_first / _step) with
                               the estimate accumulated on the device in fp64
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import blas, chebcoef
from ._lib import EF_RAND_NORMAL, EF_RAND_RADEMACHER, EF_RAND_RADEMACHER_C, call
from .blas import combine, deflate, gram
from .solver import deflate_chunk_rows, ortho_block

_LANCZOS_STREAM = 0x4C414E
_KPM_COUNT_STREAM = 0x4B504D
_CHEBSI_STREAM = 0x434845


def random_block(op, m: int, seed: int, stream: int, kind: int = EF_RAND_NORMAL) -> torch.Tensor:
    X = torch.empty(op.vec_shape(m), dtype=torch.complex64, device=op.device)
    call("ef_rand_block", op.handle, X.data_ptr(), m, int(seed), int(stream), int(kind),
         blas._stream())
    return X


def lanczos_lambda_max(op, iters: int = 24, seed: int = 0, n_seeds: int = 2, v0=None) -> float:
    """Probable upper bound on λ_max (callers add the 1.05 margin, run_interior.py:112).

    `v0` replaces the seeded start vector (it is masked and normalized)."""
    if n_seeds > 1:
        return max(lanczos_lambda_max(op, iters, seed + 1000 * s, n_seeds=1) for s in range(n_seeds))
    if v0 is None:
        v = random_block(op, 1, seed, _LANCZOS_STREAM)
    else:
        v = op._as_block(v0).clone()
        call("ef_apply_mask", op.handle, v.data_ptr(), 1, blas._stream())
    blas.scale_rows(v, 1.0 / blas.row_norms(v))
    alphas, betas = [], []
    v_prev = None
    beta = 0.0
    for _ in range(iters):
        w = op.theta(v)
        alpha = float(blas.rowdot(v, w).real.item())
        blas.axpby(v, w, -alpha, 1.0)
        if v_prev is not None:
            blas.axpby(v_prev, w, -beta, 1.0)
        beta_new = float(blas.row_norms(w).item())
        alphas.append(alpha)
        betas.append(beta_new)
        if beta_new < 1e-20:
            break
        v_prev = v
        v = blas.scale_rows(w, torch.tensor([1.0 / beta_new], dtype=torch.float64, device=op.device))
        beta = beta_new
    T = np.diag(alphas) + np.diag(betas[:-1], 1) + np.diag(betas[:-1], -1)
    theta = np.linalg.eigvalsh(T)
    return float(theta[-1] + betas[-1])


@dataclass
class ChebStats:
    theta_applications: int = 0
    outer: list = field(default_factory=list)
    lambda_max: float = 0.0
    wall_seconds: float = 0.0


def _cheb_filter_chunk(op, X, degree: int, lam_c: float, lam_max: float):
    """[λ_c, λ_max]-damping filter (chebyshev.py:67-92) with row rescaling every 32."""
    e = (lam_max - lam_c) / 2.0
    c = (lam_max + lam_c) / 2.0
    # Y = (Θ X - c X) / e : recurrence written with axpby on library kernels
    Xk_prev = X.clone()
    Xk = op.theta(X)
    blas.axpby(X, Xk, -c / e, 1.0 / e)
    for j in range(degree - 1):
        Xn = op.theta(Xk)
        blas.axpby(Xk, Xn, -c * 2.0 / e, 2.0 / e)
        blas.axpby(Xk_prev, Xn, -1.0, 1.0)
        Xk_prev, Xk = Xk, Xn
        if (j + 1) % 32 == 0:
            s = Xk.reshape(Xk.shape[0], -1).abs().amax(dim=1).double()
            big = s > 1e30
            if bool(big.any()):
                sc = torch.where(big, 1.0 / torch.clamp(s, min=1e-30), torch.ones_like(s))
                blas.scale_rows(Xk, sc)
                blas.scale_rows(Xk_prev, sc)
    blas.scale_rows(Xk, 1.0 / torch.clamp(blas.row_norms(Xk), min=1e-30))
    return Xk


def chebsi_bottom_up(op, nev: int, guard: int = 48, degree: int = 200, tol: float = 1e-4,
                     max_outer: int = 30, chunk: int = 64, seed: int = 0,
                     lam_max: float | None = None, verbose: bool = True):
    """Lowest `nev` eigenpairs by bottom-up ChebSI with locking (chebyshev.py:103-210)."""
    t0 = time.perf_counter()
    m = nev + guard
    stats = ChebStats()
    if lam_max is None:
        lam_max = 1.05 * lanczos_lambda_max(op)
        stats.theta_applications += 24
    stats.lambda_max = lam_max
    X = ortho_block(random_block(op, m, seed, _CHEBSI_STREAM))
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
            stats.theta_applications += degree * int(piece.shape[0])
        act = torch.cat(outs, dim=0)
        if n_locked:
            act = deflate(act, X[:n_locked].contiguous(), 128)
            act = deflate(act, X[:n_locked].contiguous(), 128)
        act = ortho_block(act)
        Hact = torch.cat([op.theta(act[s:s + chunk]) for s in range(0, act.shape[0], chunk)])
        stats.theta_applications += int(act.shape[0])
        A = gram(act, Hact).cpu().numpy()
        A = (A + A.conj().T) / 2
        dead = np.sqrt(np.maximum(blas.rowdot(act, act).real.cpu().numpy(), 0)) < 0.5
        A[np.diag_indices_from(A)] += np.where(dead, 1e4, 0.0)
        wA, VA = np.linalg.eigh(A)
        C = VA.astype(np.complex64)
        act = combine(C, act)
        Hact = combine(C, Hact)
        lam_act = wA
        R = blas.residual(Hact, act, torch.from_numpy(lam_act).to(op.device))
        rr = blas.rowdot(R, R).real.cpu().numpy()
        hh = blas.rowdot(Hact, Hact).real.cpu().numpy()
        rn = np.sqrt(np.maximum(rr, 0)) / np.maximum(np.sqrt(np.maximum(hh, 0)), 1e-30)
        want = nev - n_locked
        conv_prefix = 0
        for i in range(min(want, len(rn))):
            if rn[i] < tol:
                conv_prefix += 1
            else:
                break
        X = torch.cat([X[:n_locked], act], dim=0)
        lam_full = np.concatenate([locked_vals, lam_act])
        if conv_prefix:
            locked_vals = lam_full[:n_locked + conv_prefix]
            n_locked += conv_prefix
        lam = lam_full
        stats.outer.append({"outer": outer, "locked": n_locked, "lam_c": lam_c,
                            "median_res": float(np.median(rn))})
        if verbose:
            print(f"  outer {outer:2d}: locked {n_locked:4d}/{nev}  lam_c {lam_c:8.4f}", flush=True)
        if n_locked >= nev:
            break
    blas.raise_on_tc_error("chebsi_bottom_up")
    stats.wall_seconds = time.perf_counter() - t0
    return lam[:nev], X[:nev], stats


def step_jackson_coeffs(lam_b: float, lam_max: float, degree: int) -> np.ndarray:
    """Jackson-damped Chebyshev coefficients of 1_{λ<λ_b} (chebyshev.py:232-242)."""
    return chebcoef.damped_step(lam_b, lam_max, degree)


def kpm_count_below(op, lam_b: float, lam_max: float, degree: int = 500, n_probe: int = 30,
                    seed: int = 1, locked=None, probe_kind: str = "real", Z=None):
    """Stochastic #eigenvalues below λ_b: (estimate, standard_error)."""
    coef = step_jackson_coeffs(lam_b, lam_max, degree).astype(np.float32)
    if Z is None:
        kind = EF_RAND_RADEMACHER if probe_kind == "real" else EF_RAND_RADEMACHER_C
        Z = random_block(op, n_probe, seed, _KPM_COUNT_STREAM, kind)
    else:
        Z = op._as_block(Z).clone()
        call("ef_apply_mask", op.handle, Z.data_ptr(), int(Z.shape[0]), blas._stream())
    n_probe = int(Z.shape[0])
    if locked is not None:
        if not isinstance(locked, torch.Tensor):
            locked = torch.from_numpy(np.ascontiguousarray(np.asarray(locked, np.complex64)))
        locked = locked.to(op.device).contiguous()
        cr = deflate_chunk_rows(op.grid_size)
        deflate(Z, locked, cr)
        deflate(Z, locked, cr)
    s = 2.0 / lam_max
    prev = Z.clone()
    cur = torch.empty_like(Z)
    est = torch.zeros((n_probe,), dtype=torch.float64, device=op.device)
    ws = op.workspace(n_probe)
    st = blas._stream()
    call("ef_kpm_count_first", op.handle, Z.data_ptr(), cur.data_ptr(), n_probe, s,
         float(coef[0]), float(coef[1]), est.data_ptr(), ws.data_ptr(), ws.numel(), st)
    for k in range(2, degree + 1):
        call("ef_kpm_count_step", op.handle, cur.data_ptr(), prev.data_ptr(), Z.data_ptr(), n_probe,
             s, float(coef[k]), est.data_ptr(), ws.data_ptr(), ws.numel(), st)
        prev, cur = cur, prev
    op.n_theta += degree * n_probe
    per_probe = est.cpu().numpy()
    blas.raise_on_tc_error("kpm_count_below")
    return float(per_probe.mean()), float(per_probe.std(ddof=1) / np.sqrt(n_probe))
