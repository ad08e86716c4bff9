"""The interior-window methods that lost the reference's bake-off, on the GPU path.

eigenfns/interior.py keeps three alternatives to the bandpass filter beside its
production path; they are here with the same names, arguments and return values:

  FoldedOperator / folded_subspace  :243-307  LOBPCG on (Θ - σ)^2, with the
                                    Wang-Zunger diagonal preconditioner
                                    a^2 / ((kn^2 <1/eps> - σ)^2 + a^2) or MPB's
                                    transverse projection applied twice
  minres_batched                    :618-687  preconditioned MINRES for
                                    (Θ - σ) Y = B, one recurrence per vector
  shift_invert_subspace             :690-754  subspace iteration on (Θ - σ)^-1
                                    through chunked MINRES, Rayleigh-Ritz on Θ
  polish_subspace                   :468-613  preconditioned-residual expansion of
                                    window Ritz pairs with a continuity selection
                                    and a periodic low-degree bandpass strip

Θ, the preconditioner, the per-vector inner products (ef_rowstats, fp64 sums) and
the Gram/rotation work of the polish step run on the library's kernels. The MINRES
recurrences update their vectors with fp32 element-wise arithmetic, as the reference
does (a Krylov recurrence's attainable accuracy follows the rounding of these
updates, so they do not go through the 3xTF32 tensor-core rotation); the per-vector
MINRES scalars stay on the device in float64 (the reference keeps them in float32),
and the convergence test reads them every fourth step, as the reference does.
Random starting blocks come from ef_rand_block (the reference draws them from
jax.random, which cannot be reproduced bit for bit outside JAX).
"""
from __future__ import annotations

import time

import numpy as np
import torch

from . import blas
from .blas import combine, gram, rotate
from .chebyshev import random_block
from .interior import _apply_cheb_poly, bandpass_coeffs, rr_extract
from .solver import ortho_block

_SHIFT_INVERT_STREAM = 0x534931


class FoldedOperator:
    """(Θ - σ)^2 with a folded diagonal preconditioner (interior.py:243-284).

    Quacks like MaxwellOperator for `solver.lobpcg_blocks`: `theta`, `precondition`,
    `basis`, `grid_size`, the block shape and the random-block handle. One `theta`
    is two Θ applications (counted in `n_theta`).
    """

    def __init__(self, op, sigma: float, precond_reg: float | None = None):
        self.op = op
        self.sigma = float(sigma)
        self.basis = op.basis
        self.grid_size = op.grid_size
        self.box_size = op.box_size
        self.dtype = op.dtype
        self.device = op.device
        self.eps_mean_inv = op.eps_mean_inv
        self.kn_floor = op.kn_floor
        if precond_reg is None:
            precond_reg = self.sigma ** 2
        self.precond_reg = float(precond_reg)
        self.precond_kind = "wz"      # "wz" diagonal | "psq" transverse projection twice
        kin = op.basis.kn.to(torch.float64) ** 2 * op.eps_mean_inv
        self._fold_diag = (1.0 / ((kin - self.sigma) ** 2 + self.precond_reg)).to(torch.float32)
        self.n_theta = 0

    @property
    def handle(self):
        return self.op.handle

    def vec_shape(self, m: int):
        return self.op.vec_shape(m)

    def _as_block(self, X) -> torch.Tensor:
        return self.op._as_block(X)

    def workspace(self, m: int) -> torch.Tensor:
        return self.op.workspace(m)

    def theta(self, X, out: torch.Tensor | None = None) -> torch.Tensor:
        """(Θ - σ)^2 X = Θ(ΘX) - 2σ ΘX + σ^2 X."""
        X = self.op._as_block(X)
        self.n_theta += 2 * int(X.shape[0])
        s = self.sigma
        Y = self.op.theta(X)
        if out is None or out.data_ptr() == X.data_ptr() or out.data_ptr() == Y.data_ptr():
            Z = self.op.theta(Y)
        else:
            Z = self.op.theta(Y, out=out)
        blas.axpby(Y, Z, -2.0 * s, 1.0)
        blas.axpby(X, Z, s * s, 1.0)
        if out is not None and Z.data_ptr() != out.data_ptr():
            out.copy_(Z)
            return out
        return Z

    def precondition(self, R, target: float = 0.0, out: torch.Tensor | None = None) -> torch.Tensor:
        R = self.op._as_block(R)
        if self.precond_kind == "psq":
            Y = self.op.precondition(self.op.precondition(R))
            if out is not None:
                out.copy_(Y)
                return out
            return Y
        if out is None:
            out = torch.empty_like(R)
        return torch.mul(R, self._fold_diag, out=out)


def folded_subspace(op, sigma: float, nev: int, m: int = 64, guard: int = 14, tol: float = 1e-3,
                    maxit: int = 400, theta_chunk: int = 8, seed: int = 0,
                    precond_reg: float | None = None, log_every: int = 0, verbose: bool = True):
    """LOBPCG on (Θ - σ)^2 (interior.py:287-307); returns (subspace, stats dict).

    `tol` is on the folded residual; `mu` are the folded eigenvalues (λ - σ)^2.
    """
    from .solver import lobpcg_blocks
    fop = FoldedOperator(op, sigma, precond_reg=precond_reg)
    t0 = time.perf_counter()
    vals, vecs, st = lobpcg_blocks(fop, nev, m=m, guard=guard, tol=tol, maxit=maxit,
                                   theta_chunk=theta_chunk, seed=seed, verbose=verbose,
                                   log_every=log_every, locked_storage="host")
    wall = time.perf_counter() - t0
    blas.raise_on_tc_error("folded_subspace")
    return vecs, {"method": "folded", "sigma": sigma, "mu": np.asarray(vals),
                  "theta_applications": fop.n_theta, "wall_seconds": wall,
                  "outer_stats": st.rounds}


def _bc(a: torch.Tensor) -> torch.Tensor:
    """Per-vector float64 scalars as float32 factors broadcast over (m, 2, G, G, G)."""
    return a.to(torch.float32)[:, None, None, None, None]


def _re_dot(P: torch.Tensor, Q: torch.Tensor) -> torch.Tensor:
    """Re <p_i, q_i> per vector, float64 on the device."""
    return blas.rowstats(P, Q)[:, 0]


def minres_batched(op, B, sigma: float, tol: float = 1e-3, maxit: int = 200,
                   use_precond: bool = True):
    """Solve (Θ - σ) Y = B per vector by preconditioned MINRES (interior.py:618-687).

    Returns (Y, iterations, n_theta). The preconditioner is the transverse projection
    (SPD, ≈ Θ^-1); each vector stops contributing once |η| < tol γ_1, but the batch
    iterates until all have (checked every fourth step), as in the reference. The
    Θ count charges a preconditioner application 2/3 of a Θ, as the reference does.
    """
    B = op._as_block(B)
    m = int(B.shape[0])
    dev = B.device
    n_theta = 0
    n_precond = 0

    def precond(V):
        nonlocal n_precond
        if not use_precond:
            return V.clone()
        n_precond += int(V.shape[0])
        return op.precondition(V)

    X = torch.zeros_like(B)
    v_old = torch.zeros_like(B)
    v = B.clone()
    z = precond(v)
    gamma = torch.sqrt(torch.clamp(_re_dot(z, v), min=1e-38))
    gamma_old = torch.ones_like(gamma)
    eta = gamma.clone()
    gamma1 = gamma.clone()
    zeros = torch.zeros(m, dtype=torch.float64, device=dev)
    s_old, s = zeros.clone(), zeros.clone()
    c_old, c = torch.ones_like(zeros), torch.ones_like(zeros)
    w = torch.zeros_like(B)
    w_old = torch.zeros_like(B)
    it_used = 0
    for j in range(maxit):
        zt = z * _bc(1.0 / gamma)
        Az = op.theta(zt)
        Az.sub_(zt, alpha=sigma)                      # (Θ - σ) zt
        n_theta += m
        delta = _re_dot(Az, zt)
        v_new = Az - v * _bc(delta / gamma) - v_old * _bc(gamma / gamma_old)
        del Az
        z_new = precond(v_new)
        gamma_new = torch.sqrt(torch.clamp(_re_dot(z_new, v_new), min=1e-38))
        a0 = c * delta - c_old * s * gamma
        a1 = torch.sqrt(a0 * a0 + gamma_new * gamma_new)
        a2 = s * delta + c_old * c * gamma
        a3 = s_old * gamma
        c_new = a0 / a1
        s_new = gamma_new / a1
        w_new = (zt - w_old * _bc(a3) - w * _bc(a2)) * _bc(1.0 / a1)
        X.add_(w_new * _bc(c_new * eta))
        eta = -s_new * eta
        v_old, v, z = v, v_new, z_new
        gamma_old, gamma = gamma, gamma_new
        s_old, s, c_old, c = s, s_new, c, c_new
        w_old, w = w, w_new
        it_used = j + 1
        if (j + 1) % 4 == 0:
            r = (eta.abs() / gamma1).cpu().numpy()
            if (r < tol).all():
                break
    return X, it_used, n_theta + (2 * n_precond) // 3


def shift_invert_subspace(op, sigma: float, m: int = 64, max_outer: int = 12,
                          inner_tol: float = 1e-2, inner_maxit: int = 200, res_tol: float = 1e-4,
                          lam_window: tuple | None = None, target_count: int | None = None,
                          chunk: int = 8, theta_chunk: int = 8, seed: int = 0,
                          verbose: bool = True):
    """Subspace iteration on (Θ - σ)^-1 through batched MINRES (interior.py:690-754).

    Each outer: Y = (Θ - σ)^-1 X per chunk, then orthonormalisation and
    Rayleigh-Ritz on Θ (rr_extract) with residual bookkeeping. Stops at
    `target_count` converged pairs, or once the converged count stops growing
    after the fourth outer. Returns (X_ritz, stats dict).
    """
    X = random_block(op, m, seed, _SHIFT_INVERT_STREAM)
    X = ortho_block(X)
    n_theta = 0
    t0 = time.perf_counter()
    hist = []
    best = -1
    lam = Xr = rn = None
    for outer in range(max_outer):
        outs, iters = [], []
        for s in range(0, int(X.shape[0]), chunk):
            Y, it, nt = minres_batched(op, X[s:s + chunk], sigma, tol=inner_tol, maxit=inner_maxit)
            outs.append(Y)
            iters.append(it)
            n_theta += nt
        del X
        X = torch.cat(outs, dim=0)
        del outs
        lam, Xr, rn = rr_extract(op, X, theta_chunk)
        del X
        n_theta += 2 * m
        if lam_window:
            inwin = (lam >= lam_window[0]) & (lam <= lam_window[1]) & np.isfinite(lam)
        else:
            inwin = np.isfinite(lam)
        conv = inwin & (rn < res_tol)
        hist.append({"outer": outer, "inner_iters": iters, "in_window": int(inwin.sum()),
                     "converged": int(conv.sum()),
                     "median_res_inwin": float(np.median(rn[inwin])) if inwin.any() else np.nan})
        if verbose:
            print(f"  shift-invert outer {outer}: inner {iters} in-window {inwin.sum():3d} "
                  f"converged {conv.sum():3d} med-res {hist[-1]['median_res_inwin']:.1e} "
                  f"elapsed {time.perf_counter() - t0:.0f}s", flush=True)
        if target_count is not None and conv.sum() >= target_count:
            break
        if int(conv.sum()) <= best and outer >= 3:
            break
        best = max(best, int(conv.sum()))
        X = Xr
    blas.raise_on_tc_error("shift_invert_subspace")
    return Xr, {"method": "shift_invert", "sigma": sigma, "m": m, "theta_applications": n_theta,
                "wall_seconds": time.perf_counter() - t0, "outer_stats": hist,
                "lam": lam, "res": rn}


def polish_subspace(op, X, lam_lo: float, lam_hi: float, lam_max: float, max_sweeps: int = 8,
                    res_tol: float = 1e-4, strip_degree: int = 300, strip_every: int = 2,
                    strip_w: bool = False, theta_chunk: int = 8, verbose: bool = True):
    """Drive window Ritz pairs to `res_tol` by preconditioned-residual expansion
    (interior.py:468-613). Returns (X, lam, res, stats).

    Each sweep: W = mask · P(ΘX - λX) for all pairs (dead rows get λ = 0), W made
    orthogonal to X (two passes) and orthonormal, Rayleigh-Ritz on span[X, W], and
    the m pairs kept by continuity (weight in the old X block ≥ 0.7 first, then by
    distance to the window); every `strip_every` sweeps the basis is re-filtered by
    a degree-`strip_degree` bandpass. `X` may be a one-element list (emptied).
    """
    if isinstance(X, list):
        X = X.pop()
    X = op._as_block(X)
    m = int(X.shape[0])
    coef = bandpass_coeffs(lam_lo, lam_hi, lam_max, strip_degree)
    n_theta = 0
    t0 = time.perf_counter()
    hist = []
    lam, X, rn = rr_extract(op, X, theta_chunk)
    n_theta += 2 * m
    for sweep in range(max_sweeps):
        conv = np.isfinite(lam) & (rn < res_tol) & (lam >= lam_lo) & (lam <= lam_hi)
        inwin = np.isfinite(lam) & (lam >= lam_lo) & (lam <= lam_hi)
        med = float(np.median(rn[inwin])) if inwin.any() else None
        if verbose:
            print(f"  polish sweep {sweep}: in-window {int(inwin.sum()):3d} converged "
                  f"{int(conv.sum()):3d} med-res {med if med is not None else np.nan:.1e} "
                  f"elapsed {time.perf_counter() - t0:.0f}s", flush=True)
        hist.append({"sweep": sweep, "in_window": int(inwin.sum()), "converged": int(conv.sum()),
                     "med_res": med})
        if inwin.any() and conv.sum() == inwin.sum():
            break
        # residuals of all pairs (fixed shape), preconditioned and masked
        lam_d = torch.from_numpy(np.where(np.isfinite(lam), lam, 0.0)).to(X.device)
        HX = op.theta(X)
        R = blas.residual(HX, X, lam_d)
        del HX
        W = op.precondition(R, out=R)
        from ._lib import call
        call("ef_apply_mask", op.handle, W.data_ptr(), m, blas._stream())
        n_theta += 2 * m
        if strip_w:
            W = _apply_cheb_poly(op, W, coef, lam_max)
            n_theta += strip_degree * m
        for _ in range(2):
            rotate(gram(X, W).to(torch.complex64), X, W, -1)
        W = ortho_block(W)
        # Rayleigh-Ritz on span[X, W]
        S = torch.cat([X, W], dim=0)
        del W
        HS = op.theta(S)
        n_theta += 2 * m
        A = gram(S, HS).cpu().numpy()
        del HS
        A = (A + A.conj().T) / 2
        rownorm = np.sqrt(np.maximum(blas.rowstats(S, S)[:, 2].cpu().numpy(), 0.0))
        A[np.diag_indices_from(A)] += np.where(rownorm < 0.5, 1e8, 0.0)
        wA, VA = np.linalg.eigh(A)
        # continuity selection: refinements carry their weight in the old X block
        cen = 0.5 * (lam_lo + lam_hi)
        half = 0.5 * (lam_hi - lam_lo)
        score = np.maximum(np.abs(wA - cen) - half, 0.0)
        xw = (np.abs(VA[:m, :]) ** 2).sum(axis=0)
        score = score + np.where(xw >= 0.7, 0.0, 1e3)
        keep = np.argsort(score, kind="stable")[:m]
        keep = keep[np.argsort(wA[keep])]
        X = combine(VA[:, keep].astype(np.complex64), S)
        del S
        if strip_every and (sweep + 1) % strip_every == 0:
            outs = [_apply_cheb_poly(op, X[s:s + 16], coef, lam_max) for s in range(0, m, 16)]
            n_theta += strip_degree * m
            X = torch.cat(outs, dim=0)
            del outs
        lam, X, rn = rr_extract(op, X, theta_chunk)
        n_theta += 2 * m
    blas.raise_on_tc_error("polish_subspace")
    return X, lam, rn, {"method": "polish", "theta_applications": n_theta,
                        "wall_seconds": time.perf_counter() - t0, "sweeps": hist}
