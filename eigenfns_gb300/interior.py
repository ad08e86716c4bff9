"""Interior-window (bandpass ChebSI) machinery on the GPU.

A drop-in for the production path of eigenfns/interior.py of the reference:
  rr_extract          :37-88   SVQB, X^H Θ X, dead rows +1e8, fp64 host eigh,
                               rotation, normalized Rayleigh quotient, relative
                               residual |Θx - λx| / |Θx|
  gram_chunked        :432-441 / ortho_block_lowmem :444-466 (same values; the
                               device basis needs no row chunking)
  _jackson / _step_coeffs / bandpass_coeffs :312-333
  _apply_cheb_poly    :336-354 fused: each degree is one operator pipeline whose
                               last FFT pass also forms T_{k+1} and Y += c_k T_{k+1}
                               (ef_cheb_first / ef_cheb_step)
  bandpass_subspace   :357-427
  bandpass_subspace_hosted / rr_extract_hosted (:141-238) exist in the reference
  only because a 192^3 basis did not fit a 12 GB card; on GB300 the basis stays
  on the device and the hosted names alias the device versions.
The bake-off methods (folded spectrum, shift-invert MINRES, expansion polish,
interior.py:243-307, 468-754) live in eigenfns_gb300.bakeoff and are reachable
under their reference names from this module as well.
"""
from __future__ import annotations

import time

import numpy as np
import torch

from . import blas, chebcoef
from ._lib import call
from .blas import combine, gram
from .chebyshev import random_block
from .solver import _SVQB_DROP, ortho_block, svqb_coeffs

_BANDPASS_STREAM = 0x425031


def gram_chunked(A, B, rows: int = 8) -> np.ndarray:
    return gram(A, B).cpu().numpy()


def ortho_block_lowmem(X, passes: int = 2, rows: int = 8):
    return ortho_block(X, passes, _SVQB_DROP)


def rr_extract(op, X, theta_chunk: int = 8):
    """Orthonormalize X, Rayleigh-Ritz on Θ, return (lam, Xr, relres) sorted by λ."""
    if isinstance(X, list):
        X = X.pop()
    X = op._as_block(X)
    m = int(X.shape[0])
    X = ortho_block(X)
    HX = op.theta(X)
    A = gram(X, HX).cpu().numpy()
    del HX
    A = (A + A.conj().T) / 2
    dead = np.sqrt(np.maximum(blas.rowdot(X, X).real.cpu().numpy(), 0)) < 0.5
    A[np.diag_indices_from(A)] += np.where(dead, 1e8, 0.0)
    wA, VA = np.linalg.eigh(A)
    Xr = combine(VA.astype(np.complex64), X)
    del X
    Hr = op.theta(Xr)
    xn2 = blas.rowdot(Xr, Xr).real
    lam_d = blas.rowdot(Xr, Hr).real / torch.clamp(xn2, min=1e-30)
    R = blas.residual(Hr, Xr, lam_d)
    st = torch.stack([blas.rowdot(R, R).real, blas.rowdot(Hr, Hr).real, xn2]).cpu().numpy()
    lam = lam_d.cpu().numpy()
    rn = np.sqrt(np.maximum(st[0], 0)) / np.maximum(np.sqrt(np.maximum(st[1], 0)), 1e-30)
    bad = np.sqrt(np.maximum(st[2], 0)) < 0.5
    lam = np.where(bad, np.inf, lam)
    rn = np.where(bad, np.inf, rn)
    blas.raise_on_tc_error("rr_extract")
    return lam, Xr, rn


# The reference's names for the filter coefficients (interior.py:312-333); one
# implementation in chebcoef serves the filters, the count and the KPM analysis.
_jackson = chebcoef.jackson_damping
_step_coeffs = chebcoef.step_below
bandpass_coeffs = chebcoef.bandpass


def _apply_cheb_poly(op, X, coef, lam_max: float):
    """Y = sum_k coef_k T_k(B) X, B = (2Θ - λ_max)/λ_max, unit rows. len(coef)-1 Θ."""
    c = np.asarray(coef, np.float32)
    T0 = op._as_block(X).clone()
    m = int(T0.shape[0])
    T1 = torch.empty_like(T0)
    Y = torch.empty_like(T0)
    s = 2.0 / lam_max
    ws = op.workspace(m)
    st = blas._stream()
    call("ef_cheb_first", op.handle, T0.data_ptr(), T1.data_ptr(), Y.data_ptr(), m, s,
         float(c[0]), float(c[1]), ws.data_ptr(), ws.numel(), st)
    prev, cur = T0, T1
    for k in range(2, len(c)):
        call("ef_cheb_step", op.handle, cur.data_ptr(), prev.data_ptr(), Y.data_ptr(), m, s,
             float(c[k]), ws.data_ptr(), ws.numel(), st)
        prev, cur = cur, prev
    op.n_theta += (len(c) - 1) * m
    del prev, cur
    blas.scale_rows(Y, 1.0 / torch.clamp(blas.row_norms(Y), min=1e-30))
    return Y


def bandpass_subspace(op, lam_lo: float, lam_hi: float, lam_max: float, m: int = 64,
                      degree: int = 2000, max_outer: int = 8, res_tol: float = 1e-4,
                      target_count: int | None = None, chunk: int = 16, theta_chunk: int = 8,
                      seed: int = 0, X0=None, verbose: bool = True):
    """Filtered subspace iteration with the bandpass polynomial (interior.py:357-427)."""
    if X0 is not None:
        if isinstance(X0, list):
            X0 = X0.pop()
        X = op._as_block(X0)
        m = int(X.shape[0])
    else:
        X = random_block(op, m, seed, _BANDPASS_STREAM)
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
        del X
        X = torch.cat(outs, dim=0) if len(outs) > 1 else outs[0]
        del outs
        lam, Xr, rn = rr_extract(op, X, theta_chunk)
        del X
        n_theta += m + m
        inwin = (lam >= lam_lo) & (lam <= lam_hi) & np.isfinite(lam)
        conv = inwin & (rn < res_tol)
        hist.append({"outer": outer, "in_window": int(inwin.sum()), "converged": int(conv.sum()),
                     "median_res_inwin": float(np.median(rn[inwin])) if inwin.any() else np.nan})
        if verbose:
            print(f"  bandpass outer {outer}: in-window {inwin.sum():3d} converged {conv.sum():3d} "
                  f"elapsed {time.perf_counter() - t0:.0f}s", flush=True)
        if target_count is not None and conv.sum() >= target_count:
            break
        if int(conv.sum()) <= best and outer >= 2:
            break
        best = max(best, int(conv.sum()))
        X = Xr
    blas.raise_on_tc_error("bandpass_subspace")
    return Xr, {"method": "bandpass", "degree": degree, "m": m, "lam_window": (lam_lo, lam_hi),
                "theta_applications": n_theta, "wall_seconds": time.perf_counter() - t0,
                "outer_stats": hist, "lam": lam, "res": rn}


# the hosted variants of the reference exist for 12 GB cards; on GB300 they are the device path
rr_extract_hosted = rr_extract
bandpass_subspace_hosted = bandpass_subspace


_BAKEOFF = ("FoldedOperator", "folded_subspace", "minres_batched", "shift_invert_subspace",
            "polish_subspace")


def __getattr__(name):
    """The bake-off methods under their reference names (interior.py:243-754)."""
    if name in _BAKEOFF:
        from . import bakeoff
        return getattr(bakeoff, name)
    raise AttributeError(f"module {__name__!r} has no attribute {name!r}")
