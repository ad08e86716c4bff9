"""Oracle restatement of the two-stage (build -> polish) bandpass ChebSI driver.

TEST INFRASTRUCTURE ONLY (the checker, never the shipped path).

Follows scripts/run_interior.py of the reference:
  one_stage         :154-208  per outer: filter every chunk with the stage's
                              degree, rr_extract, in-window/converged counts;
                              the polish stage stops once every in-window pair
                              has converged
  build -> polish   :210-216
  final gate        :218-227  converged in-window pairs sorted by λ
The first build outer starts from a random block through bandpass_subspace
with one outer (:170-177). Checkpoint, CLI and save steps are out of scope.
"""
from __future__ import annotations

import numpy as np

from .interior import _apply_cheb_poly, bandpass_coeffs, bandpass_subspace, rr_extract


def two_stage(op, lam_lo: float, lam_hi: float, lam_max: float, m: int,
              build_degree: int = 3000, build_outers: int = 2,
              polish_degree: int = 12000, polish_outers: int = 4,
              tol: float = 1e-4, chunk: int = 8, theta_chunk: int = 8, seed: int = 0,
              X_init=None):
    history = []
    n_theta = 0

    def one_stage(X, stage_name, degree, first_outer, max_outers):
        nonlocal n_theta
        coef = bandpass_coeffs(lam_lo, lam_hi, lam_max, degree)
        lam = rn = None
        for outer in range(first_outer, max_outers):
            if X is None:
                X, st = bandpass_subspace(op, lam_lo, lam_hi, lam_max, m=m, degree=degree,
                                          max_outer=1, res_tol=tol, chunk=chunk,
                                          theta_chunk=theta_chunk, seed=seed, X0=X_init)
                n_theta += st["theta_applications"]
                lam, rn = st["lam"], st["res"]
            else:
                outs = [_apply_cheb_poly(op, X[s:s + chunk], coef, lam_max)
                        for s in range(0, X.shape[0], chunk)]
                n_theta += degree * int(X.shape[0])
                lam, X, rn = rr_extract(op, np.concatenate(outs, axis=0), theta_chunk)
                n_theta += 2 * m
            inwin = np.isfinite(lam) & (lam >= lam_lo) & (lam <= lam_hi)
            conv = inwin & (rn < tol)
            history.append({"stage": stage_name, "outer": outer,
                            "in_window": int(inwin.sum()), "converged": int(conv.sum())})
            if stage_name == "polish" and inwin.any() and conv.sum() == inwin.sum():
                break
        return X, lam, rn

    X, lam, rn = one_stage(None, "build", build_degree, 0, build_outers)
    X, lam, rn = one_stage(X, "polish", polish_degree, 0, polish_outers)
    inwin = np.isfinite(lam) & (lam >= lam_lo) & (lam <= lam_hi)
    conv = inwin & (rn < tol)
    idx = np.where(conv)[0][np.argsort(lam[conv], kind="stable")]
    return {"vals": lam[idx], "res": rn[idx], "vecs": X[idx], "lam": lam, "rn": rn,
            "n_converged": int(conv.sum()), "n_inwindow_unconverged": int((inwin & ~conv).sum()),
            "theta_applications": n_theta, "history": history}
