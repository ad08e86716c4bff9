"""Two-stage bandpass ChebSI (build -> polish) on the GPU.

The solver logic of scripts/run_interior.py of the reference without its CLI,
file output or GPU-busy guard:
  one_stage         :154-208  per outer: filter every chunk with the stage's
                              degree, rr_extract, in-window / converged counts;
                              the polish stage stops once every in-window pair
                              has converged
  build -> polish   :210-216
  final gate        :218-227  converged in-window pairs sorted by λ; in-window
                              pairs that did not converge are returned apart
λ_max defaults to 1.05 x Lanczos (:111-113). `checkpoint`, when given, is
called after every outer with (X, stage, outer, n_theta, lam_max, history),
the content of the reference's rolling interior_state.npz (:116-121).
"""
from __future__ import annotations

import time

import numpy as np
import torch

from . import blas
from .chebyshev import lanczos_lambda_max
from .interior import _apply_cheb_poly, bandpass_coeffs, bandpass_subspace, rr_extract


def two_stage(op, lam_lo: float, lam_hi: float, m: int, lam_max: float = 0.0,
              build_degree: int = 3000, build_outers: int = 2, polish_degree: int = 12000,
              polish_outers: int = 4, tol: float = 1e-4, chunk: int = 8, theta_chunk: int = 8,
              seed: int = 0, X_init=None, checkpoint=None, resume_state=None,
              verbose: bool = False) -> dict:
    t_start = time.perf_counter()
    n_theta = 0
    history = []
    if lam_max <= 0:
        lam_max = 1.05 * lanczos_lambda_max(op)
        n_theta += 48
    stage, outer0, X0 = "build", 0, None
    if resume_state is not None:
        X0 = resume_state["X"]
        stage = str(resume_state["stage"])
        outer0 = int(resume_state["outer"]) + 1
        n_theta = int(resume_state["n_theta"])
        lam_max = float(resume_state["lam_max"])
        history = list(resume_state.get("history", []))

    def one_stage(X, stage_name, degree, first_outer, max_outers, lam=None, rn=None):
        """Outers of one stage; (lam, rn) are the previous stage's Ritz values, returned
        as they are when the stage runs no outer."""
        nonlocal n_theta
        coef = bandpass_coeffs(lam_lo, lam_hi, lam_max, degree)
        for outer in range(first_outer, max_outers):
            t0 = time.perf_counter()
            if X is None:
                X, st = bandpass_subspace(op, lam_lo, lam_hi, lam_max, m=m, degree=degree,
                                          max_outer=1, res_tol=tol, chunk=chunk,
                                          theta_chunk=theta_chunk, seed=seed, X0=X_init,
                                          verbose=False)
                n_theta += st["theta_applications"]
                lam, rn = st["lam"], st["res"]
            else:
                outs = []
                for s in range(0, X.shape[0], chunk):
                    outs.append(_apply_cheb_poly(op, X[s:s + chunk], coef, lam_max))
                    n_theta += degree * int(X[s:s + chunk].shape[0])
                del X
                Xf = torch.cat(outs, dim=0) if len(outs) > 1 else outs[0]
                del outs
                lam, X, rn = rr_extract(op, [Xf], theta_chunk)
                n_theta += 2 * m
            inwin = np.isfinite(lam) & (lam >= lam_lo) & (lam <= lam_hi)
            conv = inwin & (rn < tol)
            rec = {"stage": stage_name, "outer": outer, "in_window": int(inwin.sum()),
                   "converged": int(conv.sum()),
                   "med_res_inwin": float(np.median(rn[inwin])) if inwin.any() else None,
                   "outer_seconds": time.perf_counter() - t0,
                   "elapsed": time.perf_counter() - t_start}
            history.append(rec)
            if verbose:
                print(f"  {stage_name} outer {outer}: in-window {rec['in_window']:3d} "
                      f"converged {rec['converged']:3d} [{rec['outer_seconds']:.1f}s]", flush=True)
            if checkpoint is not None:
                checkpoint(X, stage_name, outer, n_theta, lam_max, history)
            if stage_name == "polish" and inwin.any() and conv.sum() == inwin.sum():
                break
        return X, lam, rn

    X, lam, rn = X0, None, None
    if stage == "build":
        X, lam, rn = one_stage(X, "build", build_degree, outer0, build_outers)
        outer0 = 0
    X, lam, rn = one_stage(X, "polish", polish_degree, outer0, polish_outers, lam, rn)
    if lam is None:
        raise ValueError("two_stage ran no outer: give build_outers or polish_outers > 0")
    inwin = np.isfinite(lam) & (lam >= lam_lo) & (lam <= lam_hi)
    conv = inwin & (rn < tol)
    unconv = inwin & ~conv
    idx = np.where(conv)[0][np.argsort(lam[conv], kind="stable")]
    uidx = np.where(unconv)[0][np.argsort(lam[unconv], kind="stable")]
    dev_idx = torch.from_numpy(idx).to(X.device)
    blas.raise_on_tc_error("two_stage")
    return {"vals": lam[idx], "res": rn[idx], "vecs": X.index_select(0, dev_idx),
            "unconverged_vals": lam[uidx], "unconverged_res": rn[uidx],
            "lam": lam, "rn": rn, "lam_max": lam_max, "n_converged": int(conv.sum()),
            "n_inwindow_unconverged": int(unconv.sum()), "theta_applications": int(n_theta),
            "history": history, "wall_seconds": time.perf_counter() - t_start}
