"""Oracle (test infrastructure only): per-mode energy density and participation ratio.

Restates eigenfns/localization.py:23-29 (PR = (sum u)^2 / sum u^2 in voxels,
fraction PR / N_vox) and the energy density u = eps |E|^2 of scripts/run_modes.py:
119-124, with E from the oracle operator's e_realspace.
"""
from __future__ import annotations

import numpy as np


def participation(u) -> dict:
    u = np.asarray(u, np.float64)
    s1 = float(u.sum())
    s2 = float((u * u).sum())
    pr = s1 * s1 / max(s2, 1e-300)
    return {"pr_vox": pr, "pr_fraction": pr / u.size}


def energy_density(op, H, vals) -> np.ndarray:
    """u (m, G, G, G) = eps * sum_c |E_c|^2 for the oracle MaxwellOperator `op`."""
    E = np.asarray(op.e_realspace(H, np.asarray(vals, np.float64)))
    return np.asarray(op.eps_grid, np.float64)[None] * (np.abs(E) ** 2).sum(1)
