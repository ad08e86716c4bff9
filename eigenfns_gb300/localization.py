"""Per-mode energy density and participation ratio on the GPU.

u(r) = eps(r) |E(r)|^2 with E the real-space field of a mode (the reference's
run_modes.py:119-124 computes it band by band after the solve), and the
participation ratio PR = (sum u)^2 / sum u^2 in voxels, with the participation
fraction PR / N_vox (eigenfns/localization.py:23-29). The field, the density and
both sums are produced by the library (e_realspace passes plus one fused
map-and-reduce kernel); only the two fp64 sums per mode come back to the host.
"""
from __future__ import annotations

import numpy as np
import torch

from . import blas
from ._lib import call, load


def _as_vals(vals, n):
    v = np.asarray(vals.cpu() if isinstance(vals, torch.Tensor) else vals, np.float64).reshape(-1)
    if v.size != n:
        raise ValueError(f"{v.size} eigenvalues for {n} modes")
    return v


def energy_density(op, H, vals, chunk: int = 8, keep: bool = True):
    """(u, sums): u (m,G,G,G) float32 on the device (None when keep=False) and
    sums (m, 2) float64 = (sum u, sum u^2) per mode."""
    X = op._as_block(H)
    m = int(X.shape[0])
    G = op.grid_size
    lam = _as_vals(vals, m)
    u = torch.empty((m, G, G, G), dtype=torch.float32, device=op.device) if keep else None
    sums = torch.empty((m, 2), dtype=torch.float64, device=op.device)
    ws = blas.workspace(load().ef_energy_workspace_bytes(op.handle, min(chunk, m)), op.device, "energy")
    for s in range(0, m, chunk):
        e = min(m, s + chunk)
        E = op.e_realspace(X[s:e], lam[s:e])
        call("ef_energy_density", op.handle, E.data_ptr(), u[s:e].data_ptr() if keep else None,
             sums[s:e].data_ptr(), e - s, ws.data_ptr(), ws.numel(), blas._stream())
        del E
    return u, sums.cpu().numpy()


def participation(u) -> dict:
    """PR metrics of one non-negative density field (any normalisation)."""
    if isinstance(u, torch.Tensor):
        t = u.to(torch.float64)
        s1, s2, n = float(t.sum()), float((t * t).sum()), int(t.numel())
    else:
        a = np.asarray(u, np.float64)
        s1, s2, n = float(a.sum()), float((a * a).sum()), int(a.size)
    pr = s1 * s1 / max(s2, 1e-300)
    return {"pr_vox": pr, "pr_fraction": pr / n}


def mode_participation(op, H, vals, chunk: int = 8) -> list:
    """participation() of every mode's energy density without keeping the densities."""
    _, sums = energy_density(op, H, vals, chunk=chunk, keep=False)
    n = op.grid_size ** 3
    out = []
    for s1, s2 in sums:
        pr = s1 * s1 / max(s2, 1e-300)
        out.append({"pr_vox": pr, "pr_fraction": pr / n})
    return out
