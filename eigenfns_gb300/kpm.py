"""KPM density-of-states moments on the GPU, and their CPU analysis.

`kpm_moments` runs the recurrence of scripts/exp/exp_kpm_dos.py:125-163 of the
reference: probes z masked at |k+G| > 0, T_0 = z, T_1 = B z with
B = 2Θ/λ_max - 1, then T_{k+1} = 2 B T_k - T_{k-1} for k = 1..p/2 with the
doubling identities μ_2k = 2<T_k,T_k> - μ_0 and μ_2k+1 = 2<T_{k+1},T_k> - μ_1.
Each step is one operator pipeline whose last FFT pass forms T_{k+1} and the two
inner products (fp64 partial sums, reduced on the device), so no scalar crosses
to the host until the whole moment table is done; the reference copies both
dots to the host every step.

The analysis helpers restate scripts/exp/exp_kpm_analyze.py:22-70 (CPU numpy,
post-processing of the moments).
"""
from __future__ import annotations

import numpy as np
import torch

from . import blas
from ._lib import EF_RAND_RADEMACHER, EF_RAND_RADEMACHER_C, call
from .chebyshev import random_block


def kpm_moments(op, lam_max: float, degree: int, probes: int, seed: int = 7,
                chunk: int | None = None, probe_kind: str = "real", Z=None) -> np.ndarray:
    """Per-probe moments, fp64 (probes, 2*(degree//2)+2)."""
    half = degree // 2
    n_mom = 2 * half + 2
    chunk = chunk or probes
    s = 2.0 / lam_max
    mom = torch.zeros((probes, n_mom), dtype=torch.float64, device=op.device)
    kind = EF_RAND_RADEMACHER if probe_kind == "real" else EF_RAND_RADEMACHER_C
    st = blas._stream()
    for s0 in range(0, probes, chunk):
        c = min(chunk, probes - s0)
        if Z is None:
            T0 = random_block(op, c, seed, s0, kind)
        else:
            T0 = op._as_block(Z[s0:s0 + c]).clone()
            call("ef_apply_mask", op.handle, T0.data_ptr(), c, st)
        T1 = torch.empty_like(T0)
        ws = op.workspace(c)
        msub = mom[s0:s0 + c]
        call("ef_kpm_first", op.handle, T0.data_ptr(), T1.data_ptr(), c, s, msub.data_ptr(), n_mom,
             ws.data_ptr(), ws.numel(), st)
        prev, cur = T0, T1
        for k in range(1, half + 1):
            call("ef_kpm_step", op.handle, cur.data_ptr(), prev.data_ptr(), c, s, k, msub.data_ptr(),
                 n_mom, ws.data_ptr(), ws.numel(), st)
            prev, cur = cur, prev
        op.n_theta += c * (half + 1)
    return mom.cpu().numpy()


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
    """N(λ) per probe -> (mean, se, per-probe) over thresholds `lams`."""
    p = (mom.shape[1] - 1) if degree is None else degree
    g = jackson(p)
    xs = (2.0 * np.asarray(lams) - lam_max) / lam_max
    est = np.empty((mom.shape[0], len(xs)))
    for j, xb in enumerate(xs):
        est[:, j] = mom[:, :p + 1] @ (step_coeffs(xb, p) * g)
    return est.mean(0), est.std(0, ddof=1) / np.sqrt(mom.shape[0]), est


def dos_curve(mom, lam_max, n_pts=4000, degree=None):
    """Jackson-damped DOS on a Chebyshev-Gauss λ grid."""
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
