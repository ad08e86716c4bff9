"""KPM density-of-states moments on the GPU, and their CPU analysis.

`kpm_moments` runs the recurrence of scripts/exp/exp_kpm_dos.py:125-163 of the
reference: probes z masked at |k+G| > 0, T_0 = z, T_1 = B z with
B = 2Θ/λ_max - 1, then T_{k+1} = 2 B T_k - T_{k-1} for k = 1..p/2 with the
doubling identities μ_2k = 2<T_k,T_k> - μ_0 and μ_2k+1 = 2<T_{k+1},T_k> - μ_1.
Each step is one operator pipeline whose last FFT pass forms T_{k+1} and the two
inner products (fp64 partial sums, reduced on the device), so no scalar crosses
to the host until the whole moment table is done; the reference copies both
dots to the host every step.

The analysis helpers (`counting`, `dos_curve`, `smearing_width`) give the
results of scripts/exp/exp_kpm_analyze.py:39-64 from the kernel polynomial
method's formulas (Weiße et al., Rev. Mod. Phys. 78, 275 (2006), II.C-II.D):
the counting function is a damped step expansion contracted with the moments of
every probe at once, and the DOS on the Chebyshev-Gauss nodes is one DCT-III of
the damped moments (orders above the node count folded back by the cosine's
symmetries), CPU numpy post-processing of the moments.
"""
from __future__ import annotations

import numpy as np
import torch

from . import blas
from ._lib import EF_RAND_RADEMACHER, EF_RAND_RADEMACHER_C, call
from . import chebcoef
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


def jackson(p: int) -> np.ndarray:
    """Jackson damping factors g_0..g_p (exp_kpm_analyze.py:22-26)."""
    return chebcoef.jackson_damping(p)


def step_coeffs(xb: float, p: int) -> np.ndarray:
    """Undamped coefficients of 1{x < xb} on [-1, 1] (exp_kpm_analyze.py:29-36)."""
    return chebcoef.step_below(xb, p)


def counting(mom, lam_max, lams, degree=None):
    """Counting function N(λ) = Σ_k g_k μ_k c_k(x_λ) for every probe and threshold.

    Returns (mean over probes, standard error of the mean, per-probe estimates
    (probes, len(lams))), as exp_kpm_analyze.py:39-48 does.
    """
    mom = np.asarray(mom, np.float64)
    p = (mom.shape[1] - 1) if degree is None else int(degree)
    g = chebcoef.jackson_damping(p)
    xs = np.atleast_1d(chebcoef.unit_interval(lams, lam_max))
    filt = np.stack([g * chebcoef.step_below(x, p) for x in xs], axis=1)   # (p+1, n_lams)
    est = mom[:, :p + 1] @ filt
    n = mom.shape[0]
    return est.mean(0), est.std(0, ddof=1) / np.sqrt(n), est


def _fold_orders(mu: np.ndarray, n: int) -> np.ndarray:
    """DCT-III input x_0..x_{n-1} with x_0 + 2 Σ_m x_m cos(m θ_j) = μ_0 + 2 Σ_k μ_k cos(k θ_j)
    on the n nodes θ_j = π(j + 1/2)/n. There cos(k θ_j) is 4n-periodic in k, changes
    sign under k -> k + 2n, is odd about k = n (zero at k = n), so orders k >= n fold
    back onto 0..n-1."""
    w = np.full(mu.size, 2.0)
    w[0] = 1.0
    k = np.arange(mu.size)
    r = k % (4 * n)
    sign = np.where(r < 2 * n, 1.0, -1.0)
    r = np.where(r < 2 * n, r, r - 2 * n)
    wa = sign * w * mu                      # weighted terms, before folding
    full = np.zeros(n)                      # Σ of weighted terms per folded order
    low = r < n
    high = (r > n)
    np.add.at(full, r[low], wa[low])
    np.add.at(full, 2 * n - r[high], -wa[high])
    x = full / 2.0
    x[0] = full[0]
    return x


def dos_curve(mom, lam_max, n_pts=4000, degree=None):
    """Jackson-damped density of states on n_pts Chebyshev-Gauss nodes (probe mean).

    ρ(x_j) = [g_0 μ_0 + 2 Σ_k g_k μ_k T_k(x_j)] / (π sqrt(1 - x_j^2)), evaluated as
    one DCT-III; returned as (λ ascending, ρ(λ)) with ρ(λ) = ρ(x) 2/λ_max
    (exp_kpm_analyze.py:51-64).
    """
    from scipy.fft import dct
    mom = np.asarray(mom, np.float64)
    p = (mom.shape[1] - 1) if degree is None else int(degree)
    mu = mom.mean(0)[:p + 1] * chebcoef.jackson_damping(p)
    coef = _fold_orders(mu, n_pts)
    theta = np.pi * (np.arange(n_pts) + 0.5) / n_pts
    rho_x = dct(coef, type=3) / (np.pi * np.sin(theta))
    lam = (np.cos(theta) + 1.0) * (0.5 * lam_max)
    return lam[::-1].copy(), (rho_x * (2.0 / lam_max))[::-1].copy()


def smearing_width(lam, lam_max, degree):
    """Jackson resolution in λ at λ: (π/p) sqrt(1 - x^2) in x, times λ_max/2."""
    x = np.clip(chebcoef.unit_interval(lam, lam_max), -1 + 1e-12, 1 - 1e-12)
    return (np.pi / degree) * np.sqrt(1.0 - x * x) * (0.5 * lam_max)
