"""Chebyshev expansion coefficients of the spectral filters (host, float64).

One module serves the bandpass filter of the interior solver, the completeness
count and the KPM analysis. The formulas are the kernel polynomial method's
standard ones (Weiße, Wellein, Alvermann and Fehske, Rev. Mod. Phys. 78, 275
(2006), sections II.C-II.D):

* Jackson damping for a truncation at degree p (orders 0..p), with a = π/(p+1):
  g_k = [(p + 1 - k) cos(k a) + sin(k a) cot(a)] / (p + 1);
* the step 1{x < x_b} on [-1, 1] in Chebyshev polynomials: with x = cos θ and
  x_b = cos θ_b the step is 1{θ > θ_b}, so
  c_0 = (1/π) ∫_{θ_b}^{π} dθ = 1 - θ_b/π and
  c_k = (2/π) ∫_{θ_b}^{π} cos kθ dθ = -2 sin(k θ_b) / (k π);
* a window [λ_lo, λ_hi] as the difference of two steps, damped.

The spectrum [0, λ_max] maps to [-1, 1] by x = 2λ/λ_max - 1. The reference
evaluates the same quantities at eigenfns/interior.py:312-333 (bandpass),
eigenfns/chebyshev.py:232-242 (count) and scripts/exp/exp_kpm_analyze.py:22-36
(analysis); the values agree to rounding.
"""
from __future__ import annotations

import numpy as np


def jackson_damping(degree: int) -> np.ndarray:
    """Jackson factors g_0..g_p for degree p (g_0 = 1)."""
    p = int(degree)
    a = np.pi / (p + 1)
    ka = a * np.arange(p + 1, dtype=np.float64)
    cot_a = np.cos(a) / np.sin(a)
    return ((p + 1 - np.arange(p + 1)) * np.cos(ka) + np.sin(ka) * cot_a) / (p + 1)


def unit_interval(lam, lam_max: float):
    """Map λ in [0, λ_max] to x in [-1, 1]."""
    return 2.0 * np.asarray(lam, np.float64) / float(lam_max) - 1.0


def step_below(x_b: float, degree: int) -> np.ndarray:
    """Undamped Chebyshev coefficients c_0..c_p of 1{x < x_b}."""
    theta_b = float(np.arccos(np.clip(float(x_b), -1.0, 1.0)))
    k = np.arange(1, int(degree) + 1, dtype=np.float64)
    c = np.empty(int(degree) + 1)
    c[0] = 1.0 - theta_b / np.pi
    c[1:] = np.sin(k * theta_b) * (-2.0 / np.pi) / k
    return c


def damped_step(lam_b: float, lam_max: float, degree: int) -> np.ndarray:
    """Jackson-damped coefficients of 1{λ < λ_b} (the completeness count's filter)."""
    return jackson_damping(degree) * step_below(unit_interval(lam_b, lam_max), degree)


def bandpass(lam_lo: float, lam_hi: float, lam_max: float, degree: int) -> np.ndarray:
    """Jackson-damped coefficients of 1{λ_lo < λ < λ_hi}."""
    hi = step_below(unit_interval(lam_hi, lam_max), degree)
    lo = step_below(unit_interval(lam_lo, lam_max), degree)
    return jackson_damping(degree) * (hi - lo)
