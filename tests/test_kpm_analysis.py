"""KPM post-processing against the reference's own analysis functions.

Fixtures: tests/golden/make_golden.py --kpm runs counting, dos_curve and
smearing_width of scripts/exp/exp_kpm_analyze.py:39-70 on two moment tables
(degree 120 on 500 nodes, and degree 1500 on 400 nodes, where the DCT
evaluation folds orders above the node count).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

KPM_GOLDEN = Path(__file__).resolve().parent / "golden" / "reference_kpm_golden.npz"


@pytest.fixture(scope="module")
def kg():
    return dict(np.load(KPM_GOLDEN, allow_pickle=False))


def _close(a, b, rtol):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    assert np.abs(a - b).max() <= rtol * max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("tag", ["ka0", "ka1"])
@pytest.mark.parametrize("impl", ["library", "oracle"])
def test_counting_dos_smearing_match_reference(kg, tag, impl):
    if impl == "library":
        from eigenfns_gb300 import kpm as mod
    else:
        from oracle import kpm as mod
    mom, lams = kg[f"{tag}_mom"], kg[f"{tag}_lams"]
    lmax, n_pts = kg[f"{tag}_args"]
    mean, se, est = mod.counting(mom, lmax, lams)
    _close(est, kg[f"{tag}_count_est"], 1e-12)
    _close(mean, kg[f"{tag}_count_mean"], 1e-12)
    # the spread is a difference of numbers ~1e3 times larger: compare on their scale
    assert np.abs(se - kg[f"{tag}_count_se"]).max() <= 1e-12 * np.abs(est).max()
    lam, rho = mod.dos_curve(mom, lmax, n_pts=int(n_pts))
    _close(lam, kg[f"{tag}_dos_lam"], 1e-14)
    _close(rho, kg[f"{tag}_dos_rho"], 1e-11)
    _close(mod.smearing_width(lams, lmax, mom.shape[1] - 1), kg[f"{tag}_smear"], 1e-14)


def test_coefficient_module_matches_bandpass_fixtures(golden):
    """One coefficient implementation serves the filters: the reference's bandpass
    coefficients (interior.py:312-333) to rounding."""
    from eigenfns_gb300 import chebcoef
    for tag in ("bp0", "bp1", "bp2"):
        lo, hi, lmax, p = golden[f"{tag}_args"]
        _close(chebcoef.bandpass(lo, hi, lmax, int(p)), golden[f"{tag}_coef"], 1e-13)


def test_jackson_damping_properties():
    from eigenfns_gb300 import chebcoef
    for p in (1, 7, 100, 3000):
        g = chebcoef.jackson_damping(p)
        assert g.shape == (p + 1,) and g[0] == pytest.approx(1.0, abs=1e-14)
        assert abs(g[-1]) < 1e-12 and np.all(np.diff(g) <= 1e-15)
    # a step's expansion evaluated away from the edge is the indicator
    c = chebcoef.damped_step(3.0, 10.0, 400)
    x = np.cos(np.linspace(0.05, np.pi - 0.05, 41))
    vals = np.polynomial.chebyshev.chebval(x, c)
    lam = (x + 1) * 5.0
    far = np.abs(lam - 3.0) > 0.3
    assert np.allclose(vals[far], (lam[far] < 3.0).astype(float), atol=2e-3)


def test_interior_window_is_the_lowest_with_the_target_count():
    """bench_interior.pick_window: the first window on the λ grid whose estimated count
    reaches the target, for a count growing like λ^1.5 (the photonic band DOS)."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench_interior as bi
    lo = np.geomspace(1e-3, 10.0, 500)
    count = lambda lam: 300.0 * lam ** 1.5
    j = bi.pick_window(lo, count(lo), count(lo * bi.WINDOW_RATIO), 69)
    inside = count(lo * bi.WINDOW_RATIO) - count(lo)
    assert inside[j] >= 69 and (j == 0 or inside[j - 1] < 69)
    assert bi.pick_window(lo, count(lo), count(lo * bi.WINDOW_RATIO), 10 ** 9) == len(lo) - 1
