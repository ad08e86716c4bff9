"""The oracle against the reference's own outputs and known-answer tests (CPU).

Golden values come from executing the reference modules themselves
(tests/golden/make_golden.py); the analytic spectra restate the reference's
tests/test_operator.py:27-65.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import chebyshev as ocheb
from oracle import interior as oint
from oracle import kpm as okpm
from oracle import solver as osol
from oracle.dense import dense_spectrum
from oracle.operator import MaxwellOperator, make_basis
from oracle.two_stage import two_stage


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


@pytest.mark.parametrize("tag", ["b0", "b1", "b2", "b3"])
def test_basis_matches_reference(golden, tag):
    G, L, k = int(golden[f"basis_{tag}_G"]), float(golden[f"basis_{tag}_L"]), golden[f"basis_{tag}_k"]
    b = make_basis(G, L, k, rdtype=np.float64)
    assert np.array_equal(b.kn, golden[f"basis_{tag}_kn"])
    assert np.array_equal(b.t, golden[f"basis_{tag}_t"])


@pytest.mark.parametrize("tag", ["op8", "op6k", "op12k"])
@pytest.mark.parametrize("dname,dtype,tol", [("c128", np.complex128, 1e-12), ("c64", np.complex64, 2e-6)])
def test_operator_matches_reference(golden, tag, dname, dtype, tol):
    op = MaxwellOperator(golden[f"{tag}_eps"], float(golden[f"{tag}_L"]), golden[f"{tag}_k"], dtype=dtype)
    X = golden[f"{tag}_X"].astype(dtype)
    assert rel(op.theta(X), golden[f"{tag}_{dname}_theta"]) < tol
    assert rel(op.precondition(X), golden[f"{tag}_{dname}_precond"]) < tol
    assert rel(op.precondition_simple(X, 3.0), golden[f"{tag}_{dname}_precond_simple"]) < tol
    assert rel(op.h_realspace(X), golden[f"{tag}_{dname}_h"]) < tol
    assert rel(op.e_realspace(X, np.asarray([2.0, 3.0, 5.0])), golden[f"{tag}_{dname}_e"]) < tol
    assert op.kn_floor == pytest.approx(float(golden[f"{tag}_{dname}_kn_floor"]), rel=1e-6)
    assert op.eps_mean_inv == pytest.approx(float(golden[f"{tag}_{dname}_eps_mean_inv"]), rel=1e-12)


def test_block_linear_algebra_matches_reference(golden):
    A, B, L, C = golden["la_A"], golden["la_B"], golden["la_L"], golden["la_C"]
    assert rel(osol.gram(A, B), golden["la_gram"]) < 1e-6
    assert rel(osol.combine(C, A, B), golden["la_combine"]) < 1e-6
    assert rel(osol.deflate(B, L, 3), golden["la_deflate"]) < 1e-6
    assert rel(osol.ortho_block(B), golden["la_ortho"]) < 1e-5
    Od = osol.ortho_block(golden["la_Bdep"])
    ref = golden["la_ortho_dep"]
    assert (np.linalg.norm(Od.reshape(7, -1), axis=1) < 0.5).sum() == \
        (np.linalg.norm(ref.reshape(7, -1), axis=1) < 0.5).sum() == 1
    # the kept span agrees (rotation within near-degenerate SVQB directions is free)
    Qa = np.linalg.qr(Od.reshape(7, -1).T)[0][:, :6]
    Qb = np.linalg.qr(ref.reshape(7, -1).T)[0][:, :6]
    sv = np.linalg.svd(Qa.conj().T @ Qb, compute_uv=False)
    assert sv.min() > 0.9999


@pytest.mark.parametrize("tag", ["bp0", "bp1", "bp2"])
def test_bandpass_coeffs_match_reference(golden, tag):
    lo, hi, lmax, p = golden[f"{tag}_args"]
    assert np.array_equal(oint.bandpass_coeffs(lo, hi, lmax, int(p)), golden[f"{tag}_coef"])


def _op8(golden):
    return MaxwellOperator(golden["op8_eps"], float(golden["op8_L"]), dtype=np.complex64)


def test_lanczos_matches_reference(golden):
    op = _op8(golden)
    lm = ocheb.lanczos_lambda_max(op, iters=24, n_seeds=1, v0=golden["lanczos_v0"])
    assert lm == pytest.approx(float(golden["lanczos_lmax"]), rel=1e-5)


def test_cheb_poly_matches_reference(golden):
    op = _op8(golden)
    Y = oint._apply_cheb_poly(op, golden["cheb_X"], golden["cheb_coef"], float(golden["cheb_lmax"]))
    assert rel(Y, golden["cheb_Y"]) < 1e-5


def test_rr_extract_matches_reference(golden):
    op = _op8(golden)
    lam, Xr, rn = oint.rr_extract(op, golden["rr_X"], theta_chunk=4)
    assert np.allclose(lam, golden["rr_lam"], rtol=1e-5)
    assert np.allclose(rn, golden["rr_rn"], rtol=1e-4)
    ov = np.abs(np.sum(Xr.reshape(6, -1).conj() * golden["rr_Xr"].reshape(6, -1), axis=1))
    assert np.all(ov > 1 - 1e-5)


def test_kpm_count_matches_reference(golden):
    op = _op8(golden)
    mean, se, lb, lmax, deg, npb = golden["kpmcount_out"]
    m2, s2 = ocheb.kpm_count_below(op, lb, lmax, degree=int(deg), Z=golden["kpmcount_Z"])
    assert m2 == pytest.approx(mean, abs=1e-3)
    assert s2 == pytest.approx(se, abs=1e-3)


def test_kpm_moments_match_reference(golden):
    eps = golden["kpmdos_eps"]
    op = MaxwellOperator(eps, float(golden["kpmdos_L"]), dtype=np.complex64)
    Z = golden["kpmdos_Z"]
    mom = okpm.kpm_moments(op, float(golden["kpmdos_lmax"]), 40, Z.shape[0], chunk=2, Z=Z)
    ref = golden["kpmdos_moments"]
    assert mom.shape == ref.shape
    assert np.abs(mom / mom[:, :1] - ref / ref[:, :1]).max() < 1e-5


def test_lobpcg_matches_reference_and_dense(golden):
    op = _op8(golden)
    nev, m, guard, tol = golden["lobpcg_args"]
    vals, vecs, _ = osol.lobpcg_blocks(op, int(nev), m=int(m), guard=int(guard), tol=tol, maxit=300)
    assert np.allclose(vals, golden["lobpcg_vals"], rtol=2e-6)
    w = dense_spectrum(MaxwellOperator(golden["op8_eps"], 1.0, dtype=np.complex128))[2:2 + int(nev)]
    assert np.abs(vals - w).max() / w.max() < 2e-6
    V = vecs.reshape(int(nev), -1)
    assert np.abs(V.conj() @ V.T - np.eye(int(nev))).max() < 5e-4


def test_two_stage_matches_reference(golden):
    lo, hi, lmax, m, bd, bo, pd, po, tol, chunk, tchunk = golden["two_args"]
    op = MaxwellOperator(golden["two_eps"], float(golden["two_L"]), dtype=np.complex64)
    res = two_stage(op, lo, hi, lmax, int(m), int(bd), int(bo), int(pd), int(po), tol,
                    int(chunk), int(tchunk), X_init=golden["two_X0"])
    assert res["vals"].shape == golden["two_vals"].shape
    assert np.allclose(res["vals"], golden["two_vals"], rtol=1e-5)


# ---- the reference's analytic operator tests (tests/test_operator.py:27-65) ----

def test_homogeneous_matches_analytic():
    G, L, eps0 = 8, 1.0, 4.0
    w = dense_spectrum(MaxwellOperator(np.full((G, G, G), eps0, np.float32), L))
    k = 2 * np.pi * np.fft.fftfreq(G, d=L / G)
    g2 = (np.array(np.meshgrid(k, k, k, indexing="ij")) ** 2).sum(0).ravel()
    ana = np.sort(np.concatenate([g2[g2 > 0] / eps0] * 2))
    assert (np.abs(w) < 1e-5).sum() == 2
    assert (np.abs(np.sort(w)[2:] - ana) / ana).max() < 5e-6


def test_hermitian_and_psd_on_disordered():
    from oracle.dense import dense_theta
    rng = np.random.default_rng(0)
    G = 8
    eps = np.asarray(1.0 + 7.57 * (rng.random((G, G, G)) > 0.7), np.float32)
    M = dense_theta(MaxwellOperator(eps, 1.0))
    assert np.abs(M - M.conj().T).max() / np.abs(M).max() < 1e-5
    w = np.linalg.eigvalsh((M + M.conj().T) / 2)
    assert w.min() > -1e-4 * abs(w).max()


def test_bloch_k_reduces_to_shifted_planewaves():
    G, L, eps0 = 6, 1.0, 2.25
    kf = (0.5, 0.0, 0.0)
    w = dense_spectrum(MaxwellOperator(np.full((G, G, G), eps0, np.float32), L, k_frac=kf))
    k1 = 2 * np.pi * np.fft.fftfreq(G, d=L / G)
    k0 = 2 * np.pi * np.asarray(kf) / L
    KX, KY, KZ = np.meshgrid(k1 + k0[0], k1 + k0[1], k1 + k0[2], indexing="ij")
    ana = np.sort(np.concatenate([(KX ** 2 + KY ** 2 + KZ ** 2).ravel() / eps0] * 2))
    assert (np.abs(w - ana) / np.maximum(ana, 1e-12)).max() < 5e-6


def test_oracle_participation_limits():
    """PR of a uniform density is N_vox (fraction 1); of a single voxel 1."""
    from oracle.localization import participation
    u = np.ones((4, 4, 4))
    assert participation(u)["pr_vox"] == pytest.approx(64.0)
    assert participation(u)["pr_fraction"] == pytest.approx(1.0)
    v = np.zeros((4, 4, 4))
    v[1, 2, 3] = 5.0
    assert participation(v)["pr_vox"] == pytest.approx(1.0)
