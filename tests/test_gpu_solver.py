"""GPU parity of the solvers: LOBPCG, Lanczos, bandpass ChebSI, two-stage, KPM.

Eigenvalues are compared within 1e-5 relative (the stated parity bar) against
the reference's own solver outputs, dense eigendecompositions and the oracle;
KPM moments within 1e-4 absolute on moments normalised by μ_0.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def gpu():
    from eigenfns_gb300 import _lib
    _lib.load()
    assert torch.cuda.is_available()
    return torch.device("cuda", 0)


def op_from(golden, prefix, k=(0.0, 0.0, 0.0)):
    from eigenfns_gb300.operator import MaxwellOperator
    return MaxwellOperator(golden[f"{prefix}_eps"], float(golden[f"{prefix}_L"]), k_frac=k)


def test_lobpcg_matches_reference_and_dense(golden, gpu):
    from eigenfns_gb300.solver import lobpcg_blocks
    from oracle.dense import dense_spectrum
    from oracle.operator import MaxwellOperator as Ref
    op = op_from(golden, "op8")
    nev, m, guard, tol = golden["lobpcg_args"]
    vals, vecs, st = lobpcg_blocks(op, int(nev), m=int(m), guard=int(guard), tol=tol, maxit=300,
                                   verbose=False)
    assert np.allclose(vals, golden["lobpcg_vals"], rtol=1e-5)
    w = dense_spectrum(Ref(golden["op8_eps"], 1.0, dtype=np.complex128))[2:2 + int(nev)]
    assert np.abs(vals - w).max() / w.max() < 1e-5
    assert (np.diff(vals) > -1e-8).all() and vals[0] > 1e-3
    V = vecs.reshape(int(nev), -1).cpu().numpy()
    assert np.abs(V.conj() @ V.T - np.eye(int(nev))).max() < 5e-4
    assert st.theta_applications > 0 and len(st.rounds) >= 2


def test_lobpcg_subspaces_match_dense_after_cluster_alignment(golden, gpu):
    """Principal-angle overlap >= 0.9999 per degenerate cluster (exp_g4_degeneracy.py:46-70)."""
    from eigenfns_gb300.solver import lobpcg_blocks
    from oracle.dense import dense_eigh
    from oracle.operator import MaxwellOperator as Ref
    op = op_from(golden, "op8")
    vals, vecs, _ = lobpcg_blocks(op, 12, m=8, guard=3, tol=1e-6, maxit=300, verbose=False)
    w, V = dense_eigh(Ref(golden["op8_eps"], 1.0, dtype=np.complex128))
    Vd = V[:, 2:2 + 20]
    wd = w[2:2 + 20]
    X = vecs.reshape(12, -1).cpu().numpy().astype(np.complex128)
    i = 0
    while i < 12:
        j = i + 1
        while j < 12 and (vals[j] - vals[j - 1]) / vals[j] < 1e-3:
            j += 1
        if j == 12:
            break  # the top cluster may continue past the computed set
        cl = np.where(np.abs(wd - vals[i:j].mean()) / vals[i:j].mean() < 2e-3)[0]
        Qa = np.linalg.qr(X[i:j].T)[0]
        Qb = np.linalg.qr(Vd[:, cl])[0]
        s = np.linalg.svd(Qb.conj().T @ Qa, compute_uv=False)
        assert s.min() >= 0.9999, (i, j, s)
        i = j


def test_lanczos_matches_reference(golden, gpu):
    from eigenfns_gb300.chebyshev import lanczos_lambda_max
    op = op_from(golden, "op8")
    lm = lanczos_lambda_max(op, iters=24, n_seeds=1, v0=golden["lanczos_v0"])
    assert lm == pytest.approx(float(golden["lanczos_lmax"]), rel=1e-5)


def test_cheb_poly_matches_reference(golden, gpu):
    from eigenfns_gb300.interior import _apply_cheb_poly
    op = op_from(golden, "op8")
    Y = _apply_cheb_poly(op, golden["cheb_X"], golden["cheb_coef"], float(golden["cheb_lmax"]))
    ref = golden["cheb_Y"]
    assert np.abs(Y.cpu().numpy() - ref).max() / np.abs(ref).max() < 1e-5


def test_rr_extract_matches_reference(golden, gpu):
    from eigenfns_gb300.interior import rr_extract
    op = op_from(golden, "op8")
    lam, Xr, rn = rr_extract(op, golden["rr_X"], theta_chunk=4)
    assert np.allclose(lam, golden["rr_lam"], rtol=1e-5)
    assert np.allclose(rn, golden["rr_rn"], rtol=1e-3)
    ov = np.abs(np.sum(Xr.reshape(6, -1).cpu().numpy().conj() * golden["rr_Xr"].reshape(6, -1), axis=1))
    assert np.all(ov > 1 - 1e-5)


def test_kpm_count_matches_reference(golden, gpu):
    from eigenfns_gb300.chebyshev import kpm_count_below
    op = op_from(golden, "op8")
    mean, se, lb, lmax, deg, npb = golden["kpmcount_out"]
    m2, s2 = kpm_count_below(op, lb, lmax, degree=int(deg), Z=golden["kpmcount_Z"])
    assert m2 == pytest.approx(mean, abs=1e-3)
    assert s2 == pytest.approx(se, abs=1e-3)


@pytest.mark.parametrize("tag", ["kd_plain", "kd_defl"])
def test_kpm_count_deflated_probes_match_reference(tag, gpu):
    """Completeness-gate mode (chebyshev.py:221-252): probes deflated twice against the
    locked eigenvectors below λ_b, against the reference's run on the same probes."""
    from pathlib import Path
    from eigenfns_gb300.chebyshev import kpm_count_below
    from eigenfns_gb300.operator import MaxwellOperator
    kg = np.load(Path(__file__).resolve().parent / "golden" / "reference_kpm_golden.npz")
    op = MaxwellOperator(kg["kd_eps"], 1.0)
    mean, se, lb, lmax, deg, npb = kg[f"{tag}_out"]
    locked = kg["kd_locked"] if tag == "kd_defl" else None
    m2, s2 = kpm_count_below(op, lb, lmax, degree=int(deg), Z=kg[f"{tag}_Z"], locked=locked)
    assert m2 == pytest.approx(mean, abs=1e-3)
    assert s2 == pytest.approx(se, abs=1e-3)


def test_kpm_moments_match_reference(golden, gpu):
    from eigenfns_gb300.kpm import kpm_moments
    from eigenfns_gb300.operator import MaxwellOperator
    op = MaxwellOperator(golden["kpmdos_eps"], float(golden["kpmdos_L"]))
    Z = golden["kpmdos_Z"]
    mom = kpm_moments(op, float(golden["kpmdos_lmax"]), 40, Z.shape[0], chunk=2, Z=Z)
    ref = golden["kpmdos_moments"]
    assert mom.shape == ref.shape
    assert np.abs(mom / mom[:, :1] - ref / ref[:, :1]).max() < 1e-4


def test_kpm_moments_match_oracle_complex_probes(gpu):
    """Complex Rademacher probes at 32^3 on a generated structure, seeded identically."""
    from eigenfns_gb300.kpm import kpm_moments
    from eigenfns_gb300.operator import MaxwellOperator
    from eigenfns_gb300.structure import make_structure
    from oracle.kpm import kpm_moments as ref_moments
    from oracle.operator import MaxwellOperator as Ref
    from oracle.chebyshev import lanczos_lambda_max as ref_lanczos
    eps, L, _ = make_structure(64, 32, seed=5)
    ref_op = Ref(eps, L, dtype=np.complex128)
    lam_max = 1.05 * ref_lanczos(ref_op, iters=24, n_seeds=1)
    mom = kpm_moments(MaxwellOperator(eps, L), lam_max, 60, 3, seed=2, probe_kind="complex")
    ref = ref_moments(ref_op, lam_max, 60, 3, seed=2, probe_kind="complex")
    assert np.abs(mom / mom[:, :1] - ref / ref[:, :1]).max() < 1e-4


def test_two_stage_matches_reference(golden, gpu):
    from eigenfns_gb300.operator import MaxwellOperator
    from eigenfns_gb300.run_interior import two_stage
    lo, hi, lmax, m, bd, bo, pd, po, tol, chunk, tchunk = golden["two_args"]
    op = MaxwellOperator(golden["two_eps"], float(golden["two_L"]))
    res = two_stage(op, lo, hi, int(m), lam_max=lmax, build_degree=int(bd), build_outers=int(bo),
                    polish_degree=int(pd), polish_outers=int(po), tol=tol, chunk=int(chunk),
                    theta_chunk=int(tchunk), X_init=golden["two_X0"])
    assert res["vals"].shape == golden["two_vals"].shape
    assert np.allclose(res["vals"], golden["two_vals"], rtol=1e-5)
    # build stage alone (no polish outer): the build's last Ritz values come back
    b = two_stage(op, lo, hi, int(m), lam_max=lmax, build_degree=int(bd), build_outers=int(bo),
                  polish_degree=int(pd), polish_outers=0, tol=tol, chunk=int(chunk),
                  theta_chunk=int(tchunk), X_init=golden["two_X0"])
    assert b["lam"].shape == (int(m),)
    assert [h["stage"] for h in b["history"]] == ["build"] * int(bo)


def test_rasterizer_matches_oracle(gpu):
    from eigenfns_gb300.structure import generate_network, rasterize
    from oracle.structure import rasterize_averaged
    net = generate_network(64, seed=3)
    eps = rasterize(net, 16, sub=3)
    ref = rasterize_averaged(net.rods, 16, net.box_size, sub=3)
    assert np.array_equal(eps, ref)
    assert 1.0 <= eps.min() and eps.max() <= 8.41 + 1e-6


def test_chebsi_bottom_up_matches_dense(golden, gpu):
    """Bottom-up ChebSI (chebyshev.py:103-210): lowest bands equal the dense spectrum."""
    from eigenfns_gb300.chebyshev import chebsi_bottom_up
    from oracle.dense import dense_spectrum
    from oracle.operator import MaxwellOperator as Ref
    op = op_from(golden, "op8")
    vals, vecs, st = chebsi_bottom_up(op, 8, guard=8, degree=60, tol=1e-5, max_outer=40, verbose=False)
    w = dense_spectrum(Ref(golden["op8_eps"], 1.0, dtype=np.complex128))[2:2 + 8]
    assert vals.shape == (8,)
    assert np.abs(vals - w).max() / w.max() < 1e-5
    assert st.theta_applications > 0


def test_lobpcg_resumable_checkpoint_and_resume(golden, gpu, tmp_path):
    """Blocks are checkpointed as they lock; a resumed run continues from them and
    reproduces the uninterrupted eigenvalues (solver.py:385-411, io.py:31-67)."""
    from eigenfns_gb300.io import BlockCheckpointer
    from eigenfns_gb300.solver import lobpcg_blocks, lobpcg_blocks_resumable
    op = op_from(golden, "op8")
    full, _, _ = lobpcg_blocks(op, 12, m=8, guard=3, tol=1e-6, maxit=300, verbose=False)
    ck = BlockCheckpointer(tmp_path, "solve")
    part, _, _ = lobpcg_blocks_resumable(op, 5, m=8, guard=3, tol=1e-6, maxit=300, verbose=False,
                                         checkpointer=ck)
    assert (tmp_path / "solve_block000_vals.npy").exists()
    res, vecs, _ = lobpcg_blocks_resumable(op, 12, m=8, guard=3, tol=1e-6, maxit=300, verbose=False,
                                           checkpointer=ck, resume=True)
    assert np.allclose(res[:5], part, rtol=1e-6)
    assert np.abs(res - full).max() / full.max() < 1e-5
    assert vecs.shape[0] == 12
