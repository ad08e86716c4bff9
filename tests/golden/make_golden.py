"""Generate the golden fixtures by executing the reference's own code.

Run in the development container (the reference checkout must be present;
its path is the first argument or $EIGENFNS_REFERENCE):

    python tests/golden/make_golden.py <reference checkout>          # reference_golden.npz
    python tests/golden/make_golden.py <reference checkout> --kpm    # reference_kpm_golden.npz

JAX is not installed there, so `jax_standin` maps jax.numpy onto numpy and
records every random draw; the reference modules (eigenfns/operator.py,
solver.py, chebyshev.py, interior.py) and scripts (scripts/exp/exp_kpm_dos.py,
scripts/run_interior.py) then run unmodified. Each fixture stores the inputs
(including the random draws the reference consumed) and the reference's
outputs. The fixtures are small .npz files; tests/test_oracle_golden.py checks
the oracle against them, and tests/test_gpu_*.py check the CUDA library.
"""
from __future__ import annotations

import os
import sys
import json
import pathlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import jax_standin  # noqa: E402

jax_standin.install()


def disordered_eps(G, seed, p=0.7, contrast=7.57):
    rng = np.random.default_rng(seed)
    return np.asarray(1.0 + contrast * (rng.random((G, G, G)) > p), np.float32)


def rand_c(rng, shape, dtype):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(dtype)


def main(ref_root: str):
    ref = Path(ref_root)
    sys.path.insert(0, str(ref))
    sys.path.insert(0, str(ref / "scripts"))
    import jax.numpy as jnp
    from eigenfns.operator import MaxwellOperator, make_basis
    from eigenfns import solver as rsolver
    from eigenfns import chebyshev as rcheb
    from eigenfns import interior as rint

    out = {}
    rng = np.random.default_rng(1234)

    # ---- frame ---------------------------------------------------------------
    for tag, (G, L, k) in {"b0": (8, 1.0, (0, 0, 0)), "b1": (6, 1.0, (0.5, 0, 0)),
                           "b2": (8, 2.3, (0.1, -0.37, 0.25)), "b3": (12, 1.7, (0.0, 0.0, 0.45))}.items():
        b = make_basis(G, L, k, rdtype=np.float64)
        out[f"basis_{tag}_G"] = np.int64(G)
        out[f"basis_{tag}_L"] = np.float64(L)
        out[f"basis_{tag}_k"] = np.asarray(k, np.float64)
        out[f"basis_{tag}_kn"] = np.asarray(b.kn)
        out[f"basis_{tag}_t"] = np.asarray(b.t)

    # ---- operator applications -------------------------------------------------
    cases = {"op8": (disordered_eps(8, 0), 1.0, (0, 0, 0)),
             "op6k": (disordered_eps(6, 5, 0.6, 3.0), 1.3, (0.5, 0.0, -0.25)),
             "op12k": (disordered_eps(12, 9, 0.75, 7.41), 2.0, (0.21, -0.4, 0.33))}
    for tag, (eps, L, k) in cases.items():
        G = eps.shape[0]
        out[f"{tag}_eps"] = eps
        out[f"{tag}_L"] = np.float64(L)
        out[f"{tag}_k"] = np.asarray(k, np.float64)
        X = rand_c(rng, (3, 2, G, G, G), np.complex128)
        out[f"{tag}_X"] = X
        for dname, dt in (("c128", jnp.complex128), ("c64", jnp.complex64)):
            op = MaxwellOperator(eps, L, k_frac=k, dtype=dt)
            Xd = jnp.asarray(X.astype(dt))
            out[f"{tag}_{dname}_theta"] = np.asarray(op.theta(Xd))
            out[f"{tag}_{dname}_precond"] = np.asarray(op.precondition(Xd))
            out[f"{tag}_{dname}_precond_simple"] = np.asarray(op.precondition_simple(Xd, 3.0))
            out[f"{tag}_{dname}_h"] = np.asarray(op.h_realspace(Xd))
            out[f"{tag}_{dname}_e"] = np.asarray(op.e_realspace(Xd, jnp.asarray([2.0, 3.0, 5.0])))
            out[f"{tag}_{dname}_kn_floor"] = np.float64(op.kn_floor)
            out[f"{tag}_{dname}_eps_mean_inv"] = np.float64(op.eps_mean_inv)

    # ---- block linear algebra --------------------------------------------------
    G = 8
    A = rand_c(rng, (5, 2, G, G, G), np.complex64)
    B = rand_c(rng, (7, 2, G, G, G), np.complex64)
    Lk = np.asarray(rsolver.ortho_block(jnp.asarray(rand_c(rng, (4, 2, G, G, G), np.complex64))))
    C = rand_c(rng, (12, 7), np.complex64)
    out["la_A"], out["la_B"], out["la_L"], out["la_C"] = A, B, Lk, C
    out["la_gram"] = np.asarray(rsolver.gram(jnp.asarray(A), jnp.asarray(B)))
    out["la_combine"] = np.asarray(rsolver.combine(jnp.asarray(C), jnp.asarray(A), jnp.asarray(B)))
    out["la_deflate"] = np.asarray(rsolver.deflate(jnp.asarray(B), jnp.asarray(Lk), 3))
    out["la_ortho"] = np.asarray(rsolver.ortho_block(jnp.asarray(B)))
    Bd = B.copy()
    Bd[3] = Bd[1] + 1e-7 * Bd[2]        # near-dependent row: SVQB drops a direction
    out["la_Bdep"] = Bd
    out["la_ortho_dep"] = np.asarray(rsolver.ortho_block(jnp.asarray(Bd)))

    # ---- bandpass coefficients and polynomial filter ----------------------------
    for tag, (lo, hi, lmax, p) in {"bp0": (5.0, 15.0, 400.0, 800), "bp1": (1.757, 1.93, 2208.9, 3000),
                                  "bp2": (0.3, 0.9, 12.0, 57)}.items():
        out[f"{tag}_args"] = np.asarray([lo, hi, lmax, p], np.float64)
        out[f"{tag}_coef"] = rint.bandpass_coeffs(lo, hi, lmax, int(p))
    eps, L, k = cases["op8"]
    op64 = MaxwellOperator(eps, L, dtype=jnp.complex64)
    mask = np.asarray(op64.basis.kn > 0, np.float32)[None, None]
    Xc = (rand_c(rng, (2, 2, 8, 8, 8), np.complex64) * mask).astype(np.complex64)
    lam_max_8 = 1.05 * float(np.max(np.abs(np.asarray(out["op8_c128_theta"]))))  # placeholder, replaced below
    jax_standin.DRAWS.clear()
    lm = rcheb.lanczos_lambda_max(op64, iters=24, seed=3, n_seeds=1)
    out["lanczos_v0"] = jax_standin.DRAWS[0][1] + 1j * jax_standin.DRAWS[1][1]
    out["lanczos_lmax"] = np.float64(lm)
    lam_max_8 = 1.05 * lm
    out["cheb_X"] = Xc
    out["cheb_lmax"] = np.float64(lam_max_8)
    coef = rint.bandpass_coeffs(20.0, 60.0, lam_max_8, 40)
    out["cheb_coef"] = coef
    out["cheb_Y"] = np.asarray(rint._apply_cheb_poly(op64, jnp.asarray(Xc), coef, lam_max_8))

    # ---- rr_extract ------------------------------------------------------------------
    Xr = (rand_c(rng, (6, 2, 8, 8, 8), np.complex64) * mask).astype(np.complex64)
    out["rr_X"] = Xr
    lam, Xo, rn = rint.rr_extract(op64, jnp.asarray(Xr), theta_chunk=4)
    out["rr_lam"], out["rr_Xr"], out["rr_rn"] = np.asarray(lam), np.asarray(Xo), np.asarray(rn)

    # ---- KPM count -------------------------------------------------------------------
    jax_standin.DRAWS.clear()
    mean, se = rcheb.kpm_count_below(op64, 40.0, lam_max_8, degree=60, n_probe=4, seed=2)
    out["kpmcount_Z"] = np.where(jax_standin.DRAWS[0][1], 1.0, -1.0).astype(np.complex64)
    out["kpmcount_out"] = np.asarray([mean, se, 40.0, lam_max_8, 60, 4], np.float64)

    # ---- LOBPCG (reference solver, c64) -------------------------------------------------
    jax_standin.DRAWS.clear()
    vals, vecs, st = rsolver.lobpcg_blocks(op64, 12, m=8, guard=3, tol=1e-6, maxit=300, verbose=False)
    out["lobpcg_vals"] = np.asarray(vals)
    out["lobpcg_vecs"] = np.asarray(vecs)
    out["lobpcg_args"] = np.asarray([12, 8, 3, 1e-6], np.float64)

    # ---- KPM moments (scripts/exp/exp_kpm_dos.py main) -------------------------------
    import tempfile
    tmp = Path(tempfile.mkdtemp())
    rods = np.asarray([[-0.8, -0.6, -0.3, 0.5, 0.4, 0.7],
                       [0.5, 0.4, 0.7, 0.9, -0.8, 0.1],
                       [-0.7, 0.8, 0.2, 0.3, 0.5, -0.6]])
    rodfile = tmp / "tiny_N8_ends.txt"
    np.savetxt(rodfile, rods)
    captured = {}
    real_savez = np.savez_compressed
    real_write = pathlib.Path.write_text

    def fake_savez(path, **kw):
        captured.update(kw)
    np.savez_compressed = fake_savez
    pathlib.Path.write_text = lambda self, *a, **k: None
    import importlib
    sys.argv = ["exp_kpm_dos.py", str(rodfile), "--grid", "8", "--degree", "40",
                "--probes", "3", "--chunk", "2", "--tag", "golden", "--lam-max", "380.0",
                "--force", "--radius", "0.2", "--aspect", "1.0", "--eps-rod", "8.41"]
    jax_standin.DRAWS.clear()
    kmod = importlib.import_module("exp.exp_kpm_dos") if (ref / "scripts/exp/__init__.py").exists() \
        else _load(ref / "scripts/exp/exp_kpm_dos.py", "exp_kpm_dos")
    kmod.main()
    np.savez_compressed = real_savez
    pathlib.Path.write_text = real_write
    # draws: [timing probe, chunk 0 probes, chunk 1 probes]
    zs = [np.where(d[1], 1.0, -1.0).astype(np.complex64) for d in jax_standin.DRAWS[1:]]
    out["kpmdos_Z"] = np.concatenate(zs, axis=0)
    out["kpmdos_moments"] = np.asarray(captured["moments"])
    out["kpmdos_lmax"] = np.float64(380.0)
    from eigenfns.structure import load_rods, rasterize_penlike
    r_, N_, L_ = load_rods(rodfile)
    out["kpmdos_eps"] = rasterize_penlike(r_, 8, L_, minor_radius=0.2, aspect_ratio=1.0, eps_rod=8.41)
    out["kpmdos_L"] = np.float64(L_)

    # ---- two-stage driver (scripts/run_interior.py main) -------------------------------
    saved = {}
    real_save, real_savez2 = np.save, np.savez
    real_mkdir, real_replace = pathlib.Path.mkdir, pathlib.Path.replace
    np.save = lambda path, arr, *a, **k: saved.__setitem__(Path(str(path)).name, np.asarray(arr))
    np.savez = lambda *a, **k: None
    pathlib.Path.mkdir = lambda self, *a, **k: None
    pathlib.Path.replace = lambda self, target: None
    pathlib.Path.write_text = lambda self, text, *a, **k: saved.__setitem__(self.name, text)
    r2 = tmp / "tiny_N8_two.txt"
    np.savetxt(r2, rods)
    sys.argv = ["run_interior.py", str(r2), "--grid", "8", "--lam-lo", "9.4", "--lam-hi", "11.2",
                "--m", "10", "--build-degree", "60", "--build-outers", "2",
                "--polish-degree", "400", "--polish-outers", "2", "--tol", "1e-3",
                "--radius", "0.2", "--aspect", "1.0", "--eps-rod", "8.41", "--lam-max", "380.0",
                "--chunk", "4", "--theta-chunk", "4", "--tag", "golden", "--force"]
    jax_standin.DRAWS.clear()
    imod = _load(ref / "scripts/run_interior.py", "run_interior")
    imod.main()
    np.save, np.savez = real_save, real_savez2
    pathlib.Path.mkdir, pathlib.Path.replace = real_mkdir, real_replace
    pathlib.Path.write_text = real_write
    out["two_X0"] = (jax_standin.DRAWS[0][1] + 1j * jax_standin.DRAWS[1][1]).astype(np.complex64)
    out["two_vals"] = saved["window_eigenvalues.npy"]
    out["two_res"] = saved["window_residuals.npy"]
    out["two_vecs"] = saved["window_vecs_spectral.npy"]
    out["two_report"] = np.asarray(saved["interior_report.json"])
    r2_, N2, L2 = load_rods(r2)
    out["two_eps"] = rasterize_penlike(r2_, 8, L2, minor_radius=0.2, aspect_ratio=1.0,
                                       eps_rod=8.41)
    out["two_L"] = np.float64(L2)
    out["two_args"] = np.asarray([9.4, 11.2, 380.0, 10, 60, 2, 400, 2, 1e-3, 4, 4], np.float64)

    dest = HERE / "reference_golden.npz"
    np.savez_compressed(dest, **out)
    print(f"wrote {dest} ({dest.stat().st_size / 1024:.0f} KiB, {len(out)} arrays)")


def main_kpm(ref_root: str):
    """KPM analysis (scripts/exp/exp_kpm_analyze.py:39-64) and the deflated-probe
    completeness count (eigenfns/chebyshev.py:213-267 with `locked`)."""
    ref = Path(ref_root)
    sys.path.insert(0, str(ref))
    import jax.numpy as jnp
    from eigenfns.operator import MaxwellOperator
    from eigenfns import chebyshev as rcheb
    from eigenfns import solver as rsolver
    ka = _load(ref / "scripts/exp/exp_kpm_analyze.py", "exp_kpm_analyze")
    out = {}
    rng = np.random.default_rng(4321)

    # analysis of a moment table: decaying per-probe moments, as a DOS produces
    for tag, (probes, p, lmax, n_pts) in {"ka0": (6, 120, 40.0, 500),
                                          "ka1": (4, 1500, 2208.9, 400)}.items():
        k = np.arange(p + 1)
        mom = rng.standard_normal((probes, p + 1)) / (1.0 + 0.05 * k) + np.cos(0.3 * k)
        mom[:, 0] = 2 * 8 ** 3 - 2
        lams = np.linspace(0.05 * lmax, 0.95 * lmax, 9)
        out[f"{tag}_mom"] = mom
        out[f"{tag}_args"] = np.asarray([lmax, n_pts], np.float64)
        out[f"{tag}_lams"] = lams
        mean, se, est = ka.counting(mom, lmax, lams)
        out[f"{tag}_count_mean"], out[f"{tag}_count_se"], out[f"{tag}_count_est"] = mean, se, est
        lam, rho = ka.dos_curve(mom, lmax, n_pts=n_pts)
        out[f"{tag}_dos_lam"], out[f"{tag}_dos_rho"] = lam, rho
        out[f"{tag}_smear"] = ka.smearing_width(lams, lmax, p)

    # deflated-probe count on the 8^3 operator of the main fixture set
    eps = disordered_eps(8, 0)
    op64 = MaxwellOperator(eps, 1.0, dtype=jnp.complex64)
    vals, vecs, _ = rsolver.lobpcg_blocks(op64, 12, m=8, guard=3, tol=1e-5, maxit=300,
                                         verbose=False)
    lam_b = float(0.5 * (vals[5] + vals[6]))          # six eigenvalues below lam_b
    locked = np.asarray(vecs)[:6]
    lam_max = 1.05 * rcheb.lanczos_lambda_max(op64, iters=24, seed=3, n_seeds=1)
    for tag, lk in (("kd_plain", None), ("kd_defl", locked)):
        jax_standin.DRAWS.clear()
        mean, se = rcheb.kpm_count_below(op64, lam_b, lam_max, degree=80, n_probe=6, seed=5,
                                         locked=None if lk is None else jnp.asarray(lk))
        out[f"{tag}_Z"] = np.where(jax_standin.DRAWS[0][1], 1.0, -1.0).astype(np.complex64)
        out[f"{tag}_out"] = np.asarray([mean, se, lam_b, lam_max, 80, 6], np.float64)
    out["kd_eps"] = eps
    out["kd_locked"] = locked
    out["kd_vals"] = np.asarray(vals)

    dest = HERE / "reference_kpm_golden.npz"
    np.savez_compressed(dest, **out)
    print(f"wrote {dest} ({dest.stat().st_size / 1024:.0f} KiB, {len(out)} arrays)")


def _load(path: Path, name: str):
    import importlib.util
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    root = args[0] if args else os.environ.get("EIGENFNS_REFERENCE", "")
    if "--kpm" in sys.argv:
        main_kpm(root)
    else:
        main(root)
