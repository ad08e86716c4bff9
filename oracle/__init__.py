"""CPU oracle for the Maxwell eigensolver hot path.

TEST INFRASTRUCTURE ONLY. This package is a numpy/scipy restatement of the
reference implementation (fhernandez93/eigenfns, JAX) used as the checker in
`tests/`, in `__graft_entry__.smoke()` and as the timed CPU baseline in
`bench.py`. Nothing in `eigenfns_gb300/` imports it; the product path runs on
the CUDA library and fails loudly when that library is missing.

Modules and the reference files they restate:

* `oracle.operator`   -- eigenfns/operator.py:29-184 (frame, Θ, preconditioners)
* `oracle.solver`     -- eigenfns/solver.py:31-411 (Gram, SVQB, deflation, LOBPCG)
* `oracle.chebyshev`  -- eigenfns/chebyshev.py:28-267 (Lanczos λ_max, ChebSI, KPM count)
* `oracle.interior`   -- eigenfns/interior.py:37-88, 312-466 (RR extract, bandpass ChebSI)
* `oracle.kpm`        -- scripts/exp/exp_kpm_dos.py:125-163 and
                         scripts/exp/exp_kpm_analyze.py:22-70 (KPM moments, DOS)
* `oracle.two_stage`  -- scripts/run_interior.py:154-224 (build -> polish driver)
* `oracle.dense`      -- tests/test_operator.py:16-24 (dense Θ by columns)

Parity pin: the restatement is checked against fixtures produced by executing
the reference's own modules under a numpy-backed stand-in for `jax`
(`tests/golden/make_golden.py`), and against the reference's known-answer tests
(analytic homogeneous and Bloch spectra, tests/test_operator.py:27-65).
"""
