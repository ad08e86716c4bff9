"""eigenfns_gb300 -- GB300-native Maxwell eigensolver hot path.

A drop-in for the operator / solver / chebyshev / interior surface of
fhernandez93/eigenfns, computed by hand-written sm_103a CUDA kernels behind the
C ABI in include/eigenfns_gb300.h (ctypes binding in `_lib`):

  eigenfns_gb300.operator.MaxwellOperator     eigenfns.operator.MaxwellOperator
  eigenfns_gb300.solver.lobpcg_blocks         eigenfns.solver.lobpcg_blocks
  eigenfns_gb300.chebyshev.lanczos_lambda_max / kpm_count_below / chebsi_bottom_up
  eigenfns_gb300.interior.rr_extract / bandpass_coeffs / _apply_cheb_poly /
                         bandpass_subspace
  eigenfns_gb300.kpm.kpm_moments              scripts/exp/exp_kpm_dos.py moments
  eigenfns_gb300.run_interior.two_stage       scripts/run_interior.py solver logic
  eigenfns_gb300.io.BlockCheckpointer         eigenfns.io.BlockCheckpointer

Submodules are imported on use; importing one that computes loads the CUDA
library and raises if it has not been built.
"""
__version__ = "0.1.0"
