"""The Maxwell operator on the GPU: a drop-in for eigenfns.operator.MaxwellOperator.

Mirrors eigenfns/operator.py:130-184 of the reference: same constructor
arguments (a cubic eps grid, box size, Bloch k in units of 2π/L), same
attributes (`grid_size`, `box_size`, `dtype`, `basis.kn`, `basis.t`,
`inv_eps`, `eps_grid`, `eps_mean_inv`, `kn_floor`) and methods (`theta`,
`precondition`, `precondition_simple`, `to_cartesian_spectral`,
`h_realspace`, `e_realspace`). Vectors are torch complex64 CUDA tensors of shape
(m, 2, G, G, G); numpy inputs are copied to the device first.

Θ and the preconditioners run in the library's fused FFT pipeline
(include/eigenfns_gb300.h: ef_theta, ef_precondition, ...). A complex128
operator is not provided on the GPU; asking for one raises ValueError.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import blas, profiling
from ._lib import call, load


@dataclass
class TransverseBasis:
    """Per-(k+G) frame and |k+G| for one k-point (operator.py:29-41)."""

    grid_size: int
    box_size: float
    k_frac: tuple
    kn: torch.Tensor   # (G,G,G) float32
    t: torch.Tensor    # (2,3,G,G,G) float32

    @property
    def n_dof(self) -> int:
        return 2 * self.grid_size ** 3


def _is_c128(dtype) -> bool:
    return dtype in (np.complex128, torch.complex128, "complex128") or \
        (isinstance(dtype, np.dtype) and dtype == np.complex128)


class MaxwellOperator:
    def __init__(self, eps, box_size: float, k_frac=(0.0, 0.0, 0.0), dtype=np.complex64,
                 device=None):
        eps = np.asarray(eps)
        if eps.ndim != 3 or len(set(eps.shape)) != 1:
            raise ValueError(f"eps must be a cube, got {eps.shape}")
        if _is_c128(dtype):
            raise ValueError("the GPU operator computes in complex64; complex128 is not provided")
        lib = load()
        self.dtype = np.complex64
        self.grid_size = int(eps.shape[0])
        self.box_size = float(box_size)
        self.k_frac = tuple(float(x) for x in k_frac)
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        if not lib.ef_supported_grid(self.grid_size):
            raise ValueError(f"grid size {self.grid_size} has no FFT plan")
        eps32 = np.ascontiguousarray(eps, dtype=np.float32)
        handle = C.c_void_p()
        with torch.cuda.device(self.device):
            call("ef_op_create", self.grid_size, self.box_size, *self.k_frac,
                 eps32.ctypes.data, C.byref(handle))
        self._h = handle
        self._lib = lib
        G = self.grid_size
        # eps_mean_inv and kn_floor exactly as the reference computes them (operator.py:148-151)
        self.eps_mean_inv = float(np.mean(1.0 / eps))
        kfl = C.c_double()
        call("ef_op_info", self._h, None, C.byref(kfl), None)
        self.kn_floor = float(kfl.value)
        self.eps_grid = torch.from_numpy(eps32).to(self.device)
        self.inv_eps = torch.from_numpy((1.0 / eps32).astype(np.float32)).to(self.device)
        with torch.cuda.device(self.device):
            kn = torch.empty((G, G, G), dtype=torch.float32, device=self.device)
            t = torch.empty((2, 3, G, G, G), dtype=torch.float32, device=self.device)
            call("ef_op_basis", self._h, kn.data_ptr(), t.data_ptr(), blas._stream())
            self.mask = torch.empty((G, G, G), dtype=torch.float32, device=self.device)
            call("ef_op_mask", self._h, self.mask.data_ptr(), blas._stream())
        self.basis = TransverseBasis(G, self.box_size, self.k_frac, kn, t)
        self.n_theta = 0

    # ---- housekeeping -------------------------------------------------------------
    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.ef_op_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    def vec_shape(self, m: int):
        G = self.grid_size
        return (m, 2, G, G, G)

    def _as_block(self, X) -> torch.Tensor:
        if not isinstance(X, torch.Tensor):
            X = torch.from_numpy(np.ascontiguousarray(np.asarray(X, np.complex64)))
        X = X.to(device=self.device, dtype=torch.complex64).contiguous()
        G = self.grid_size
        if X.dim() != 5 or tuple(X.shape[1:]) != (2, G, G, G):
            raise ValueError(f"expected a block (m, 2, {G}, {G}, {G}), got {tuple(X.shape)}")
        return X

    def configure(self, passes: int = 0, subbatch_bytes: int = 0) -> None:
        """Pipeline of the operator applications: passes 0 (automatic), 3 (z / xy-plane / z,
        grid edges 32, 48, 64, 96, 128) or 5 (pencil passes, every grid edge), and the
        sub-batch workspace cap in bytes (0 = the library default). Set by the autotuner
        (eigenfns_gb300.tune)."""
        call("ef_op_configure", self._h, int(passes), int(subbatch_bytes))

    @property
    def pipeline(self) -> int:
        """The pipeline the operator applications use now: 3 or 5."""
        return int(self._lib.ef_op_pipeline(self._h))

    def workspace(self, m: int) -> torch.Tensor:
        nbytes = self._lib.ef_op_workspace_bytes(self._h, int(m))
        return blas.workspace(nbytes, self.device, "op")

    # ---- operator applications --------------------------------------------------------
    def theta(self, Hs, out: torch.Tensor | None = None) -> torch.Tensor:
        """Θ Hs for a block (m, 2, G, G, G) (operator.py:153-155)."""
        X = self._as_block(Hs)
        m = int(X.shape[0])
        Y = torch.empty_like(X) if out is None else out
        ws = self.workspace(m)
        tm = profiling.active()
        ev = tm.begin() if tm is not None else None
        call("ef_theta", self._h, X.data_ptr(), Y.data_ptr(), m, ws.data_ptr(), ws.numel(),
             blas._stream())
        if tm is not None:
            N = self.grid_size ** 3
            tm.end("theta", ev, 32.0 * N * m + 4.0 * N, 630.0 * N * m, m)
        self.n_theta += m
        return Y

    def precondition(self, Rs, target: float = 0.0, out: torch.Tensor | None = None) -> torch.Tensor:
        """Transverse-projection preconditioner (operator.py:157-161; `target` unused)."""
        X = self._as_block(Rs)
        m = int(X.shape[0])
        Y = torch.empty_like(X) if out is None else out
        ws = self.workspace(m)
        tm = profiling.active()
        ev = tm.begin() if tm is not None else None
        call("ef_precondition", self._h, X.data_ptr(), Y.data_ptr(), m, ws.data_ptr(), ws.numel(),
             blas._stream())
        if tm is not None:
            N = self.grid_size ** 3
            tm.end("precondition", ev, 32.0 * N * m + 4.0 * N, 630.0 * N * m, m)
        return Y

    def precondition_simple(self, Rs, target: float = 0.0) -> torch.Tensor:
        """Diagonal kinetic preconditioner (operator.py:163-166)."""
        X = self._as_block(Rs)
        scale = np.float32(max(target / self.eps_mean_inv, 1e-6) * self.eps_mean_inv + 1e-6)
        Y = torch.empty_like(X)
        call("ef_precondition_simple", self._h, X.data_ptr(), Y.data_ptr(), int(X.shape[0]),
             float(scale), blas._stream())
        return Y

    # ---- conversions (operator.py:169-184) ----------------------------------------------
    def to_cartesian_spectral(self, Hs) -> torch.Tensor:
        X = self._as_block(Hs)
        t = self.basis.t
        return X[:, 0:1] * t[0][None] + X[:, 1:2] * t[1][None]

    def h_realspace(self, Hs) -> torch.Tensor:
        X = self._as_block(Hs)
        m = int(X.shape[0])
        G = self.grid_size
        H = torch.empty((m, 3, G, G, G), dtype=torch.complex64, device=self.device)
        call("ef_h_realspace", self._h, X.data_ptr(), H.data_ptr(), m, blas._stream())
        return H

    def e_realspace(self, Hs, eigvals) -> torch.Tensor:
        X = self._as_block(Hs)
        m = int(X.shape[0])
        G = self.grid_size
        lam = np.asarray(eigvals.cpu() if isinstance(eigvals, torch.Tensor) else eigvals, np.float64)
        scale = torch.from_numpy((1.0 / np.sqrt(lam)).astype(np.float32)).to(self.device)
        E = torch.empty((m, 3, G, G, G), dtype=torch.complex64, device=self.device)
        call("ef_e_realspace", self._h, X.data_ptr(), scale.data_ptr(), E.data_ptr(), m,
             blas._stream())
        return E
