"""Oracle restatement of the transverse-H Maxwell operator.

TEST INFRASTRUCTURE ONLY (the checker, never the shipped path).

Follows eigenfns/operator.py of the reference:
  make_basis                :44-79   k+G grid in numpy fftfreq order, |k+G|,
                                     transverse frame with the z->x reference
                                     switch, zeroed at k+G = 0
  _theta_block              :82-95   curl -> IFFT3 -> eps^-1 -> FFT3 -> curl^T
  _precondition_block       :98-101  diagonal kinetic preconditioner
  _precondition_fancy_block :104-127 transverse-projection preconditioner
  MaxwellOperator           :130-184

FFTs follow the numpy convention (the one jnp.fft uses): inverse carries 1/N.
complex64 operators compute their FFTs in single precision (scipy.fft keeps
the input precision), like XLA's c64 FFT; complex128 operators in double.
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np
import scipy.fft as sfft

_WORKERS = int(os.environ.get("ORACLE_FFT_WORKERS", os.cpu_count() or 1))


def set_fft_workers(n: int) -> None:
    global _WORKERS
    _WORKERS = max(1, int(n))


def _ifftn(x):
    return sfft.ifftn(x, axes=(-3, -2, -1), workers=_WORKERS)


def _fftn(x):
    return sfft.fftn(x, axes=(-3, -2, -1), workers=_WORKERS)


@dataclass(frozen=True)
class TransverseBasis:
    """Per-(k+G) frame and |k+G| (operator.py:29-41)."""

    grid_size: int
    box_size: float
    k_frac: tuple
    kn: np.ndarray   # (G,G,G) real
    t: np.ndarray    # (2,3,G,G,G) real

    @property
    def n_dof(self) -> int:
        return 2 * self.grid_size ** 3


def axis_wavevectors(grid_size: int, box_size: float, k_frac=(0.0, 0.0, 0.0)):
    """Per-axis k+G components in rad/length, fp64 (operator.py:47-49)."""
    G, L = int(grid_size), float(box_size)
    g1 = 2 * np.pi * np.fft.fftfreq(G, d=L / G)
    k0 = 2 * np.pi * np.asarray(k_frac, np.float64) / L
    return g1 + k0[0], g1 + k0[1], g1 + k0[2]


def frame_f64(grid_size: int, box_size: float, k_frac=(0.0, 0.0, 0.0)):
    """fp64 kn, t1, t2 and the reference-axis switch mask (operator.py:49-71)."""
    kx, ky, kz = axis_wavevectors(grid_size, box_size, k_frac)
    KX, KY, KZ = np.meshgrid(kx, ky, kz, indexing="ij")
    K = np.stack([KX, KY, KZ])
    kn = np.sqrt((K ** 2).sum(0))
    ref = np.zeros_like(K)
    ref[2] = 1.0
    swap = np.abs(K[2]) > 0.9 * np.maximum(kn, 1e-300)
    ref[2][swap] = 0.0
    ref[0][swap] = 1.0
    t1 = np.cross(K, ref, axis=0)
    n1 = np.linalg.norm(t1, axis=0)
    sing = n1 == 0
    n1[sing] = 1.0
    t1 /= n1
    t2 = np.cross(K, t1, axis=0)
    n2 = np.linalg.norm(t2, axis=0)
    n2[n2 == 0] = 1.0
    t2 /= n2
    t1[:, sing] = 0.0
    t2[:, sing] = 0.0
    return kn, t1, t2, swap


def make_basis(grid_size: int, box_size: float, k_frac=(0.0, 0.0, 0.0),
               rdtype=np.float32) -> TransverseBasis:
    kn, t1, t2, _ = frame_f64(grid_size, box_size, k_frac)
    return TransverseBasis(
        grid_size=int(grid_size), box_size=float(box_size),
        k_frac=tuple(float(x) for x in k_frac),
        kn=kn.astype(rdtype), t=np.stack([t1, t2]).astype(rdtype))


def _theta_block(Hs, kn, t, inv_eps):
    """Θ on a block (m,2,G,G,G) (operator.py:82-95)."""
    cdt = Hs.dtype
    a, b = Hs[:, 0], Hs[:, 1]
    c1 = (-1j * kn * b).astype(cdt)
    c2 = (1j * kn * a).astype(cdt)
    Ec = c1[:, None] * t[0][None] + c2[:, None] * t[1][None]
    E = _ifftn(Ec.astype(cdt))
    D = (inv_eps * E).astype(cdt)
    Dc = _fftn(D)
    f1 = (t[0][None] * Dc).sum(1)
    f2 = (t[1][None] * Dc).sum(1)
    return np.stack([-1j * kn * f2, 1j * kn * f1], axis=1).astype(cdt)


def _precondition_block(Rs, kn, scale):
    """R / (|k+G|^2 + s) (operator.py:98-101)."""
    return (Rs / (kn ** 2 + scale)).astype(Rs.dtype)


def _precondition_fancy_block(Rs, kn, t, eps, floor):
    """Transverse-projection preconditioner K^-1 eps K^-1 (operator.py:104-127)."""
    cdt = Rs.dtype
    a, b = Rs[:, 0], Rs[:, 1]
    knr = np.maximum(kn, floor)
    c1 = (1j * b / knr).astype(cdt)
    c2 = (-1j * a / knr).astype(cdt)
    Ec = c1[:, None] * t[0][None] + c2[:, None] * t[1][None]
    E = _ifftn(Ec.astype(cdt))
    D = (eps * E).astype(cdt)
    Dc = _fftn(D)
    f1 = (t[0][None] * Dc).sum(1)
    f2 = (t[1][None] * Dc).sum(1)
    o1 = 1j * f2 / knr
    o2 = -1j * f1 / knr
    return np.stack([o1, o2], axis=1).astype(cdt)


class MaxwellOperator:
    """Matrix-free Θ for a fixed scalar eps grid and k-point (operator.py:130-184)."""

    def __init__(self, eps: np.ndarray, box_size: float, k_frac=(0.0, 0.0, 0.0),
                 dtype=np.complex64):
        eps = np.asarray(eps)
        if eps.ndim != 3 or len(set(eps.shape)) != 1:
            raise ValueError(f"eps must be a cube, got {eps.shape}")
        self.dtype = np.dtype(dtype)
        rdtype = np.float64 if self.dtype == np.complex128 else np.float32
        self.rdtype = rdtype
        self.grid_size = eps.shape[0]
        self.box_size = float(box_size)
        self.k_frac = tuple(float(x) for x in k_frac)
        self.basis = make_basis(self.grid_size, self.box_size, k_frac, rdtype=rdtype)
        self.inv_eps = np.asarray(1.0 / eps, rdtype)
        self.eps_grid = np.asarray(eps, rdtype)
        self.eps_mean_inv = float(np.mean(1.0 / eps))
        kn_np = np.asarray(self.basis.kn)
        self.kn_floor = float(0.5 * kn_np[kn_np > 0].min())
        self.mask = (self.basis.kn > 0).astype(rdtype)

    def theta(self, Hs):
        return _theta_block(np.asarray(Hs, self.dtype), self.basis.kn, self.basis.t,
                            self.inv_eps)

    def precondition(self, Rs, target: float = 0.0):
        return _precondition_fancy_block(np.asarray(Rs, self.dtype), self.basis.kn,
                                         self.basis.t, self.eps_grid,
                                         self.rdtype(self.kn_floor))

    def precondition_simple(self, Rs, target: float = 0.0):
        scale = np.float32(max(target / self.eps_mean_inv, 1e-6) * self.eps_mean_inv + 1e-6)
        return _precondition_block(np.asarray(Rs, self.dtype), self.basis.kn, scale)

    def to_cartesian_spectral(self, Hs):
        t = self.basis.t
        Hs = np.asarray(Hs, self.dtype)
        return (Hs[:, 0:1] * t[0][None] + Hs[:, 1:2] * t[1][None]).astype(self.dtype)

    def h_realspace(self, Hs):
        return _ifftn(self.to_cartesian_spectral(Hs))

    def e_realspace(self, Hs, eigvals):
        kn, t = self.basis.kn, self.basis.t
        Hs = np.asarray(Hs, self.dtype)
        a, b = Hs[:, 0], Hs[:, 1]
        Ec = ((-1j * kn * b)[:, None] * t[0][None]
              + (1j * kn * a)[:, None] * t[1][None]).astype(self.dtype)
        E = self.inv_eps * _ifftn(Ec)
        return (E / np.sqrt(np.asarray(eigvals))[:, None, None, None, None]).astype(self.dtype)
