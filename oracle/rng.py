"""Counter-based random blocks shared by the oracle and the CUDA library.

TEST INFRASTRUCTURE ONLY.

The reference draws its start blocks and probes with JAX's threefry
(eigenfns/solver.py:196-205, chebyshev.py:43-45, chebyshev.py:248,
scripts/exp/exp_kpm_dos.py:139-140). JAX is not available here, so both the
oracle and the CUDA library use one counter-based generator instead: element i
of stream s under seed k takes the 64-bit word mix(key(k, s) + (i+1)·φ) with
the splitmix64 finaliser. Parity against the reference is therefore assessed on
converged results, never on the random stream itself. The CUDA kernel
(`eigenfns_gb300/csrc/blas.cu`, `rng_key`/`rng_word`) computes the same words;
its float32 Box-Muller transform agrees with this one to a few ulp.
"""
from __future__ import annotations

import numpy as np

_PHI = np.uint64(0x9E3779B97F4A7C15)
_C2 = np.uint64(0xC2B2AE3D27D4EB4F)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _mix(z):
    z = np.asarray(z, np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def rng_key(seed: int, stream: int) -> np.uint64:
    with np.errstate(over="ignore"):
        s = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) * _PHI + np.uint64(stream & 0xFFFFFFFFFFFFFFFF) * _C2
        return _mix(s + np.uint64(1))


def rng_words(seed: int, stream: int, n: int) -> np.ndarray:
    key = rng_key(seed, stream)
    i = np.arange(1, n + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        return _mix(key + i * _PHI)


def _uniforms(w):
    u1 = ((w >> np.uint64(40)).astype(np.float32) + np.float32(0.5)) * np.float32(2.0 ** -24)
    u2 = (((w >> np.uint64(16)) & np.uint64(0xFFFFFF)).astype(np.float32)
          + np.float32(0.5)) * np.float32(2.0 ** -24)
    return u1, u2


def complex_normal(seed: int, stream: int, shape) -> np.ndarray:
    """Complex64 block whose real and imaginary parts are N(0,1) (Box-Muller)."""
    n = int(np.prod(shape))
    u1, u2 = _uniforms(rng_words(seed, stream, n))
    r = np.sqrt(np.float32(-2.0) * np.log(u1))
    ang = np.float32(2.0 * np.pi) * u2
    z = (r * np.cos(ang)).astype(np.float32) + 1j * (r * np.sin(ang)).astype(np.float32)
    return z.astype(np.complex64).reshape(shape)


def rademacher(seed: int, stream: int, shape, kind: str = "real") -> np.ndarray:
    """±1 probes (kind "real", the reference's) or (±1 ± i)/√2 (kind "complex")."""
    n = int(np.prod(shape))
    w = rng_words(seed, stream, n)
    re = np.where((w >> np.uint64(63)) & np.uint64(1), np.float32(-1.0), np.float32(1.0))
    if kind == "real":
        return re.astype(np.complex64).reshape(shape)
    im = np.where((w >> np.uint64(62)) & np.uint64(1), np.float32(-1.0), np.float32(1.0))
    s = np.float32(1.0 / np.sqrt(2.0))
    return (re * s + 1j * (im * s)).astype(np.complex64).reshape(shape)
