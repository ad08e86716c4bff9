"""fp64 eigendecompositions of the small projected problems, on the host.

The SVQB, P-whitening and Rayleigh-Ritz matrices of LOBPCG have at most a few hundred
rows. They go to LAPACK through numpy, as in the reference (eigenfns/solver.py:46-66,
281-301), with numpy's OpenBLAS held to one thread for the call: at these sizes its
worker threads cost more than they give, and two multi-threaded calls at once
oversubscribe the cores (a 96 x 96 complex eigh took 287 ms instead of 1.5 ms that way).
A stack of problems from a batch of solves runs on a pool of host threads, one core
per problem, so the single-threaded LAPACK calls of all instances proceed in parallel.
Every problem is decomposed by the same single-threaded LAPACK call whichever way it
arrives, so a solve computes the same numbers alone and in a batch.
"""
from __future__ import annotations

import ctypes
import glob
import os
import threading
from concurrent.futures import ThreadPoolExecutor
from contextlib import contextmanager

import numpy as np

_LOCK = threading.Lock()
_SETTER = None          # (get, set) of numpy's OpenBLAS thread count, or () if not found
_DEPTH = 0
_SAVED = 0
_POOL = None


def _blas_thread_control():
    """The get/set thread-count entry points of the OpenBLAS numpy was built with."""
    global _SETTER
    if _SETTER is not None:
        return _SETTER
    found = ()
    here = os.path.dirname(np.__file__)
    names = (("scipy_openblas_get_num_threads64_", "scipy_openblas_set_num_threads64_"),
             ("openblas_get_num_threads64_", "openblas_set_num_threads64_"),
             ("openblas_get_num_threads", "openblas_set_num_threads"))
    for path in sorted(glob.glob(os.path.join(here, "..", "numpy.libs", "*openblas*")) +
                       glob.glob(os.path.join(here, ".libs", "*openblas*"))):
        try:
            lib = ctypes.CDLL(path)
        except OSError:
            continue
        for g, s in names:
            if hasattr(lib, g) and hasattr(lib, s):
                get, set_ = getattr(lib, g), getattr(lib, s)
                get.restype = ctypes.c_int
                set_.argtypes = [ctypes.c_int]
                found = (get, set_)
                break
        if found:
            break
    _SETTER = found
    return _SETTER


@contextmanager
def one_blas_thread():
    """numpy's OpenBLAS runs single-threaded inside the block (re-entrant; a no-op when
    the BLAS exposes no thread control)."""
    global _DEPTH, _SAVED
    ctl = _blas_thread_control()
    if not ctl:
        yield
        return
    with _LOCK:
        if _DEPTH == 0:
            _SAVED = ctl[0]()
            ctl[1](1)
        _DEPTH += 1
    try:
        yield
    finally:
        with _LOCK:
            _DEPTH -= 1
            if _DEPTH == 0:
                ctl[1](_SAVED)


def eigh(A: np.ndarray):
    """numpy.linalg.eigh of one Hermitian matrix, single-threaded LAPACK."""
    with one_blas_thread():
        return np.linalg.eigh(A)


def _pool() -> ThreadPoolExecutor:
    global _POOL
    if _POOL is None:
        _POOL = ThreadPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1)))
    return _POOL


def eigh_many(A: np.ndarray):
    """(w, V) stacked for a stack (b, n, n) of Hermitian matrices: the problems run on
    host threads in parallel when they are large enough to pay for it (n >= 48)."""
    A = np.asarray(A)
    b, n = A.shape[0], A.shape[-1]
    w = np.empty((b, n), np.float64)
    V = np.empty(A.shape, np.result_type(A.dtype, np.complex64) if np.iscomplexobj(A) else np.float64)
    with one_blas_thread():
        if b <= 1 or n < 48:
            for i in range(b):
                w[i], V[i] = np.linalg.eigh(A[i])
        else:
            for i, (wi, Vi) in enumerate(_pool().map(np.linalg.eigh, A)):
                w[i], V[i] = wi, Vi
    return w, V
