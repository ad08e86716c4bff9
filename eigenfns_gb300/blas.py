"""Block linear algebra on torch complex64 CUDA tensors through the C ABI.

Each function mirrors a reference helper of eigenfns/solver.py:
  gram      :35-43    <A_i, B_j> over the flattened vectors
  combine   :49-57    out_i = sum_j C[j, i] S_j over concatenated blocks
  rotate    tensordot(C.T, S, axes=(1, 0)) (:106, :125, :256, :261-262, :274)
  deflate   :95-110   X <- X - L (L^H X), chunk by chunk
Vectors are (m, ...) complex64 tensors; results of reductions are complex128 /
float64 device tensors. Every kernel is the library's; there is no fallback.
"""
from __future__ import annotations

import os
from contextlib import contextmanager

import numpy as np
import torch

from ._lib import call

_WS: dict = {}


try:                                    # the raw handle without torch.cuda's Python layers
    _raw_stream = torch._C._cuda_getCurrentRawStream
    _cur_device = torch._C._cuda_getDevice
except AttributeError:                  # CPU-only torch build
    _raw_stream = _cur_device = None


def _stream(device_index: int | None = None):
    """Handle of the current CUDA stream (of the current device, or of `device_index`)."""
    if _raw_stream is None:
        return torch.cuda.current_stream().cuda_stream
    return _raw_stream(_cur_device() if device_index is None else device_index)


def workspace(nbytes: int, device, slot: str = "blas") -> torch.Tensor:
    """A scratch buffer per (device, slot, stream) that only grows.

    Keyed by the current CUDA stream so solves running concurrently on different
    streams (the request server) never share scratch; work on one stream is
    ordered, so reuse within a stream is safe."""
    device = torch.device(device) if not isinstance(device, torch.device) else device
    key = (str(device), slot, _stream(device.index))
    buf = _WS.get(key)
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
        _WS[key] = buf
    return buf


def release_workspaces(stream=None) -> None:
    """Drop the scratch buffers of one stream (all streams when None)."""
    sid = None if stream is None else stream.cuda_stream
    for key in [k for k in _WS if sid is None or k[2] == sid]:
        del _WS[key]


PRECISIONS = ("mixed", "fp32")


@contextmanager
def precision(mode: str):
    """Select the arithmetic of the Gram matrices and block rotations inside the block.

    "mixed" (the default): tcgen05 tensor cores with 3xTF32 split products (fp32
    accumulation in TMEM, fp64 across K-chunks for the Gram). "fp32": CUDA-core
    kernels with plain fp32 products (fp64 split-K reduction for the Gram). The
    operator, preconditioner and recurrences are fp32 in both. The library reads the
    choice at every call (EF_GRAM_KERNEL / EF_ROTATE_KERNEL), so it applies to work
    issued inside the block from this process.
    """
    if mode not in PRECISIONS:
        raise ValueError(f"precision must be one of {PRECISIONS}, got {mode!r}")
    keys = ("EF_GRAM_KERNEL", "EF_ROTATE_KERNEL")
    saved = {k: os.environ.get(k) for k in keys}
    try:
        if mode == "fp32":
            os.environ["EF_GRAM_KERNEL"] = "simt"
            os.environ["EF_ROTATE_KERNEL"] = "simt"
        else:
            for k in keys:
                os.environ.pop(k, None)
        yield
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _c64(x: torch.Tensor) -> torch.Tensor:
    if not isinstance(x, torch.Tensor):
        raise TypeError("expected a torch tensor")
    if x.dtype != torch.complex64 or not x.is_cuda:
        raise ValueError(f"expected a complex64 CUDA tensor, got {x.dtype} on {x.device}")
    return x.contiguous()


def _rows(x: torch.Tensor):
    m = int(x.shape[0])
    K = int(x.numel() // max(m, 1))
    return m, K


def gram(A: torch.Tensor, B: torch.Tensor) -> torch.Tensor:
    """(ma, mb) complex128 device matrix <A_i, B_j>."""
    A, B = _c64(A), _c64(B)
    ma, K = _rows(A)
    mb, Kb = _rows(B)
    if K != Kb:
        raise ValueError("gram: vector sizes differ")
    out = torch.empty((ma, mb), dtype=torch.complex128, device=A.device)
    from ._lib import load
    from . import profiling
    nbytes = load().ef_gram_workspace_bytes(ma, mb, K)
    ws = workspace(nbytes, A.device, "gram")
    tm = profiling.active()
    ev = tm.begin() if tm is not None else None
    call("ef_gram", A.data_ptr(), B.data_ptr(), ma, mb, K, out.data_ptr(), ws.data_ptr(),
         ws.numel(), _stream())
    if tm is not None:
        tm.end("gram", ev, 8.0 * K * (ma + mb), 8.0 * ma * mb * K)
    return out


def gram_tc(A: torch.Tensor, B: torch.Tensor) -> tuple:
    """gram() on the tcgen05 tensor cores (3xTF32 split, TMEM accumulators): (G, err),
    err a one-int device flag that a timed-out pipeline wait sets."""
    A, B = _c64(A), _c64(B)
    ma, K = _rows(A)
    mb, Kb = _rows(B)
    if K != Kb:
        raise ValueError("gram_tc: vector sizes differ")
    out = torch.empty((ma, mb), dtype=torch.complex128, device=A.device)
    err = torch.zeros((1,), dtype=torch.int32, device=A.device)
    from ._lib import load
    ws = workspace(load().ef_gram_tc_workspace_bytes(ma, mb, K), A.device, "gram_tc")
    call("ef_gram_tc", A.data_ptr(), B.data_ptr(), ma, mb, K, out.data_ptr(), err.data_ptr(),
         ws.data_ptr(), ws.numel(), _stream())
    return out, err


def _coef(C, device) -> torch.Tensor:
    """Coefficients on the device as complex64. A host array goes through pinned staging
    and an asynchronous copy, so the host does not wait for the work queued before it."""
    if isinstance(C, torch.Tensor):
        return C.to(device=device, dtype=torch.complex64).contiguous()
    h = torch.from_numpy(np.ascontiguousarray(np.asarray(C, np.complex64)))
    return h.pin_memory().to(device, non_blocking=True)


def rotate(C, S: torch.Tensor, out: torch.Tensor | None = None, mode: int = 0) -> torch.Tensor:
    """out_i (mode 0: =, 1: +=, -1: -=) sum_j C[j, i] S_j for C (m_in, m_out)."""
    S = _c64(S)
    m_in, K = _rows(S)
    Cd = _coef(C, S.device)
    if Cd.shape[0] != m_in:
        raise ValueError(f"rotate: C has {Cd.shape[0]} rows for {m_in} vectors")
    m_out = int(Cd.shape[1])
    if out is None:
        if mode != 0:
            raise ValueError("rotate: accumulate modes need an output")
        out = torch.empty((m_out,) + tuple(S.shape[1:]), dtype=torch.complex64, device=S.device)
    from . import profiling
    tm = profiling.active()
    ev = tm.begin() if tm is not None else None
    call("ef_rotate", Cd.data_ptr(), S.data_ptr(), out.data_ptr(), m_in, m_out, K, mode, _stream())
    if tm is not None:
        tm.end("rotate", ev, 8.0 * K * (m_in + m_out * (1 if mode == 0 else 2)), 8.0 * m_in * m_out * K)
    return out


def tc_error() -> int:
    """Reads and clears the tensor-core kernels' device error flag (synchronises)."""
    import ctypes
    flag = ctypes.c_int(0)
    call("ef_tc_error", ctypes.addressof(flag))
    return int(flag.value)


def tc_error_async(host_flag: torch.Tensor) -> None:
    """Queue a copy of the tensor-core error flag into `host_flag` (a pinned int32 host
    tensor of one element) on the current stream; the flag is not cleared."""
    call("ef_tc_error_async", host_flag.data_ptr(), _stream())


def raise_on_tc_error(what: str) -> None:
    """Raise RuntimeError if a tensor-core kernel's bounded pipeline wait ran out since the
    last check (the results computed since then are not valid). Synchronises."""
    if tc_error():
        raise RuntimeError(f"{what}: a tensor-core kernel timed out waiting on its pipeline; "
                           "results invalid")


def combine(C, *blocks: torch.Tensor) -> torch.Tensor:
    Cd = _coef(C, blocks[0].device)
    out = None
    off = 0
    for Bk in blocks:
        n = int(Bk.shape[0])
        piece = Cd[off:off + n].contiguous()
        out = rotate(piece, Bk, out, 0 if out is None else 1)
        off += n
    return out


def rowdot(A: torch.Tensor, B: torch.Tensor) -> torch.Tensor:
    """complex128 (m,) <A_i, B_i>."""
    A, B = _c64(A), _c64(B)
    m, K = _rows(A)
    out = torch.empty((m,), dtype=torch.complex128, device=A.device)
    from ._lib import load
    nbytes = load().ef_rowdot_workspace_bytes(m, K)
    ws = workspace(nbytes, A.device, "rowdot")
    call("ef_rowdot", A.data_ptr(), B.data_ptr(), m, K, out.data_ptr(), ws.data_ptr(), ws.numel(),
         _stream())
    return out


def rowstats(A: torch.Tensor, B: torch.Tensor) -> torch.Tensor:
    """float64 (m, 4): Re<A_i,B_i>, Im<A_i,B_i>, |A_i|^2, |B_i|^2 in one pass."""
    A, B = _c64(A), _c64(B)
    m, K = _rows(A)
    out = torch.empty((m, 4), dtype=torch.float64, device=A.device)
    from ._lib import load
    nbytes = load().ef_rowdot_workspace_bytes(m, K)
    ws = workspace(nbytes, A.device, "rowdot")
    call("ef_rowstats", A.data_ptr(), B.data_ptr(), m, K, out.data_ptr(), ws.data_ptr(), ws.numel(),
         _stream())
    return out


def row_norms(X: torch.Tensor) -> torch.Tensor:
    return torch.sqrt(torch.clamp(rowdot(X, X).real, min=0.0))


def residual(HX: torch.Tensor, X: torch.Tensor, lam: torch.Tensor, out: torch.Tensor | None = None):
    HX, X = _c64(HX), _c64(X)
    m, K = _rows(X)
    lam = lam.to(device=X.device, dtype=torch.float64).contiguous()
    if out is None:
        out = torch.empty_like(X)
    call("ef_residual", HX.data_ptr(), X.data_ptr(), lam.data_ptr(), out.data_ptr(), m, K, _stream())
    return out


def residual_norms(HX: torch.Tensor, X: torch.Tensor, lam: torch.Tensor, out: torch.Tensor):
    """out = HX - lam X (in place into `out`); returns |out_i|^2 (float64 device)."""
    HX, X = _c64(HX), _c64(X)
    m, K = _rows(X)
    lam = lam.to(device=X.device, dtype=torch.float64).contiguous()
    r2 = torch.empty((m,), dtype=torch.float64, device=X.device)
    from ._lib import load
    ws = workspace(load().ef_rowdot_workspace_bytes(m, K), X.device, "resnorm")
    call("ef_residual_norms", HX.data_ptr(), X.data_ptr(), lam.data_ptr(), out.data_ptr(), m, K,
         r2.data_ptr(), ws.data_ptr(), ws.numel(), _stream())
    return r2


def scale_rows(X: torch.Tensor, scale: torch.Tensor) -> torch.Tensor:
    """In place X_i *= scale[i]."""
    m, K = _rows(X)
    if not X.is_contiguous():
        raise ValueError("scale_rows needs a contiguous tensor")
    scale = scale.to(device=X.device, dtype=torch.float64).contiguous()
    call("ef_scale_rows", X.data_ptr(), scale.data_ptr(), m, K, _stream())
    return X


def axpby(X: torch.Tensor, Y: torch.Tensor, a: float, b: float) -> torch.Tensor:
    """In place Y = a X + b Y."""
    X = _c64(X)
    if not Y.is_contiguous() or Y.dtype != torch.complex64:
        raise ValueError("axpby needs a contiguous complex64 output")
    call("ef_axpby", X.data_ptr(), Y.data_ptr(), int(X.numel()), float(a), float(b), _stream())
    return Y


def deflate(X: torch.Tensor, locked: torch.Tensor | None, chunk_rows: int | None = None) -> torch.Tensor:
    """X <- X - L (L^H X) over chunks of the locked set (solver.py:95-110), in place.

    `chunk_rows=None` projects against the whole locked set at once (two passes over
    it); the reference chunks only to cap a 12 GB card's transient memory."""
    if locked is None or int(locked.shape[0]) == 0:
        return X
    if not X.is_contiguous():
        raise ValueError("deflate works in place on a contiguous block")
    n = int(locked.shape[0])
    chunk_rows = n if chunk_rows is None else chunk_rows
    for s in range(0, n, chunk_rows):
        chunk = locked[s:s + chunk_rows]
        Cm = gram(chunk, X).to(torch.complex64)
        rotate(Cm, chunk, X, -1)
    return X
