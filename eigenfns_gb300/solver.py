"""Deflated block LOBPCG on the GPU: a drop-in for eigenfns.solver.

Follows eigenfns/solver.py of the reference step for step:
  gram / combine / deflate / ortho_block   :35-126  (library kernels, fp64 host eigh)
  lobpcg_blocks                            :136-382 residual test on the lowest
        m-guard Ritz pairs, preconditioned W deflated and orthogonalised against
        X twice, SVQB, P orthogonalised and whitened with zero rows for dropped
        directions, Rayleigh-Ritz with the dead-row penalty, re-deflation and a
        fresh Θ X every iteration, locking of the lowest m-guard pairs with the
        guard Ritz vectors carried into the next block
  lobpcg_blocks_resumable                  :385-411

Vectors stay on the device; only per-row scalars and the small Gram/RR matrices
cross to the host, where numpy's LAPACK eigh runs in fp64 as in the reference.
The locked set is a device buffer at full capacity (GB300 memory holds it), so
`locked_storage` is accepted for signature compatibility and always "gpu".

Deliberate difference: the final Rayleigh quotients are normalized by |x|^2
(`normalize_rq=True`), the correction the reference applies in its interior
path (interior.py:69-77); pass False for the reference's unnormalized values.
"""
from __future__ import annotations

import time
import warnings
from dataclasses import dataclass, field

import numpy as np
import torch

from . import blas
from .blas import combine, deflate, gram, rotate

_SVQB_DROP = 1e-5
_RR_DEAD_PENALTY = 1e4


def _flat(X):
    return X.reshape(X.shape[0], -1)


def deflate_chunk_rows(grid_size: int, target_bytes: float = 0.75e9) -> int:
    bytes_per_vec = 2 * grid_size ** 3 * 8
    return max(16, int(target_bytes // bytes_per_vec))


def svqb_coeffs(Gm: np.ndarray, drop: float = _SVQB_DROP):
    """SVQB rotation V diag(w^-1/2) from a Gram matrix, zero columns where dropped."""
    Gm = np.asarray(Gm).astype(np.complex128)
    Gm = (Gm + Gm.conj().T) / 2
    return svqb_from_eig(*np.linalg.eigh(Gm), drop)


def svqb_from_eig(w: np.ndarray, V: np.ndarray, drop: float = _SVQB_DROP):
    """The SVQB rotation from the eigendecomposition of the (symmetrised) Gram matrix."""
    keep = w > drop * max(w.max(), 1e-300)
    scale = np.where(keep, 1.0 / np.sqrt(np.where(keep, w, 1.0)), 0.0)
    return V * scale[None, :], keep


class HostEigh:
    """A step generator's request for the fp64 eigendecomposition (numpy.linalg.eigh
    convention) of a Hermitian device matrix, or of a stack (b, n, n) of them.

    The driver returns (w, V), stacked for a stack (eigenfns_gb300.hosteig: single-
    threaded LAPACK per problem, the problems of a stack on parallel host threads)."""
    __slots__ = ("A",)

    def __init__(self, A: torch.Tensor):
        self.A = A


class HostCopy:
    """A device tensor's copy into pinned host memory, queued when this is made, with an
    event behind it. A step generator that yields HostEigh(HostCopy(A)) can queue more
    device work between the two; the driver waits for this copy only, not for that
    work, so the device runs it while the host computes the eigendecomposition."""
    __slots__ = ("host", "event")

    def __init__(self, t: torch.Tensor):
        self.host = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        self.host.copy_(t, non_blocking=True)
        self.event = torch.cuda.Event()
        self.event.record()

    def numpy(self) -> np.ndarray:
        self.event.synchronize()
        return self.host.numpy()


class HostMany:
    """A step generator's request for several host reads at once: a list of device
    tensors and HostEigh requests; the driver sends back the list of their results."""
    __slots__ = ("items",)

    def __init__(self, items):
        self.items = list(items)


def _hermitian(G: torch.Tensor) -> torch.Tensor:
    return 0.5 * (G + G.conj().T)


def ortho_block(X: torch.Tensor, passes: int = 2, drop: float = _SVQB_DROP) -> torch.Tensor:
    """SVQB orthonormalisation (solver.py:113-126); dropped directions become zero rows."""
    for _ in range(passes):
        C, _ = svqb_coeffs(gram(X, X).cpu().numpy(), drop)
        X = rotate(C.astype(np.complex64), X)
    return X


def apply_chunked(fn, X: torch.Tensor, rows: int) -> torch.Tensor:
    if X.shape[0] <= rows:
        return fn(X)
    return torch.cat([fn(X[s:s + rows]) for s in range(0, X.shape[0], rows)], dim=0)


@dataclass
class SolveStats:
    theta_applications: int = 0
    rounds: list = field(default_factory=list)
    wall_seconds: float = 0.0
    iterations: int = 0


def rand_block(op, n: int, seed: int, stream: int) -> torch.Tensor:
    """Masked complex-normal block with unit rows (solver.py:196-205)."""
    X = torch.empty(op.vec_shape(n), dtype=torch.complex64, device=op.device)
    from ._lib import call, EF_RAND_NORMAL
    call("ef_rand_block", op.handle, X.data_ptr(), n, int(seed), int(stream), EF_RAND_NORMAL,
         blas._stream())
    norms = blas.row_norms(X)
    blas.scale_rows(X, 1.0 / torch.clamp(norms, min=1e-30))
    return X


def _theta(op, X, stats, out=None):
    stats.theta_applications += int(X.shape[0])
    return op.theta(X, out=out)


def _ortho_steps(X: torch.Tensor, passes: int = 2, drop: float = _SVQB_DROP, first=None):
    """SVQB on a contiguous block slot, written back into the slot (a step generator:
    it yields the one device matrix it reads on the host; `first`, the host eigh of the
    symmetrised Gram X^H X already read by the caller, replaces that read).

    The first pass is the reference's SVQB (host fp64 eigh with the 1e-5 drop). After it
    every row is unit or zero, so the second pass is a well-conditioned re-orthonormalisation
    within the same span: it runs as a device fp64 Cholesky-QR (ef_cholqr_f64, zero rows
    stay zero), which saves a device-to-host round trip and a host eigh; the Rayleigh-Ritz
    step that follows depends only on the span."""
    from . import dense
    m = int(X.shape[0])
    for p in range(passes):
        if p > 0 and m <= dense.MAX_N:
            C, _ = dense.cholqr_coeffs(gram(X, X), tol=drop)
        else:
            if p == 0 and first is not None:
                w, V = first
            else:
                w, V = yield HostEigh(_hermitian(gram(X, X)))
            C, _ = svqb_from_eig(w, V, drop)
            C = C.astype(np.complex64)
        if m <= 32:
            rotate(C, X, X)
        else:
            X.copy_(rotate(C, X))


def _ortho_inplace(X: torch.Tensor, passes: int = 2, drop: float = _SVQB_DROP) -> None:
    run_steps(_ortho_steps(X, passes, drop))


def _to_host(req):
    if isinstance(req, HostMany):
        return [_to_host(r) for r in req.items]
    if isinstance(req, HostEigh):
        from . import hosteig
        A = req.A.numpy() if isinstance(req.A, HostCopy) else req.A.cpu().numpy()
        return hosteig.eigh_many(A) if A.ndim == 3 else hosteig.eigh(A)
    if isinstance(req, tuple):
        return tuple(t.cpu().numpy() for t in req)
    return req.cpu().numpy()


def run_steps(gen):
    """Drive a step generator alone: each yielded device tensor (or tuple of tensors) is
    read on the host and sent back as numpy; returns the generator's return value."""
    try:
        req = next(gen)
        while True:
            req = gen.send(_to_host(req))
    except StopIteration as stop:
        return stop.value


def _normalize_rows(X: torch.Tensor, floor: float) -> None:
    st = blas.rowstats(X, X)
    blas.scale_rows(X, 1.0 / torch.clamp(torch.sqrt(torch.clamp(st[:, 2], min=0.0)), min=floor))


def _rr_gram(act: torch.Tensor, hact: torch.Tensor, m: int) -> torch.Tensor:
    """Rayleigh-Ritz matrix act^H (Θ act) of the active basis (m-row blocks).

    Θ is Hermitian, so only the block upper triangle is computed (block row i against
    the image blocks i..end, reading 2/3 of the rows a full Gram reads at three blocks)
    and the lower triangle is its conjugate transpose; the caller symmetrises the
    diagonal blocks as the reference does (solver.py:281-301).
    """
    nb = int(act.shape[0])
    if nb % m or nb // m < 2:
        return gram(act, hact)
    A = torch.empty((nb, nb), dtype=torch.complex128, device=act.device)
    for i in range(0, nb, m):
        blk = gram(act[i:i + m], hact[i:])
        A[i:i + m, i:] = blk
        if i + m < nb:
            A[i + m:, i:i + m] = blk[:, m:].conj().T
    return A


def _ritz_request(X, HX, R, normalize: bool) -> torch.Tensor:
    """Queue the per-row (lam, |x|^2, |Θx|^2, |R|^2) of X, with R = HX - lam X written
    into `R`: one pass for <x, Θx>, |x|^2, |Θx|^2 and one fused pass for R and |R|^2."""
    st = blas.rowstats(X, HX)
    lam_d = st[:, 0] / torch.clamp(st[:, 2], min=1e-30) if normalize else st[:, 0].contiguous()
    r2 = blas.residual_norms(HX, X, lam_d, R)
    return torch.cat([lam_d[:, None], st[:, 2:4], r2[:, None]], dim=1)


def _ritz_from_host(h):
    """(lam, relres, |x|) from the host copy of a _ritz_request."""
    lam, xx, hh, rr = h[..., 0], h[..., 1], h[..., 2], h[..., 3]
    rn = np.sqrt(np.maximum(rr, 0.0)) / np.maximum(np.sqrt(np.maximum(hh, 0.0)), 1e-30)
    return lam, rn, np.sqrt(np.maximum(xx, 0.0))


def _ritz_steps(X, HX, R, normalize: bool):
    """(lam, relres, |x|) for the rows of X, with R = HX - lam X written into `R`; the
    small per-row vectors reach the host in a single copy (the one yield)."""
    return _ritz_from_host((yield _ritz_request(X, HX, R, normalize)))


def lobpcg_steps(op, nev: int, m: int = 96, guard: int = 48, tol: float = 1e-4,
                 maxit: int = 400, seed: int = 0, precond_shift: str = "median",
                 verbose: bool = True, log_every: int = 0, initial_locked=None,
                 initial_vals=None, on_block=None, locked_storage: str = "auto",
                 theta_chunk: int = 0, normalize_rq: bool = True, deflate_chunk: int | None = None,
                 autotune: bool | None = None, check_tc: bool = True):
    """Bottom-up deflated block LOBPCG as a step generator (see lobpcg_blocks).

    Every point where the algorithm needs device data on the host (residuals, the SVQB
    and P-whitening Grams, the Rayleigh-Ritz matrix) is a `yield` of the device tensor(s);
    the driver sends back the numpy copy. run_steps drives one solve; the batched driver
    (eigenfns_gb300.batched) advances many solves between one shared host transfer.

    `autotune` (default: on when EF_AUTOTUNE=1) times the operator pipeline and the
    Gram schedules of this block size once on the running GPU before the solve and
    reuses the cached choice afterwards (eigenfns_gb300.tune). Left at None without
    EF_AUTOTUNE, a pipeline stored by an earlier tuning of this grid edge and block
    size is applied without timing; False leaves the operator as it is.

    Working set: two (3m, 2, G, G, G) slabs holding the blocks as [P; X; W] (the
    Rayleigh-Ritz basis is contiguous, so its Gram is one call and the Ritz
    combination writes [P_new; X_new] in one pass into the other slab) and one
    slab of operator images [ΘP; ΘX; ΘW]. The basis order [P, X, W] is a
    permutation of the reference's [X, W, P]; the Ritz pairs are the same.
    """
    G = op.grid_size
    dev = op.device
    from . import tune
    if tune.enabled(autotune) and hasattr(op, "configure"):
        tune.autotune(op, m)
    elif autotune is None:
        tune.apply_cached(op, m)        # a pipeline chosen earlier on this GPU, if any
    vshape = op.vec_shape(1)[1:]
    cap = int(np.ceil(nev / max(m - guard, 1))) * (m - guard) + m
    n_init = 0 if initial_locked is None else int(initial_locked.shape[0])
    locked_buf = torch.zeros((max(cap, n_init + nev),) + vshape, dtype=torch.complex64, device=dev)
    n_locked_now = 0
    if initial_locked is not None:
        il = initial_locked
        if not isinstance(il, torch.Tensor):
            il = torch.from_numpy(np.ascontiguousarray(np.asarray(il, np.complex64)))
        locked_buf[:n_init] = il.to(dev)
        n_locked_now = n_init
    locked_vals = (np.empty((0,)) if initial_vals is None
                   else np.asarray(initial_vals, np.float64))
    slabs = [torch.empty((3 * m,) + vshape, dtype=torch.complex64, device=dev) for _ in range(2)]
    HS = torch.empty((3 * m,) + vshape, dtype=torch.complex64, device=dev)
    HP, HX, HW = HS[0:m], HS[m:2 * m], HS[2 * m:3 * m]
    stats = SolveStats()
    t0 = time.perf_counter()
    carry = None
    block_no = 0
    cur = 0
    while locked_vals.size < nev:
        locked = locked_buf[:n_locked_now] if n_locked_now > 0 else None
        S = slabs[cur]
        P, X, W = S[0:m], S[m:2 * m], S[2 * m:3 * m]
        nc = 0 if carry is None else int(carry.shape[0])
        if nc:
            X[:nc] = carry
        if nc < m:
            Xr = X[nc:]
            from ._lib import call, EF_RAND_NORMAL
            call("ef_rand_block", op.handle, Xr.data_ptr(), m - nc, int(seed), int(block_no),
                 EF_RAND_NORMAL, blas._stream())
            _normalize_rows(Xr, 1e-30)
        block_no += 1
        deflate(X, locked, deflate_chunk)
        yield from _ortho_steps(X)
        _theta(op, X, stats, out=HX)
        have_p = False
        n_lock = min(m - guard, nev - locked_vals.size)
        it = 0
        for it in range(maxit):
            # R = HX - lam X lands in the W slot, where the preconditioner needs it. The
            # iteration's work up to the first SVQB Gram of W touches W only, so it is
            # queued before the convergence test and both reach the host in one read (if
            # the block has converged, W is recomputed at the block's end).
            ritz = _ritz_request(X, HX, W, False)
            op.precondition(W, out=W)
            deflate(W, locked, deflate_chunk)
            for _ in range(2):
                rotate(gram(X, W).to(torch.complex64), X, W, -1)
            h, eig_w = yield HostMany([ritz, HostEigh(_hermitian(gram(W, W)))])
            lam, rn, xnorm = _ritz_from_host(h)
            dead_rows = xnorm < 0.5
            lam_h = np.where(dead_rows, np.inf, lam)
            rn = np.where(dead_rows, np.inf, rn)
            order = np.argsort(lam_h)
            if (rn[order[:n_lock]] < tol).all():
                break
            if log_every and it % log_every == 0 and verbose:
                lo = np.sort(lam_h)
                print(f"    it {it:3d}  lam[0,{n_lock-1},{m-1}] = {lo[0]:.4f} {lo[n_lock-1]:.4f} "
                      f"{lo[-1]:.4f}  res q50/q90 {np.quantile(rn, 0.5):.1e}/{np.quantile(rn, 0.9):.1e}",
                      flush=True)
            stats.iterations += 1
            yield from _ortho_steps(W, first=eig_w)
            if have_p:
                XW = S[m:3 * m]
                for _ in range(2):
                    rotate(gram(XW, P).to(torch.complex64), XW, P, -1)
                Gp = HostCopy(_hermitian(gram(P, P)))
                # Θ W depends on W alone: queued behind the copy of P's Gram, it runs on
                # the device while the host does P's eigh
                _theta(op, W, stats, out=HW)
                Tp, keepp = svqb_from_eig(*(yield HostEigh(Gp)))
                if not keepp.any():
                    have_p = False
                elif m <= 32:
                    rotate(Tp.astype(np.complex64), P, P)
                else:
                    P.copy_(rotate(Tp.astype(np.complex64), P))
            else:
                _theta(op, W, stats, out=HW)
            if have_p:
                _theta(op, P, stats, out=HP)
                act, hact, off = S, HS, 0
            else:
                act, hact, off = S[m:3 * m], HS[m:3 * m], m
            nb = int(act.shape[0])
            A_d = _rr_gram(act, hact, m)
            rows_d = blas.rowstats(act, act)[:, 2]
            # symmetrise and lift dead rows (|x| < 0.5) by the reference's penalty
            # (solver.py:281-301) on the device, then the fp64 eigh on the host
            A_s = _hermitian(A_d)
            dead = torch.sqrt(torch.clamp(rows_d, min=0.0)) < 0.5
            penalty = torch.clamp(100.0 * A_s.diagonal().abs().max(), min=_RR_DEAD_PENALTY)
            A_s.diagonal().add_(torch.where(dead, penalty, torch.zeros_like(penalty)).to(A_s.dtype))
            wA, VA = yield HostEigh(A_s)
            Cm = VA[:, :m]
            Cp = Cm.copy()
            x_rows = slice(m - off, 2 * m - off)   # rows of the X block inside the active basis
            Cp[x_rows] = 0
            Ccat = np.concatenate([Cp, Cm], axis=1).astype(np.complex64)
            Sn = slabs[1 - cur]
            rotate(Ccat, act, Sn[0:2 * m])
            cur = 1 - cur
            S = Sn
            P, X, W = S[0:m], S[m:2 * m], S[2 * m:3 * m]
            have_p = True
            deflate(X, locked, deflate_chunk)
            _normalize_rows(S[0:2 * m], 1e-20)
            _theta(op, X, stats, out=HX)
        _theta(op, X, stats, out=HX)
        lam, rn, xnorm = yield from _ritz_steps(X, HX, W, normalize_rq)
        lam = np.where(xnorm < 0.5, np.inf, lam)
        rn = np.where(xnorm < 0.5, np.inf, rn)
        order = np.argsort(lam)
        if not np.isfinite(lam[order[:n_lock]]).all():
            raise RuntimeError(
                f"block produced only {int(np.isfinite(lam).sum())} live Ritz "
                f"pairs but needs {n_lock} to lock — rank collapse")
        lock_idx = torch.from_numpy(np.asarray(order[:n_lock])).pin_memory().to(dev, non_blocking=True)
        carry_idx = torch.from_numpy(np.asarray(order[n_lock:])).pin_memory().to(dev, non_blocking=True)
        Xl = X.index_select(0, lock_idx)
        carry = X.index_select(0, carry_idx)
        locked_buf[n_locked_now:n_locked_now + n_lock] = Xl
        n_locked_now += n_lock
        locked_vals = np.concatenate([locked_vals, lam[order[:n_lock]]])
        stats.rounds.append({"iters": it + 1, "locked": int(locked_vals.size),
                             "max_res_locked": float(rn[order[:n_lock]].max())})
        if on_block is not None:
            on_block(int(locked_vals.size), lam[order[:n_lock]], Xl.cpu().numpy())
        if verbose:
            print(f"  locked {locked_vals.size:4d}/{nev} (+{n_lock})  iters {it + 1:3d}  "
                  f"worst res {rn[order[:n_lock]].max():.1e}  "
                  f"elapsed {time.perf_counter() - t0:6.1f}s", flush=True)
        del Xl
    del slabs, HS
    if check_tc:
        torch.cuda.synchronize(dev)
        if blas.tc_error():
            raise RuntimeError("a tensor-core kernel timed out waiting on its pipeline; results invalid")
    stats.wall_seconds = time.perf_counter() - t0
    if locked_vals.size > 1 and (np.diff(locked_vals) < -1e-6 * np.abs(locked_vals[1:])).any():
        warnings.warn("locked eigenvalues non-monotone: a band was recovered out of order; "
                      "re-sorting", RuntimeWarning)
    order = np.argsort(locked_vals, kind="stable")
    locked = locked_buf[:n_locked_now].index_select(0, torch.from_numpy(order).to(dev))
    return locked_vals[order][:nev], locked, stats


def lobpcg_blocks(op, nev: int, m: int = 96, guard: int = 48, tol: float = 1e-4,
                  maxit: int = 400, seed: int = 0, precond_shift: str = "median",
                  verbose: bool = True, log_every: int = 0, initial_locked=None,
                  initial_vals=None, on_block=None, locked_storage: str = "auto",
                  theta_chunk: int = 0, normalize_rq: bool = True, deflate_chunk: int | None = None,
                  autotune: bool | None = None):
    """Bottom-up deflated block LOBPCG. Returns (eigenvalues, locked_vectors, stats).

    `autotune` (default: on when EF_AUTOTUNE=1) times the operator pipeline and the
    Gram schedules of this block size once on the running GPU before the solve and
    reuses the cached choice afterwards (eigenfns_gb300.tune).

    Working set: two (3m, 2, G, G, G) slabs holding the blocks as [P; X; W] (the
    Rayleigh-Ritz basis is contiguous, so its Gram is one call and the Ritz
    combination writes [P_new; X_new] in one pass into the other slab) and one
    slab of operator images [ΘP; ΘX; ΘW]. The basis order [P, X, W] is a
    permutation of the reference's [X, W, P]; the Ritz pairs are the same.
    """
    return run_steps(lobpcg_steps(op, nev, m=m, guard=guard, tol=tol, maxit=maxit, seed=seed,
                                  precond_shift=precond_shift, verbose=verbose, log_every=log_every,
                                  initial_locked=initial_locked, initial_vals=initial_vals,
                                  on_block=on_block, locked_storage=locked_storage,
                                  theta_chunk=theta_chunk, normalize_rq=normalize_rq,
                                  deflate_chunk=deflate_chunk, autotune=autotune))


def lobpcg_blocks_resumable(op, nev, checkpointer=None, resume=False, **kw):
    """`lobpcg_blocks` with per-block checkpointing and auto-resume (solver.py:385-411)."""
    if checkpointer is None:
        return lobpcg_blocks(op, nev, **kw)
    init_vals = init_vecs = None
    n_blocks = 0
    if resume:
        init_vals, init_vecs, n_blocks, _ = checkpointer.load()
        if init_vals is not None and len(init_vals) >= nev:
            return (init_vals[:nev], torch.from_numpy(init_vecs[:nev]).to(op.device), SolveStats())
    state = {"i": n_blocks}

    def on_block(n_locked_total, lam_block, X_block):
        checkpointer.save_block(state["i"], lam_block, X_block, extra={"n_locked": n_locked_total})
        state["i"] += 1

    return lobpcg_blocks(op, nev, initial_locked=init_vecs, initial_vals=init_vals,
                         on_block=on_block, **kw)
