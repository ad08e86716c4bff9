"""Oracle restatement of the deflated block LOBPCG.

TEST INFRASTRUCTURE ONLY (the checker, never the shipped path).

Follows eigenfns/solver.py of the reference:
  gram                 :35-43    <A_i, B_j> over the flattened vector
  combine              :49-57    out_i = sum_j C[j, i] S_j over concatenated blocks
  apply_chunked        :74-82
  deflate_chunk_rows   :85-92
  deflate              :95-110   X <- X - L (L^H X), chunk by chunk
  ortho_block          :113-126  SVQB, host fp64 eigh, drop 1e-5, zero rows
  lobpcg_blocks        :136-382  block loop, residual test, preconditioned W,
                                 P whitening, RR with dead-row penalty, locking
                                 of the lowest m-guard pairs, guard carry

Random start blocks come from `oracle.rng` (JAX's threefry is unavailable),
so iterates are compared on converged values and subspaces.

`normalize_rq=True` divides the final Rayleigh quotient by |x|^2, the fix the
reference applies in its interior path (eigenfns/interior.py:69-77); with
False the final values are the reference's unnormalized <x, Θx>
(solver.py:317).
"""
from __future__ import annotations

import time
import warnings
from dataclasses import dataclass, field

import numpy as np

from .rng import complex_normal

_SVQB_DROP = 1e-5
_RR_DEAD_PENALTY = 1e4


def _flat(X):
    return X.reshape(X.shape[0], -1)


def gram(A, B):
    return _flat(A).conj() @ _flat(B).T


def combine(C, *blocks):
    """out_i = sum_j C[j, i] S_j (solver.py:49-57)."""
    m = blocks[0].shape[0]
    shape = blocks[0].shape[1:]
    C = np.asarray(C)
    out = C[:m].T.astype(blocks[0].dtype) @ _flat(blocks[0])
    off = m
    for Bk in blocks[1:]:
        out = out + C[off:off + Bk.shape[0]].T.astype(Bk.dtype) @ _flat(Bk)
        off += Bk.shape[0]
    return out.reshape((C.shape[1],) + shape)


def rotate(C, X):
    """tensordot(C.T, X, axes=(1, 0)) : out_i = sum_j C[j, i] X_j."""
    return (np.asarray(C).T.astype(X.dtype) @ _flat(X)).reshape((C.shape[1],) + X.shape[1:])


def apply_chunked(fn, X, rows: int):
    if X.shape[0] <= rows:
        return fn(X)
    return np.concatenate([fn(X[s:s + rows]) for s in range(0, X.shape[0], rows)], axis=0)


def deflate_chunk_rows(grid_size: int, target_bytes: float = 0.75e9) -> int:
    bytes_per_vec = 2 * grid_size ** 3 * 8
    return max(16, int(target_bytes // bytes_per_vec))


def deflate(X, locked, chunk_rows: int = 128):
    if locked is None or locked.shape[0] == 0:
        return X
    for s in range(0, locked.shape[0], chunk_rows):
        chunk = locked[s:s + chunk_rows]
        C = gram(chunk, X)
        X = X - rotate(C, chunk)
    return X


def svqb_coeffs(Gm, drop=_SVQB_DROP):
    """SVQB rotation from a Gram matrix: V diag(w^-1/2), zero columns dropped."""
    Gm = np.asarray(Gm).astype(np.complex128)
    Gm = (Gm + Gm.conj().T) / 2
    w, V = np.linalg.eigh(Gm)
    keep = w > drop * max(w.max(), 1e-300)
    scale = np.where(keep, 1.0 / np.sqrt(np.where(keep, w, 1.0)), 0.0)
    return V * scale[None, :], keep


def ortho_block(X, passes: int = 2, drop: float = _SVQB_DROP):
    for _ in range(passes):
        C, _ = svqb_coeffs(gram(X, X), drop)
        X = rotate(C.astype(X.dtype), X)
    return X


def row_norms(X):
    return np.linalg.norm(_flat(X), axis=1)


def rayleigh(X, HX, normalize: bool):
    lam = np.real(np.sum(_flat(X).conj() * _flat(HX), axis=1)).astype(np.float64)
    if normalize:
        xn2 = np.real(np.sum(np.abs(_flat(X)) ** 2, axis=1)).astype(np.float64)
        lam = lam / np.maximum(xn2, 1e-30)
    return lam


@dataclass
class SolveStats:
    theta_applications: int = 0
    rounds: list = field(default_factory=list)
    wall_seconds: float = 0.0
    timeline: list = field(default_factory=list)   # (event, perf_counter)


def rand_block(op, seed: int, stream: int, n: int):
    G = op.grid_size
    Z = complex_normal(seed, stream, (n, 2, G, G, G)).astype(op.dtype)
    Z = Z * op.mask[None, None]
    ns = 1.0 / np.maximum(row_norms(Z), 1e-30)
    return (Z * ns[:, None, None, None, None]).astype(op.dtype)


def lobpcg_blocks(op, nev: int, m: int = 96, guard: int = 48, tol: float = 1e-4,
                  maxit: int = 400, seed: int = 0, verbose: bool = False,
                  initial_locked=None, initial_vals=None, on_block=None,
                  theta_chunk: int = 0, normalize_rq: bool = True,
                  max_iters_total: int | None = None):
    G = op.grid_size
    mask = op.mask[None, None]
    chunk_rows = deflate_chunk_rows(G)
    if theta_chunk <= 0:
        theta_chunk = max(4, int(1e9 // (3 * G ** 3 * 8)))
    locked_list = []
    if initial_locked is not None:
        locked_list.append(np.asarray(initial_locked, op.dtype))
    locked_vals = (np.empty((0,)) if initial_vals is None
                   else np.asarray(initial_vals, np.float64))
    stats = SolveStats()
    t0 = time.perf_counter()
    carry = None
    block_no = 0
    iters_total = 0
    while locked_vals.size < nev:
        locked = np.concatenate(locked_list, axis=0) if locked_list else None
        if carry is not None and carry.shape[0] > 0:
            X = np.concatenate([carry, rand_block(op, seed, block_no, m)[:m - carry.shape[0]]])
        else:
            X = rand_block(op, seed, block_no, m)
        block_no += 1
        X = ortho_block(deflate(X, locked, chunk_rows))
        HX = apply_chunked(op.theta, X, theta_chunk)
        stats.theta_applications += m
        stats.timeline.append(("block_ready", time.perf_counter()))
        P = None
        n_lock = min(m - guard, nev - locked_vals.size)
        it = 0
        for it in range(maxit):
            lam = rayleigh(X, HX, False)
            R = HX - lam.astype(np.float32 if op.dtype == np.complex64 else np.float64)[:, None, None, None, None] * X
            rn = row_norms(R) / np.maximum(row_norms(HX), 1e-30)
            xnorm = row_norms(X)
            dead_rows = xnorm < 0.5
            lam_h = np.where(dead_rows, np.inf, lam)
            rn = np.where(dead_rows, np.inf, rn)
            order = np.argsort(lam_h)
            if (rn[order[:n_lock]] < tol).all():
                break
            if max_iters_total is not None and iters_total >= max_iters_total:
                break
            iters_total += 1
            stats.timeline.append(("iter_start", time.perf_counter()))
            W = (apply_chunked(op.precondition, R, theta_chunk) * mask).astype(op.dtype)
            del R
            W = deflate(W, locked, chunk_rows)
            for _ in range(2):
                W = W - rotate(gram(X, W), X)
            W = ortho_block(W)
            if P is not None:
                for _ in range(2):
                    P = P - rotate(gram(X, P), X) - rotate(gram(W, P), W)
                Tp, keepp = svqb_coeffs(gram(P, P))
                if not keepp.any():
                    P = None
                else:
                    P = rotate(Tp.astype(op.dtype), P)
            blocks = [X, W] if P is None else [X, W, P]
            nb = len(blocks) * m
            A = np.zeros((nb, nb), np.complex128)
            for bi, Bk in enumerate(blocks):
                A[bi * m:(bi + 1) * m, 0:m] = gram(Bk, HX)
            col = m
            for Bsrc in blocks[1:]:
                for s in range(0, m, theta_chunk):
                    piece = Bsrc[s:s + theta_chunk]
                    Hc = op.theta(piece)
                    stats.theta_applications += int(piece.shape[0])
                    for bi, Bk in enumerate(blocks):
                        A[bi * m:(bi + 1) * m, col + s:col + s + piece.shape[0]] = gram(Bk, Hc)
                col += m
            A = (A + A.conj().T) / 2
            rownorm = np.concatenate([row_norms(Bk) for Bk in blocks])
            dead = rownorm < 0.5
            penalty = max(_RR_DEAD_PENALTY, 100.0 * float(np.abs(np.diag(A)).max()))
            A[np.diag_indices_from(A)] += np.where(dead, penalty, 0.0)
            wA, VA = np.linalg.eigh(A)
            C = VA[:, :m].astype(op.dtype)
            Xn = combine(C, *blocks)
            Xn = deflate(Xn, locked, chunk_rows)
            Xn = Xn * (1.0 / np.maximum(row_norms(Xn), 1e-20)).astype(op.rdtype)[:, None, None, None, None]
            Cp = C.copy()
            Cp[:m] = 0
            P = combine(Cp, *blocks)
            P = P * (1.0 / np.maximum(row_norms(P), 1e-20)).astype(op.rdtype)[:, None, None, None, None]
            X = Xn
            HX = apply_chunked(op.theta, X, theta_chunk)
            stats.theta_applications += m
            stats.timeline.append(("iter_end", time.perf_counter()))
        HX = apply_chunked(op.theta, X, theta_chunk)
        stats.theta_applications += m
        lam = rayleigh(X, HX, normalize_rq)
        Rf = HX - lam.astype(op.rdtype)[:, None, None, None, None] * X
        rn = row_norms(Rf) / np.maximum(row_norms(HX), 1e-30)
        xnorm = row_norms(X)
        lam = np.where(xnorm < 0.5, np.inf, lam)
        rn = np.where(xnorm < 0.5, np.inf, rn)
        order = np.argsort(lam)
        if not np.isfinite(lam[order[:n_lock]]).all():
            raise RuntimeError(
                f"block produced only {int(np.isfinite(lam).sum())} live Ritz "
                f"pairs but needs {n_lock} to lock — rank collapse")
        lock_idx = order[:n_lock]
        carry_idx = order[n_lock:]
        Xl = X[lock_idx]
        carry = X[carry_idx]
        locked_list.append(Xl)
        locked_vals = np.concatenate([locked_vals, lam[lock_idx]])
        stats.rounds.append({"iters": it + 1, "locked": int(locked_vals.size),
                             "max_res_locked": float(rn[lock_idx].max())})
        if on_block is not None:
            on_block(int(locked_vals.size), lam[lock_idx], Xl)
        if verbose:
            print(f"  locked {locked_vals.size}/{nev} iters {it + 1} "
                  f"worst res {rn[lock_idx].max():.1e}", flush=True)
        if max_iters_total is not None and iters_total >= max_iters_total:
            break
    stats.wall_seconds = time.perf_counter() - t0
    if locked_vals.size > 1 and (np.diff(locked_vals) < -1e-6 * np.abs(locked_vals[1:])).any():
        warnings.warn("locked eigenvalues non-monotone; re-sorting", RuntimeWarning)
    order = np.argsort(locked_vals, kind="stable")
    locked = np.concatenate(locked_list, axis=0)[order]
    return locked_vals[order][:nev], locked, stats
