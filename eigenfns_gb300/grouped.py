"""Grouped deflated block LOBPCG: solves of one shape advanced by one set of launches.

Many small eigensolves (k-points, seeds, structures of one size) spend most of their
time in the host work between launches, not on the GPU. A group holds B solves with
the same grid edge, block size m and guard in stacked device arrays (instance i's
[P; X; W] slab, its operator images and its locked set at a fixed stride) and runs
every operation of an iteration for all of them with one host call
(ef_group_* in the C library: the single-instance operation on each instance's
operands, queued back to back on one stream). The fp64 projected problems of all
instances go to the host as one stack (eigenfns_gb300.hosteig runs them on parallel
host threads), and one host read per request serves the whole group.

Each instance follows eigenfns_gb300.solver.lobpcg_steps (itself the reference's
eigenfns/solver.py:136-382) step for step with the same kernels on the same operands
and the same host arithmetic, so its eigenpairs, iteration counts and locked vectors
are those of the instance solved alone. Instances differ only in their data and in
when they converge: an instance whose block has converged is set aside (its X and
ΘX untouched) while the others iterate, and every instance's block is finalised and
locked together when the last one converges. Instances may ask for different band
counts; one that has all its bands leaves the group at that block boundary.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np
import torch

from . import blas, dense
from ._lib import EF_RAND_NORMAL, call, load
from .solver import (_RR_DEAD_PENALTY, _SVQB_DROP, HostCopy, HostEigh, HostMany, SolveStats,
                     _ritz_from_host,
                     svqb_from_eig)


class GroupResults:
    """Results of members of a group that have finished: {member: (vals, vecs, stats) or
    the exception that ended that member}. A grouped solve yields one whenever members
    finish at a block boundary (the driver records them and resumes the group at once)
    and returns one for the members left at the end."""
    __slots__ = ("results",)

    def __init__(self, results: dict):
        self.results = results


def _ptr(t: torch.Tensor) -> int:
    return t.data_ptr()


class _Stack:
    """Launch helpers over the stacked per-instance tensors of one group."""

    def __init__(self, ops, device):
        self.ops = ops
        self.device = device
        self.handles = (ctypes.c_void_p * len(ops))(*[op.handle.value for op in ops])
        self.G = ops[0].grid_size
        self.K = 2 * self.G ** 3
        self.lib = load()

    @staticmethod
    def ids(idx) -> np.ndarray:
        return np.ascontiguousarray(idx, dtype=np.int32)

    def _ws(self, nbytes, slot):
        return blas.workspace(nbytes, self.device, slot)

    # instance strides in complex values come from dimension 0 of each stacked view
    def theta(self, idx, X, Y, m, precondition=False):
        ws = self._ws(max(self.lib.ef_op_workspace_bytes(op.handle, int(m)) for op in self.ops), "op")
        i = self.ids(idx)
        call("ef_group_precondition" if precondition else "ef_group_theta",
             ctypes.addressof(self.handles), i.ctypes.data, len(i), _ptr(X), X.stride(0), _ptr(Y),
             Y.stride(0), int(m), _ptr(ws), ws.numel(), blas._stream())
        for j in i:
            self.ops[j].n_theta += 0 if precondition else int(m)

    def gram(self, idx, A, B, ma, mb, out=None):
        """(B_all, ma, mb) complex128: rows idx filled with <A_i, B_i>."""
        if out is None:
            out = torch.empty((len(self.ops), ma, mb), dtype=torch.complex128, device=self.device)
        ws = self._ws(self.lib.ef_gram_workspace_bytes(int(ma), int(mb), self.K), "gram")
        i = self.ids(idx)
        call("ef_group_gram", i.ctypes.data, len(i), _ptr(A), A.stride(0), _ptr(B), B.stride(0),
             int(ma), int(mb), self.K, _ptr(out), out.stride(0), _ptr(ws), ws.numel(), blas._stream())
        return out

    def rotate(self, idx, C, S, out, m_in, m_out, mode=0):
        """out_i (=, +=, -=) C_i^T-combination of S_i's rows (ef_rotate per instance);
        C (B_all, m_in, m_out) complex64 on the device."""
        i = self.ids(idx)
        call("ef_group_rotate", i.ctypes.data, len(i), _ptr(C), C.stride(0), _ptr(S), S.stride(0),
             _ptr(out), out.stride(0), int(m_in), int(m_out), self.K, int(mode), blas._stream())

    def rowstats(self, idx, A, B, m):
        out = torch.empty((len(self.ops), m, 4), dtype=torch.float64, device=self.device)
        ws = self._ws(self.lib.ef_rowdot_workspace_bytes(int(m), self.K), "rowdot")
        i = self.ids(idx)
        call("ef_group_rowstats", i.ctypes.data, len(i), _ptr(A), A.stride(0), _ptr(B), B.stride(0),
             int(m), self.K, _ptr(out), out.stride(0), _ptr(ws), ws.numel(), blas._stream())
        return out

    def residual_norms(self, idx, HX, X, lam, R, m):
        r2 = torch.empty((len(self.ops), m), dtype=torch.float64, device=self.device)
        ws = self._ws(self.lib.ef_rowdot_workspace_bytes(int(m), self.K), "resnorm")
        i = self.ids(idx)
        call("ef_group_residual_norms", i.ctypes.data, len(i), _ptr(HX), HX.stride(0), _ptr(X),
             X.stride(0), _ptr(lam), lam.stride(0), _ptr(R), R.stride(0), int(m), self.K, _ptr(r2),
             r2.stride(0), _ptr(ws), ws.numel(), blas._stream())
        return r2

    def scale_rows(self, idx, X, scale, m):
        i = self.ids(idx)
        call("ef_group_scale_rows", i.ctypes.data, len(i), _ptr(X), X.stride(0), _ptr(scale),
             scale.stride(0), int(m), self.K, blas._stream())

    def upload(self, idx, C_host: np.ndarray, shape) -> torch.Tensor:
        """Coefficient matrices of the instances idx (C_host stacked in idx order) as a
        (B_all, *shape) complex64 device array."""
        full = np.zeros((len(self.ops),) + tuple(shape), np.complex64)
        full[np.asarray(idx)] = C_host
        pinned = torch.from_numpy(full).pin_memory()
        return pinned.to(self.device, non_blocking=True)


def _to_device(a: np.ndarray, dev) -> torch.Tensor:
    """A small host array on the device without waiting for the stream (pinned staging)."""
    return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().to(dev, non_blocking=True)


def _hermitian(A: torch.Tensor) -> torch.Tensor:
    return 0.5 * (A + A.conj().transpose(-2, -1))


def lobpcg_group_steps(ops, nevs, keys=None, m: int = 32, guard: int = 8, tol: float = 1e-4,
                       maxit: int = 400, seeds=None, normalize_rq: bool = True):
    """Grouped block LOBPCG as a step generator (driven by run_steps or the batch driver).

    `ops`: MaxwellOperators of one grid edge on one device; `nevs` bands per instance (an
    int applies to all); `seeds` per instance; `keys` names the members in the
    GroupResults this yields and returns (default 0..B-1). Each member's result is
    (eigenvalues, locked vectors, SolveStats) as lobpcg_blocks(op, nev, m, guard, tol,
    maxit, seed) returns it alone, or the exception that ended that member.
    """
    B = len(ops)
    if B == 0:
        return GroupResults({})
    G = ops[0].grid_size
    dev = ops[0].device
    if any(op.grid_size != G or op.device != dev for op in ops):
        raise ValueError("a group needs one grid edge and one device")
    per = lambda v: list(v) if isinstance(v, (list, tuple, np.ndarray)) else [v] * B
    nevs = [int(v) for v in per(nevs)]
    seeds = [int(s) for s in per(0 if seeds is None else seeds)]
    keys = list(range(B)) if keys is None else list(keys)
    from . import tune
    for op in ops:                      # the pipeline a solve alone would use (solver.lobpcg_steps)
        tune.apply_cached(op, m)
    st = _Stack(ops, dev)
    vshape = ops[0].vec_shape(1)[1:]
    nl = m - guard
    cap = max(int(np.ceil(nev / max(nl, 1))) * nl + m for nev in nevs)
    locked_buf = torch.zeros((B, cap) + vshape, dtype=torch.complex64, device=dev)
    slabs = [torch.empty((B, 3 * m) + vshape, dtype=torch.complex64, device=dev) for _ in range(2)]
    HS = torch.empty((B, 3 * m) + vshape, dtype=torch.complex64, device=dev)
    HP, HX, HW = HS[:, 0:m], HS[:, m:2 * m], HS[:, 2 * m:3 * m]
    stats = [SolveStats() for _ in range(B)]
    locked_vals = [np.empty((0,)) for _ in range(B)]
    n_locked = 0                        # the same for every member still running
    carry = [None] * B
    cur = np.zeros(B, dtype=np.int64)   # which slab holds each member's current block
    block_no = 0
    live = list(range(B))               # members still solving
    t0 = time.perf_counter()

    def blocks(s, idx=None):
        S = slabs[s]
        return S[:, 0:m], S[:, m:2 * m], S[:, 2 * m:3 * m]

    def deflate(idx, Xv):
        if n_locked == 0:
            return
        L = locked_buf[:, :n_locked]
        Cm = st.gram(idx, L, Xv, n_locked, m).to(torch.complex64)
        st.rotate(idx, Cm, L, Xv, n_locked, m, -1)

    def normalize_rows(idx, Xv, rows, floor):
        sq = st.rowstats(idx, Xv, Xv, rows)
        scale = 1.0 / torch.clamp(torch.sqrt(torch.clamp(sq[:, :, 2], min=0.0)), min=floor)
        st.scale_rows(idx, Xv, scale, rows)

    def ortho_steps(idx, Xv, first=None):
        """SVQB pass on host eigh, then the device Cholesky-QR pass (solver._ortho_steps);
        `first` is the host eigh of the first pass's Gram when the caller has read it."""
        for p in range(2):
            if p == 0 and first is not None:
                w, V = first
                C = np.stack([svqb_from_eig(w[j], V[j], _SVQB_DROP)[0] for j in range(len(idx))])
                rotate_inplace(idx, st.upload(idx, C.astype(np.complex64), (m, m)), Xv, m)
                continue
            Gm = st.gram(idx, Xv, Xv, m, m)
            if p > 0 and m <= dense.MAX_N:
                C, _ = dense.cholqr_coeffs(Gm[idx_t(idx)], tol=_SVQB_DROP)
                Cf = torch.zeros((B, m, m), dtype=torch.complex64, device=dev)
                Cf[idx_t(idx)] = C
            else:
                w, V = yield HostEigh(_hermitian(Gm[idx_t(idx)]))
                C = np.stack([svqb_from_eig(w[j], V[j], _SVQB_DROP)[0] for j in range(len(idx))])
                Cf = st.upload(idx, C.astype(np.complex64), (m, m))
            rotate_inplace(idx, Cf, Xv, m)

    def rotate_inplace(idx, Cf, Xv, rows):
        if rows <= 32:
            st.rotate(idx, Cf, Xv, Xv, rows, rows)
        else:
            tmp = torch.empty((B, rows) + vshape, dtype=torch.complex64, device=dev)
            st.rotate(idx, Cf, Xv, tmp, rows, rows)
            sel = idx_t(idx)
            Xv[sel] = tmp[sel]

    idx_cache = {}

    def idx_t(idx):
        key = tuple(int(i) for i in idx)
        t = idx_cache.get(key)
        if t is None:
            t = _to_device(np.asarray(key, dtype=np.int64), dev)
            idx_cache[key] = t
        return t

    def ritz_request(idx, Xv, HXv, Wv, normalize):
        """Queue (lam, |x|^2, |Θx|^2, |R|^2) per row of the members idx, with R = HX -
        lam X into W (solver._ritz_request); (len(idx), m, 4) on the device."""
        s = st.rowstats(idx, Xv, HXv, m)
        lam_d = s[:, :, 0] / torch.clamp(s[:, :, 2], min=1e-30) if normalize else s[:, :, 0].contiguous()
        r2 = st.residual_norms(idx, HXv, Xv, lam_d, Wv, m)
        sel = idx_t(idx)
        return torch.stack([lam_d[sel], s[sel][:, :, 2], s[sel][:, :, 3], r2[sel]], dim=2)

    def ritz(idx, Xv, HXv, Wv, normalize):
        """(lam, rn, |x|) per member of idx (solver._ritz_steps)."""
        return _ritz_from_host((yield ritz_request(idx, Xv, HXv, Wv, normalize)))

    def rr_gram(idx, act, hact, nb):
        """Block upper triangle of act^H (Θ act) and its conjugate (solver._rr_gram)."""
        if nb // m < 2:
            return st.gram(idx, act, hact, nb, nb)
        A = torch.empty((B, nb, nb), dtype=torch.complex128, device=dev)
        for i in range(0, nb, m):
            blk = st.gram(idx, act[:, i:i + m], hact[:, i:], m, nb - i)
            A[:, i:i + m, i:] = blk
            if i + m < nb:
                A[:, i + m:, i:i + m] = blk[:, :, m:].conj().transpose(-2, -1)
        return A

    while live:
        # ---- block start (every live member shares n_locked; slabs reset to 0) ----
        cur[live] = 0
        P, X, W = blocks(0)
        nc = 0 if carry[live[0]] is None else int(carry[live[0]].shape[0])
        for i in live:
            if nc:
                X[i, :nc] = carry[i]
            if nc < m:
                call("ef_rand_block", ops[i].handle, X[i, nc:].data_ptr(), m - nc, seeds[i],
                     block_no, EF_RAND_NORMAL, blas._stream())
        if nc < m:
            normalize_rows(live, X[:, nc:], m - nc, 1e-30)
        block_no += 1
        deflate(live, X)
        yield from ortho_steps(live, X)
        st.theta(live, X, HX, m)
        for i in live:
            stats[i].theta_applications += m
        n_lock = {i: min(nl, nevs[i] - locked_vals[i].size) for i in live}
        have_p = {i: False for i in live}
        iters = {}
        active = list(live)
        for it in range(maxit):
            c = 0 if it % 2 == 0 else 1            # active members flip slabs together
            P, X, W = blocks(c)
            S = slabs[c]
            # the work up to W's first SVQB Gram touches W only: queued before the
            # convergence test, read with it (solver.lobpcg_steps does the same)
            ritz_t = ritz_request(active, X, HX, W, False)
            st.theta(active, W, W, m, precondition=True)
            deflate(active, W)
            for _ in range(2):
                Cm = st.gram(active, X, W, m, m).to(torch.complex64)
                st.rotate(active, Cm, X, W, m, m, -1)
            Gw = st.gram(active, W, W, m, m)
            h, (ww, Vw) = yield HostMany([ritz_t, HostEigh(_hermitian(Gw[idx_t(active)]))])
            lam, rn, xnorm = _ritz_from_host(h)
            still, keep = [], []
            for j, i in enumerate(active):
                dead = xnorm[j] < 0.5
                lam_h = np.where(dead, np.inf, lam[j])
                rnj = np.where(dead, np.inf, rn[j])
                order = np.argsort(lam_h)
                if (rnj[order[:n_lock[i]]] < tol).all():
                    iters[i] = it + 1
                    cur[i] = c
                else:
                    still.append(i)
                    keep.append(j)
                    stats[i].iterations += 1
            active = still
            if not active:
                break
            yield from ortho_steps(active, W, first=(ww[keep], Vw[keep]))

            def theta_w():
                st.theta(active, W, HW, m)
                for i in active:
                    stats[i].theta_applications += m
            with_p = [i for i in active if have_p[i]]
            if with_p:
                XW = S[:, m:3 * m]
                for _ in range(2):
                    Cm = st.gram(with_p, XW, P, 2 * m, m).to(torch.complex64)
                    st.rotate(with_p, Cm, XW, P, 2 * m, m, -1)
                Gp = HostCopy(_hermitian(st.gram(with_p, P, P, m, m)[idx_t(with_p)]))
                theta_w()                              # runs while the host does P's eigh
                w, V = yield HostEigh(Gp)
                keep_rows, Ts = [], []
                for j, i in enumerate(with_p):
                    Tp, keepp = svqb_from_eig(w[j], V[j], _SVQB_DROP)
                    if not keepp.any():
                        have_p[i] = False
                    else:
                        keep_rows.append(i)
                        Ts.append(Tp.astype(np.complex64))
                if keep_rows:
                    rotate_inplace(keep_rows, st.upload(keep_rows, np.stack(Ts), (m, m)), P, m)
            else:
                theta_w()
            with_p = [i for i in active if have_p[i]]
            if with_p:
                st.theta(with_p, P, HP, m)
                for i in with_p:
                    stats[i].theta_applications += m
            Sn = slabs[1 - c]
            for sub, act, hact, off in (([i for i in active if have_p[i]], S, HS, 0),
                                        ([i for i in active if not have_p[i]], S[:, m:3 * m],
                                         HS[:, m:3 * m], m)):
                if not sub:
                    continue
                nb = int(act.shape[1])
                A_d = rr_gram(sub, act, hact, nb)
                rows_d = st.rowstats(sub, act, act, nb)[:, :, 2]
                sel = idx_t(sub)
                A_s = _hermitian(A_d[sel])
                dead = torch.sqrt(torch.clamp(rows_d[sel], min=0.0)) < 0.5
                diag = A_s.diagonal(dim1=-2, dim2=-1)
                penalty = torch.clamp(100.0 * diag.abs().amax(dim=1, keepdim=True), min=_RR_DEAD_PENALTY)
                diag.add_(torch.where(dead, penalty, torch.zeros_like(penalty)).to(A_s.dtype))
                wA, VA = yield HostEigh(A_s)
                Cm = VA[:, :, :m]
                Cp = Cm.copy()
                Cp[:, m - off:2 * m - off] = 0
                Ccat = np.concatenate([Cp, Cm], axis=2).astype(np.complex64)
                st.rotate(sub, st.upload(sub, Ccat, (nb, 2 * m)), act, Sn[:, 0:2 * m], nb, 2 * m)
            for i in active:
                have_p[i] = True
            Pn, Xn, Wn = blocks(1 - c)
            deflate(active, Xn)
            normalize_rows(active, Sn[:, 0:2 * m], 2 * m, 1e-20)
            st.theta(active, Xn, HX, m)
            for i in active:
                stats[i].theta_applications += m
        for i in active:                           # maxit without convergence
            iters[i] = max(maxit, 1)
            cur[i] = maxit % 2
        # ---- block end: final Θ X and Ritz values of every live member ----
        done = {}
        lock_info = {}
        for c in (0, 1):
            sub = [i for i in live if cur[i] == c]
            if not sub:
                continue
            P, X, W = blocks(c)
            st.theta(sub, X, HX, m)
            for i in sub:
                stats[i].theta_applications += m
            lam, rn, xnorm = yield from ritz(sub, X, HX, W, normalize_rq)
            for j, i in enumerate(sub):
                lam_j = np.where(xnorm[j] < 0.5, np.inf, lam[j])
                rn_j = np.where(xnorm[j] < 0.5, np.inf, rn[j])
                lock_info[i] = (lam_j, rn_j, c)
        next_live = []
        for i in live:
            lam_j, rn_j, c = lock_info[i]
            order = np.argsort(lam_j)
            k = n_lock[i]
            if not np.isfinite(lam_j[order[:k]]).all():
                done[keys[i]] = RuntimeError(
                    f"block produced only {int(np.isfinite(lam_j).sum())} live Ritz "
                    f"pairs but needs {k} to lock — rank collapse")
                continue
            Xc = slabs[c][i, m:2 * m]
            lock_idx = _to_device(np.asarray(order[:k], dtype=np.int64), dev)
            carry_idx = _to_device(np.asarray(order[k:], dtype=np.int64), dev)
            locked_buf[i, n_locked:n_locked + k] = Xc.index_select(0, lock_idx)
            carry[i] = Xc.index_select(0, carry_idx)
            locked_vals[i] = np.concatenate([locked_vals[i], lam_j[order[:k]]])
            stats[i].rounds.append({"iters": iters[i], "locked": int(locked_vals[i].size),
                                    "max_res_locked": float(rn_j[order[:k]].max())})
            if locked_vals[i].size >= nevs[i]:
                stats[i].wall_seconds = time.perf_counter() - t0
                vals = locked_vals[i]
                order_v = np.argsort(vals, kind="stable")
                n_i = vals.size
                vecs = locked_buf[i, :n_i].index_select(0, _to_device(order_v.astype(np.int64), dev))
                done[keys[i]] = (vals[order_v][:nevs[i]], vecs, stats[i])
                carry[i] = None
            else:
                next_live.append(i)
        n_locked += nl
        live = next_live
        if done:
            if live:
                yield GroupResults(done)
            else:
                return GroupResults(done)
    return GroupResults({})


def run_group(gen) -> dict:
    """Drive one grouped solve alone; returns {member: result or exception}."""
    from .solver import _to_host
    out: dict = {}
    try:
        req = next(gen)
        while True:
            if isinstance(req, GroupResults):
                out.update(req.results)
                req = gen.send(None)
            else:
                req = gen.send(_to_host(req))
    except StopIteration as stop:
        if isinstance(stop.value, GroupResults):
            out.update(stop.value.results)
    return out


def lobpcg_grouped(ops, nevs, m: int = 32, guard: int = 8, tol: float = 1e-4, maxit: int = 400,
                   seeds=None, normalize_rq: bool = True) -> list:
    """Solve one group (one grid edge, one block shape) alone; [(vals, vecs, stats)] in the
    order of `ops`, raising the first member's failure."""
    res = run_group(lobpcg_group_steps(ops, nevs, m=m, guard=guard, tol=tol, maxit=maxit,
                                       seeds=seeds, normalize_rq=normalize_rq))
    out = [res[i] for i in range(len(ops))]
    for r in out:
        if isinstance(r, Exception):
            raise r
    return out
