"""FP64 reference eigenvalues for the GPU accuracy tests (run on CPU).

    python tests/golden/make_fp64_reference.py [case ...]

For seeded rod networks from eigenfns_gb300.structure (rasterized by the numpy
checker in oracle/structure.py, which the GPU rasterizer matches bit for bit),
runs the oracle's LOBPCG in complex128 at a tight tolerance and stores the
eigenvalues. The GPU complex64 solver is required to match them within 1e-6
relative (tests/test_gpu_accuracy.py).

The 128^3 case (the N=1000 workload the headline throughput is quoted on) takes
hours with the numpy operator, so for grids of 96 and up the oracle LOBPCG runs
on an operator whose FFTs and element-wise work are done by torch on the CPU in
float64 (multithreaded). It computes the same expression as oracle.operator's
complex128 Θ and preconditioner; the script checks the two against each other on
a random block before it starts (relative difference <= 1e-12). Eigenvalues are
written after every locked block, so a partial run still leaves a usable fixture.
"""
from __future__ import annotations

import hashlib
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from eigenfns_gb300.structure import generate_network  # noqa: E402
from oracle.operator import MaxwellOperator  # noqa: E402
from oracle.solver import lobpcg_blocks  # noqa: E402
from oracle.structure import rasterize_averaged  # noqa: E402

CASES = {
    # name: (nodes, grid, seed, k_frac, nev, m, guard, tol)
    "n64_g32_gamma": (64, 32, 0, (0.0, 0.0, 0.0), 24, 12, 4, 1e-9),
    "n216_g48_k": (216, 48, 7, (0.23, -0.41, 0.12), 32, 16, 4, 1e-9),
    # the headline workload: N=1000, 128^3, Gamma, block 32 / guard 8 (two blocks)
    "n1000_g128_gamma": (1000, 128, 0, (0.0, 0.0, 0.0), 48, 32, 8, 1e-7),
}


class TorchCPUOperator(MaxwellOperator):
    """complex128 Θ and transverse-projection preconditioner on torch CPU tensors.

    Same arithmetic as oracle.operator._theta_block / _precondition_fancy_block
    (eigenfns/operator.py:82-95, 104-127), evaluated with torch's multithreaded
    float64 FFTs (numpy's normalisation: 1/N on the inverse).
    """

    def __init__(self, *a, **k):
        import torch
        super().__init__(*a, **k)
        assert self.dtype == np.complex128
        self._t = torch
        self._kn = torch.from_numpy(np.ascontiguousarray(self.basis.kn))
        self._tt = torch.from_numpy(np.ascontiguousarray(self.basis.t))
        self._inv_eps = torch.from_numpy(self.inv_eps)
        self._eps = torch.from_numpy(self.eps_grid)

    def _apply(self, Hs, build, w, project):
        t = self._t
        out = np.empty(np.shape(Hs), np.complex128)
        for i in range(out.shape[0]):
            h = t.from_numpy(np.ascontiguousarray(np.asarray(Hs[i], np.complex128)))
            c1, c2 = build(h[0], h[1])
            Ec = c1[None] * self._tt[0] + c2[None] * self._tt[1]
            E = t.fft.ifftn(Ec, dim=(-3, -2, -1))
            Dc = t.fft.fftn(w * E, dim=(-3, -2, -1))
            f1 = (self._tt[0] * Dc).sum(0)
            f2 = (self._tt[1] * Dc).sum(0)
            o1, o2 = project(f1, f2)
            out[i, 0] = o1.numpy()
            out[i, 1] = o2.numpy()
        return out

    def theta(self, Hs):
        kn = self._kn
        return self._apply(Hs, lambda a, b: (-1j * kn * b, 1j * kn * a), self._inv_eps,
                           lambda f1, f2: (-1j * kn * f2, 1j * kn * f1))

    def precondition(self, Rs, target: float = 0.0):
        knr = self._t.clamp(self._kn, min=self.kn_floor)
        return self._apply(Rs, lambda a, b: (1j * b / knr, -1j * a / knr), self._eps,
                           lambda f1, f2: (1j * f2 / knr, -1j * f1 / knr))


def _check_fast(op_fast, op_ref):
    rng = np.random.default_rng(0)
    shape = (1, 2) + (op_ref.grid_size,) * 3
    X = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) * op_ref.mask
    for f, g in ((op_fast.theta, op_ref.theta), (op_fast.precondition, op_ref.precondition)):
        a, b = f(X), g(X)
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert rel <= 1e-12, rel


def main(names):
    for name in names:
        nodes, grid, seed, k, nev, m, guard, tol = CASES[name]
        t0 = time.time()
        net = generate_network(nodes, seed)
        eps = rasterize_averaged(net.rods, grid, net.box_size, sub=4)
        if grid >= 96:
            op = TorchCPUOperator(eps, net.box_size, k_frac=k, dtype=np.complex128)
            _check_fast(op, MaxwellOperator(eps, net.box_size, k_frac=k, dtype=np.complex128))
            print(name, "torch-CPU operator agrees with the numpy oracle", flush=True)
        else:
            op = MaxwellOperator(eps, net.box_size, k_frac=k, dtype=np.complex128)
        meta = dict(eps=eps, eps_sha256=hashlib.sha256(eps.tobytes()).hexdigest(),
                    box=net.box_size, k=np.asarray(k), nodes=nodes, grid=grid, seed=seed,
                    m=m, guard=guard, tol=tol)
        done = []

        def on_block(n_locked, vals, _X, done=done, meta=meta, name=name):
            done.extend(np.asarray(vals, np.float64).tolist())
            np.savez_compressed(HERE / f"fp64_{name}.npz", vals=np.sort(np.asarray(done)), **meta)
            print(name, f"locked {n_locked} after {time.time() - t0:.0f}s", flush=True)

        vals, _, st = lobpcg_blocks(op, nev, m=m, guard=guard, tol=tol, maxit=600, seed=1,
                                    on_block=on_block, verbose=True)
        np.savez_compressed(HERE / f"fp64_{name}.npz", vals=vals,
                            rounds=np.asarray([r["iters"] for r in st.rounds]), **meta)
        print(name, f"{time.time() - t0:.0f}s", vals[:4], flush=True)


if __name__ == "__main__":
    main(sys.argv[1:] or list(CASES))
