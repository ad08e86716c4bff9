"""FP64 reference eigenvalues for the GPU accuracy tests (run on CPU, minutes).

    python tests/golden/make_fp64_reference.py

For seeded rod networks from eigenfns_gb300.structure (rasterized by the numpy
checker in oracle/structure.py, which the GPU rasterizer matches bit for bit),
runs the oracle's LOBPCG in complex128 at a tight tolerance and stores the
eigenvalues. The GPU complex64 solver is required to match them within 1e-6
relative (tests/test_gpu_accuracy.py).
"""
from __future__ import annotations

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
    # name: (nodes, grid, seed, k_frac, nev, m, guard)
    "n64_g32_gamma": (64, 32, 0, (0.0, 0.0, 0.0), 24, 12, 4),
    "n216_g48_k": (216, 48, 7, (0.23, -0.41, 0.12), 32, 16, 4),
}


def main(names):
    for name in names:
        nodes, grid, seed, k, nev, m, guard = CASES[name]
        t0 = time.time()
        net = generate_network(nodes, seed)
        eps = rasterize_averaged(net.rods, grid, net.box_size, sub=4)
        op = MaxwellOperator(eps, net.box_size, k_frac=k, dtype=np.complex128)
        vals, _, st = lobpcg_blocks(op, nev, m=m, guard=guard, tol=1e-9, maxit=600, seed=1)
        np.savez_compressed(HERE / f"fp64_{name}.npz", vals=vals, eps=eps, box=net.box_size,
                            k=np.asarray(k), nodes=nodes, grid=grid, seed=seed,
                            rounds=np.asarray([r["iters"] for r in st.rounds]))
        print(name, f"{time.time() - t0:.0f}s", vals[:4], flush=True)


if __name__ == "__main__":
    main(sys.argv[1:] or list(CASES))
