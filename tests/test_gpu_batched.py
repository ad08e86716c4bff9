"""Lock-step batched solves (eigenfns_gb300.batched) give the same eigenpairs as each
solve run alone: the same kernels run in the same order per instance, so the
eigenvalues agree bit for bit (checked at 1e-12 relative) across grids, k-points and
band counts mixed in one batch."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _instances():
    from eigenfns_gb300.operator import MaxwellOperator
    from eigenfns_gb300.structure import bz_kpoint, make_structure
    out = []
    for nodes, grid, seed, nev, m, guard in ((64, 32, 3, 12, 8, 2), (64, 32, 4, 16, 16, 4),
                                            (216, 48, 5, 10, 12, 3), (64, 32, 6, 6, 8, 2)):
        eps, L, _ = make_structure(nodes, grid, seed=seed)
        out.append((MaxwellOperator(eps, L, k_frac=bz_kpoint(seed)), nev, m, guard, seed))
    return out


def test_batched_equals_alone():
    from eigenfns_gb300.batched import lobpcg_batched
    from eigenfns_gb300.solver import lobpcg_blocks
    inst = _instances()
    alone = [lobpcg_blocks(op, nev, m=m, guard=g, tol=1e-4, seed=s, verbose=False)
             for op, nev, m, g, s in inst]
    batch = lobpcg_batched([i[0] for i in inst], [i[1] for i in inst], m=[i[2] for i in inst],
                           guard=[i[3] for i in inst], tol=1e-4, seeds=[i[4] for i in inst])
    for (va, xa, sa), (vb, xb, sb) in zip(alone, batch):
        assert len(va) == len(vb)
        assert np.abs(va - vb).max() <= 1e-12 * np.abs(va).max()
        assert sa.iterations == sb.iterations
        assert torch.equal(xa, xb)


def test_batched_one_at_a_time_equals_alone():
    """The same instances as interleaved single solves (no grouping)."""
    from eigenfns_gb300.batched import lobpcg_batched
    from eigenfns_gb300.solver import lobpcg_blocks
    inst = _instances()[:2]
    alone = [lobpcg_blocks(op, nev, m=m, guard=g, tol=1e-4, seed=s, verbose=False)
             for op, nev, m, g, s in inst]
    batch = lobpcg_batched([i[0] for i in inst], [i[1] for i in inst], m=[i[2] for i in inst],
                           guard=[i[3] for i in inst], tol=1e-4, seeds=[i[4] for i in inst],
                           grouped=False)
    for (va, xa, sa), (vb, xb, sb) in zip(alone, batch):
        assert np.array_equal(va, vb) and sa.iterations == sb.iterations
        assert torch.equal(xa, xb)


def test_grouped_members_equal_alone():
    """One group (32^3, block 12, guard 4) of members with different k-points, seeds and
    band counts (1 to 3 blocks each): every member's eigenvalues, locked vectors,
    iteration counts and Θ-application counts equal its solve run alone."""
    from eigenfns_gb300.grouped import lobpcg_grouped
    from eigenfns_gb300.operator import MaxwellOperator
    from eigenfns_gb300.solver import lobpcg_blocks
    from eigenfns_gb300.structure import bz_kpoint, make_structure
    ops, nevs, seeds = [], [12, 8, 20, 16], [11, 12, 13, 14]
    for s in seeds:
        eps, L, _ = make_structure(64, 32, seed=s)
        ops.append(MaxwellOperator(eps, L, k_frac=bz_kpoint(s)))
    alone = [lobpcg_blocks(op, nev, m=12, guard=4, tol=1e-4, seed=s, verbose=False)
             for op, nev, s in zip(ops, nevs, seeds)]
    group = lobpcg_grouped(ops, nevs, m=12, guard=4, tol=1e-4, seeds=seeds)
    for (va, xa, sa), (vb, xb, sb) in zip(alone, group):
        assert np.array_equal(va, vb)
        assert torch.equal(xa, xb)
        assert sa.iterations == sb.iterations
        assert sa.theta_applications == sb.theta_applications
        assert [r["iters"] for r in sa.rounds] == [r["iters"] for r in sb.rounds]
