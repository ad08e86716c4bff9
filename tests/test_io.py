"""Checkpoint / resume file formats (eigenfns/io.py:19-67, run_interior.py:96-121)."""
from __future__ import annotations

import json

import numpy as np
import pytest


def test_block_checkpointer_layout_and_round_trip(tmp_path):
    from eigenfns_gb300.io import BlockCheckpointer
    ck = BlockCheckpointer(tmp_path, "solve", meta={"grid": 16, "nev": 6})
    assert ck.load()[0] is None and ck.load()[2] == 0
    rng = np.random.default_rng(0)
    v0, x0 = np.sort(rng.random(3)), (rng.standard_normal((3, 2, 4, 4, 4)) + 0j).astype(np.complex64)
    v1, x1 = np.sort(rng.random(3)) + 1, (rng.standard_normal((3, 2, 4, 4, 4)) + 0j).astype(np.complex64)
    ck.save_block(0, v0, x0)
    ck.save_block(1, v1, x1, extra={"theta_applications": 123})
    names = sorted(p.name for p in tmp_path.iterdir())
    assert names == ["solve_block000_vals.npy", "solve_block000_vecs.npy", "solve_block001_vals.npy",
                     "solve_block001_vecs.npy", "solve_meta.json"]
    meta = json.loads((tmp_path / "solve_meta.json").read_text())
    assert meta["n_blocks"] == 2 and meta["grid"] == 16 and meta["theta_applications"] == 123
    vals, vecs, nb, meta2 = BlockCheckpointer(tmp_path, "solve").load()
    assert nb == 2 and np.array_equal(vals, np.concatenate([v0, v1]))
    assert np.array_equal(vecs, np.concatenate([x0, x1]))


def test_block_checkpointer_detects_missing_block(tmp_path):
    from eigenfns_gb300.io import BlockCheckpointer
    ck = BlockCheckpointer(tmp_path, "t")
    ck.save_block(0, np.zeros(2), np.zeros((2, 2, 2, 2, 2), np.complex64))
    ck.save_block(1, np.ones(2), np.zeros((2, 2, 2, 2, 2), np.complex64))
    (tmp_path / "t_block001_vecs.npy").unlink()
    with pytest.raises(RuntimeError):
        ck.load()


def test_interior_state_round_trip(tmp_path):
    from eigenfns_gb300.io import load_interior_state, save_interior_state
    X = (np.arange(2 * 2 * 3 * 3 * 3, dtype=np.float32).reshape(2, 2, 3, 3, 3) + 1j).astype(np.complex64)
    hist = [{"outer": 0, "n_in": 3, "n_conv": 1}]
    p = tmp_path / "interior_state.npz"
    save_interior_state(p, X, "polish", 2, 4567, 123.5, hist)
    st = load_interior_state(p)
    assert st["stage"] == "polish" and st["outer"] == 2 and st["n_theta"] == 4567
    assert st["lam_max"] == 123.5 and st["history"] == hist and np.array_equal(st["X"], X)
