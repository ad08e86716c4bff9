"""Per-block checkpoints in the reference's on-disk layout (eigenfns/io.py:19-67).

Files, so that runs resume across the two implementations:
  <dir>/<tag>_block###_vals.npy   eigenvalues of locked block ###
  <dir>/<tag>_block###_vecs.npy   its vectors, (n, 2, G, G, G) complex64
  <dir>/<tag>_meta.json           {"n_blocks": ..., "saved_at": ..., user meta}
Every file is written to a temporary name and renamed into place; loading a
checkpoint whose meta names a block with missing files raises RuntimeError
("checkpoint corrupt"), as the reference does.

`save_interior_state` / `load_interior_state` hold the rolling state of the
two-stage driver, the reference's interior_state.npz (scripts/run_interior.py:
96-121): X, stage, outer, n_theta, lam_max and the JSON history.
"""
from __future__ import annotations

import json
import time
from pathlib import Path

import numpy as np


def _to_numpy(a):
    if hasattr(a, "detach"):
        return a.detach().cpu().numpy()
    return np.asarray(a)


class BlockCheckpointer:
    def __init__(self, directory, tag: str, meta: dict | None = None):
        self.dir = Path(directory)
        self.dir.mkdir(parents=True, exist_ok=True)
        self.tag = tag
        self.meta = dict(meta or {})

    def _meta_path(self) -> Path:
        return self.dir / f"{self.tag}_meta.json"

    def _block_paths(self, i: int):
        return (self.dir / f"{self.tag}_block{i:03d}_vals.npy",
                self.dir / f"{self.tag}_block{i:03d}_vecs.npy")

    def load(self):
        """(vals, vecs, n_blocks, meta); vals and vecs are None without a checkpoint."""
        pm = self._meta_path()
        if not pm.exists():
            return None, None, 0, self.meta
        meta = json.loads(pm.read_text())
        n_blocks = int(meta.get("n_blocks", 0))
        vals, vecs = [], []
        for i in range(n_blocks):
            pv, px = self._block_paths(i)
            if not (pv.exists() and px.exists()):
                raise RuntimeError(f"checkpoint corrupt: missing block {i} files")
            vals.append(np.load(pv))
            vecs.append(np.load(px))
        if not vals:
            return None, None, 0, meta
        return np.concatenate(vals), np.concatenate(vecs), n_blocks, meta

    def save_block(self, i: int, vals, vecs, extra: dict | None = None) -> None:
        pv, px = self._block_paths(i)
        for path, arr in ((pv, _to_numpy(vals)), (px, _to_numpy(vecs))):
            tmp = path.with_suffix(".tmp.npy")
            np.save(tmp, arr)
            tmp.replace(path)
        meta = dict(self.meta)
        meta.update(extra or {})
        meta["n_blocks"] = i + 1
        meta["saved_at"] = time.strftime("%Y-%m-%d %H:%M:%S")
        tmp = self._meta_path().with_suffix(".tmp.json")
        tmp.write_text(json.dumps(meta, indent=1))
        tmp.replace(self._meta_path())


def save_interior_state(path, X, stage: str, outer: int, n_theta: int, lam_max: float,
                        history: list) -> None:
    path = Path(path)
    tmp = path.with_suffix(".tmp.npz")
    np.savez(tmp, X=_to_numpy(X), stage=stage, outer=outer, n_theta=n_theta, lam_max=lam_max,
             history=json.dumps(history))
    tmp.replace(path)


def load_interior_state(path) -> dict:
    st = np.load(Path(path), allow_pickle=False)
    return {"X": np.asarray(st["X"]), "stage": str(st["stage"]), "outer": int(st["outer"]),
            "n_theta": int(st["n_theta"]), "lam_max": float(st["lam_max"]),
            "history": json.loads(str(st["history"]))}
