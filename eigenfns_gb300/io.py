"""Checkpoints of a blockwise eigensolve and of the two-stage interior driver.

The files keep the reference's layout (eigenfns/io.py:31-67 and
scripts/run_interior.py:96-121) so that a run started by either implementation
can be resumed by the other:

  <dir>/<tag>_block###_vals.npy   eigenvalues of locked block ###
  <dir>/<tag>_block###_vecs.npy   its vectors, (n, 2, G, G, G) complex64
  <dir>/<tag>_meta.json           {"n_blocks": ..., "saved_at": ..., user meta}
  interior_state.npz              X, stage, outer, n_theta, lam_max, history (JSON)

Blocks are append-only: saving block i never rewrites blocks 0..i-1, so the
cost of a save does not grow with the locked set. Each file is written under a
temporary name in the target directory and then renamed over the final name,
and the meta file (which is what names the blocks) goes last, so a crash
between two files leaves the previous checkpoint intact. A meta file that names
a block whose files are missing raises RuntimeError ("checkpoint corrupt").
"""
from __future__ import annotations

import json
import os
import tempfile
import time
from pathlib import Path
from typing import Callable

import numpy as np

META_SUFFIX = "_meta.json"


def _host_array(a) -> np.ndarray:
    """A numpy view of a host array or a copy of a torch tensor (any device)."""
    if hasattr(a, "detach"):
        return a.detach().cpu().numpy()
    return np.asarray(a)


def _replace_atomically(path: Path, write: Callable) -> None:
    """Run write(file object) on a temporary file next to `path`, then rename it."""
    fd, tmp = tempfile.mkstemp(dir=path.parent, prefix=f".{path.name}.", suffix=".part")
    try:
        with os.fdopen(fd, "wb") as f:
            write(f)
        os.replace(tmp, path)
    except BaseException:
        Path(tmp).unlink(missing_ok=True)
        raise


def block_file_names(tag: str, index: int) -> tuple[str, str]:
    """File names of locked block `index`: (eigenvalues, vectors)."""
    stem = f"{tag}_block{index:03d}"
    return f"{stem}_vals.npy", f"{stem}_vecs.npy"


class BlockCheckpointer:
    """Append-only store of the locked blocks of a solve (lobpcg_blocks_resumable)."""

    def __init__(self, directory, tag: str, meta: dict | None = None):
        self.dir = Path(directory)
        self.dir.mkdir(parents=True, exist_ok=True)
        self.tag = str(tag)
        self.meta = dict(meta or {})

    @property
    def meta_file(self) -> Path:
        return self.dir / f"{self.tag}{META_SUFFIX}"

    def block_files(self, index: int) -> tuple[Path, Path]:
        vals, vecs = block_file_names(self.tag, index)
        return self.dir / vals, self.dir / vecs

    def load(self):
        """(eigenvalues, vectors, number of blocks, meta) of the saved blocks.

        Without a checkpoint the arrays are None, the count is 0 and meta is the
        constructor's.
        """
        if not self.meta_file.exists():
            return None, None, 0, self.meta
        meta = json.loads(self.meta_file.read_text())
        count = int(meta.get("n_blocks", 0))
        paths = [self.block_files(i) for i in range(count)]
        absent = [i for i, (pv, px) in enumerate(paths) if not (pv.is_file() and px.is_file())]
        if absent:
            raise RuntimeError(f"checkpoint corrupt: {self.meta_file.name} lists block(s) "
                               f"{absent} whose files are missing")
        if count == 0:
            return None, None, 0, meta
        vals = np.concatenate([np.load(pv) for pv, _ in paths])
        vecs = np.concatenate([np.load(px) for _, px in paths])
        return vals, vecs, count, meta

    def save_block(self, i: int, vals, vecs, extra: dict | None = None) -> None:
        """Store block i, then record i + 1 blocks in the meta file."""
        pv, px = self.block_files(i)
        for path, arr in ((pv, _host_array(vals)), (px, _host_array(vecs))):
            _replace_atomically(path, lambda f, a=arr: np.save(f, a))
        record = {**self.meta, **(extra or {}), "n_blocks": int(i) + 1,
                  "saved_at": time.strftime("%Y-%m-%d %H:%M:%S")}
        text = json.dumps(record, indent=1).encode()
        _replace_atomically(self.meta_file, lambda f: f.write(text))


def save_interior_state(path, X, stage: str, outer: int, n_theta: int, lam_max: float,
                        history: list) -> None:
    """Rolling state of the two-stage interior driver (interior_state.npz)."""
    path = Path(path)
    fields = dict(X=_host_array(X), stage=np.str_(stage), outer=np.int64(outer),
                  n_theta=np.int64(n_theta), lam_max=np.float64(lam_max),
                  history=np.str_(json.dumps(history)))
    _replace_atomically(path, lambda f: np.savez(f, **fields))


def load_interior_state(path) -> dict:
    with np.load(Path(path), allow_pickle=False) as z:
        return {"X": np.asarray(z["X"]), "stage": str(z["stage"]), "outer": int(z["outer"]),
                "n_theta": int(z["n_theta"]), "lam_max": float(z["lam_max"]),
                "history": json.loads(str(z["history"]))}
