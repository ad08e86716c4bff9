"""Numpy sub-voxel-averaging rasterizer, the checker of ef_rasterize_rods.

TEST INFRASTRUCTURE ONLY.

Same geometry as the library: sub-sample a of a voxel edge sits at
(a + 0.5) * L / (G * sub); a sample is inside a rod when its projection t on
the axis satisfies 0 <= t <= |q - p| and its radial distance is <= r (the
membership test of eigenfns/structure.py:135-138), with periodic wrapping.
Small grids only.
"""
from __future__ import annotations

import numpy as np


def rasterize_averaged(rods: np.ndarray, grid: int, box: float, sub: int = 4,
                       eps_rod: float = 8.41, eps_bg: float = 1.0) -> np.ndarray:
    GS = grid * sub
    h = box / GS
    occ = np.zeros((GS, GS, GS), bool)
    for rod in np.asarray(rods, np.float64):
        p, q, rad = rod[0:3], rod[3:6], rod[6]
        v = q - p
        ln = float(np.sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]))
        if ln <= 0:
            continue
        u = v / ln
        lo = np.floor((np.minimum(p, q) - rad) / h - 0.5).astype(int) - 1
        hi = np.ceil((np.maximum(p, q) + rad) / h - 0.5).astype(int) + 1
        a = np.arange(lo[0], hi[0] + 1)
        b = np.arange(lo[1], hi[1] + 1)
        c = np.arange(lo[2], hi[2] + 1)
        X = ((a + 0.5) * h - p[0])[:, None, None]
        Y = ((b + 0.5) * h - p[1])[None, :, None]
        Z = ((c + 0.5) * h - p[2])[None, None, :]
        t = (X * u[0] + Y * u[1]) + Z * u[2]
        rx, ry, rz = X - t * u[0], Y - t * u[1], Z - t * u[2]
        inside = (t >= 0) & (t <= ln) & (((rx * rx + ry * ry) + rz * rz) <= rad * rad)
        ii, jj, kk = np.nonzero(inside)
        occ[a[ii] % GS, b[jj] % GS, c[kk] % GS] = True
    frac = occ.reshape(grid, sub, grid, sub, grid, sub).sum(axis=(1, 3, 5)) / float(sub ** 3)
    return (eps_bg + (eps_rod - eps_bg) * frac).astype(np.float32)
