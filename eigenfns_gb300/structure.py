"""Seeded tetravalent rod networks and their sub-voxel-averaged eps grids.

Benchmark inputs; the reference has neither piece (its structures are loaded
from files, eigenfns/structure.py:34-48, and rasterized binary,
structure.py:51-151). The generator:

* N nodes uniform in a periodic cube of edge L = (N/8)^(1/3) (numpy
  default_rng(seed));
* each node joined to its 4 nearest neighbours under the minimum image,
  edges deduplicated (so degrees are >= 4);
* rods are flat-capped cylinders of radius 0.2 x the mean bond length,
  eps_rod = 8.41 in an eps = 1 background;
* eps is the mean over sub^3 regular sub-samples per voxel, rods wrapped
  periodically (the library's ef_rasterize_rods).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._lib import call


@dataclass
class RodNetwork:
    n_nodes: int
    box_size: float
    nodes: np.ndarray      # (N, 3)
    edges: np.ndarray      # (E, 2) node indices, i < j
    rods: np.ndarray       # (E, 7) p, q (minimum image of the far node), radius
    mean_bond: float
    radius: float


def box_size_for_nodes(n_nodes: int, density: float = 8.0) -> float:
    return float((n_nodes / density) ** (1.0 / 3.0))


def generate_network(n_nodes: int, seed: int, radius_factor: float = 0.2,
                     k_neighbors: int = 4) -> RodNetwork:
    from scipy.spatial import cKDTree
    rng = np.random.default_rng(seed)
    L = box_size_for_nodes(n_nodes)
    nodes = rng.random((n_nodes, 3)) * L
    tree = cKDTree(nodes, boxsize=L)
    _, nbr = tree.query(nodes, k=k_neighbors + 1)
    pairs = set()
    for i in range(n_nodes):
        for j in nbr[i, 1:]:
            a, b = (i, int(j)) if i < j else (int(j), i)
            pairs.add((a, b))
    edges = np.asarray(sorted(pairs), np.int64)
    d = nodes[edges[:, 1]] - nodes[edges[:, 0]]
    d -= L * np.round(d / L)
    bond = np.linalg.norm(d, axis=1)
    mean_bond = float(bond.mean())
    radius = radius_factor * mean_bond
    p = nodes[edges[:, 0]]
    rods = np.concatenate([p, p + d, np.full((len(edges), 1), radius)], axis=1)
    return RodNetwork(n_nodes, L, nodes, edges, rods, mean_bond, radius)


def rasterize(net: RodNetwork, grid: int, eps_rod: float = 8.41, eps_bg: float = 1.0,
              sub: int = 4) -> np.ndarray:
    """(G, G, G) float32 eps averaged over sub^3 samples per voxel (GPU)."""
    rods = np.ascontiguousarray(net.rods, np.float64)
    eps = np.empty((grid, grid, grid), np.float32)
    call("ef_rasterize_rods", int(grid), float(net.box_size), rods.ctypes.data, int(len(rods)),
         int(sub), float(eps_rod), float(eps_bg), eps.ctypes.data)
    return eps


def make_structure(n_nodes: int, grid: int, seed: int, eps_rod: float = 8.41, sub: int = 4):
    """(eps, box_size, network) for one benchmark structure."""
    net = generate_network(n_nodes, seed)
    return rasterize(net, grid, eps_rod=eps_rod, sub=sub), net.box_size, net


def bz_kpoint(seed: int) -> tuple:
    """A k-point uniform in the first Brillouin zone, k_frac in [-1/2, 1/2)^3."""
    rng = np.random.default_rng(np.random.SeedSequence([seed, 0x4B]))
    return tuple(float(x) for x in rng.random(3) - 0.5)
