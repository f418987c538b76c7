"""Synthetic triangle meshes for the DG workloads.

A jittered n x n grid of squares on [-1, 1]^2, each square split along its
diagonal into two counter-clockwise triangles (K = 2 n^2).  Interior vertices
are moved by independent uniform offsets in [-0.1 h, 0.1 h] (h = 2 / n) drawn
from numpy's PCG64 generator seeded with ``seed``; boundary vertices stay on
the boundary.  The vertex / connectivity arrays are what the reference's
``simple_triangular_mesh_2d::fill_vertices`` / ``fill_connectivity`` take
(src/mesh/simple_triangular_mesh_2d.h:60-80): x, y interleaved and three
vertex indices per cell.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass

import numpy as np


@dataclass
class Mesh:
    xy: np.ndarray      # (nv, 2) float64
    cells: np.ndarray   # (K, 3) int32, counter-clockwise
    n: int = 0          # squares per side (0 when not a generated grid)
    seed: int = 0

    @property
    def num_cells(self) -> int:
        return int(self.cells.shape[0])

    @property
    def num_vertices(self) -> int:
        return int(self.xy.shape[0])


def jittered_square(n: int, seed: int, jitter: float = 0.1) -> Mesh:
    if n < 1:
        raise ValueError("n must be >= 1")
    h = 2.0 / n
    i, j = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="xy")
    x = -1.0 + i * h
    y = -1.0 + j * h
    rng = np.random.default_rng(seed)
    d = rng.uniform(-jitter * h, jitter * h, size=(n + 1, n + 1, 2))
    interior = (i > 0) & (i < n) & (j > 0) & (j < n)
    x = np.where(interior, x + d[..., 0], x)
    y = np.where(interior, y + d[..., 1], y)
    xy = np.stack([x.ravel(), y.ravel()], axis=1).astype(np.float64)
    vid = lambda a, b: b * (n + 1) + a  # noqa: E731
    jj, ii = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    ii = ii.ravel()
    jj = jj.ravel()
    v00, v10, v11, v01 = vid(ii, jj), vid(ii + 1, jj), vid(ii + 1, jj + 1), vid(ii, jj + 1)
    t1 = np.stack([v00, v10, v11], axis=1)
    t2 = np.stack([v00, v11, v01], axis=1)
    cells = np.stack([t1, t2], axis=1).reshape(-1, 3).astype(np.int32)
    return Mesh(xy=xy, cells=np.ascontiguousarray(cells), n=n, seed=seed)


def write_bin(mesh: Mesh, path: str) -> None:
    """int32 nv, f64 xy[2 nv], int32 K, int32 cells[3 K] (little endian)."""
    with open(path, "wb") as f:
        f.write(struct.pack("<i", mesh.num_vertices))
        f.write(np.ascontiguousarray(mesh.xy, dtype="<f8").tobytes())
        f.write(struct.pack("<i", mesh.num_cells))
        f.write(np.ascontiguousarray(mesh.cells, dtype="<i4").tobytes())


def min_edge_length(mesh: Mesh) -> float:
    p = mesh.xy[mesh.cells]                      # (K, 3, 2)
    e = p[:, [1, 2, 0], :] - p                    # edges v_e -> v_{e+1}
    return float(np.sqrt((e ** 2).sum(-1)).min())
