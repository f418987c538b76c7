"""The GPU half-edge matching (csrc/topology.cu) against the host sort.

dgc_create matches half-edges on the GPU from DGC_GPU_TOPOLOGY_MIN cells
(default 16384); dgc_host_mesh always sorts on the host.  The twin maps and
boundary numbering must be identical, on the reference's own meshes (forced
GPU path), on jittered meshes up to 524288 cells (default path), and on a
mesh with random vertex numbering; broken meshes must be refused through the
error code.
"""
import os
import time

import numpy as np
import pytest

from conftest import GOLDEN

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import dgc_gb300 as dg  # noqa: E402
from dgc_gb300 import meshes  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def built():
    from dgc_gb300 import build
    build.build()


@pytest.fixture
def force_gpu(monkeypatch):
    monkeypatch.setenv("DGC_GPU_TOPOLOGY_MIN", "0")


def _check_same(m, N=2):
    D = dg.Discretization(m, "advection", N, dg.F32)
    nbr, nb = D.neighbors()
    _, hnbr, hnb = dg.host_mesh(m, N)
    assert nb == hnb
    assert np.array_equal(nbr[:, :3], hnbr[:, :3])
    return D


@pytest.mark.parametrize("case", ["cells4_N1", "coarse_N1", "fine_N1", "jit4_N1"])
def test_gpu_topology_reference_meshes(case, force_gpu):
    d = np.load(os.path.join(GOLDEN, f"ref_{case}.npz"))
    m = meshes.Mesh(xy=d["mesh_xy"].reshape(-1, 2), cells=d["mesh_cells"].reshape(-1, 3))
    _check_same(m)


def test_gpu_topology_shuffled_numbering(force_gpu):
    m = meshes.jittered_square(40, 3)
    rng = np.random.default_rng(0)
    perm = rng.permutation(m.xy.shape[0])
    inv = np.argsort(perm)
    xy = m.xy[perm]
    cells = inv[m.cells].astype(np.int32)
    cells = cells[rng.permutation(cells.shape[0])]
    _check_same(meshes.Mesh(xy=xy, cells=np.ascontiguousarray(cells)))


@pytest.mark.parametrize("n", [91, 512, 1024])
def test_gpu_topology_large_default_path(n, monkeypatch):
    m = meshes.jittered_square(n, 11)
    K = m.cells.shape[0]
    assert K >= 16384
    _check_same(m, N=1)
    times = {}
    for name, thr in (("gpu", "16384"), ("host", str(1 << 40))):
        monkeypatch.setenv("DGC_GPU_TOPOLOGY_MIN", thr)
        best = 1e9
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            D = dg.Discretization(m, "advection", 1, dg.F32)
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
            del D
        times[name] = best
    print(f"K={K}: dgc_create {times['gpu'] * 1e3:.1f} ms with GPU half-edge matching, "
          f"{times['host'] * 1e3:.1f} ms with the host sort")


def test_gpu_topology_refuses_broken_meshes(force_gpu):
    m = meshes.jittered_square(8, 1)
    # a duplicated cell: its edges are shared by three cells, or twice in one direction
    bad = meshes.Mesh(xy=m.xy, cells=np.concatenate([m.cells, m.cells[5:6]]).astype(np.int32))
    with pytest.raises(dg.DgcError, match="dgc error -2"):
        dg.Discretization(bad, "advection", 2, dg.F32)
    # a fan of three triangles on one edge
    xy = np.array([[0, 0], [1, 0], [0.5, 1], [0.5, -1], [0.2, 2]], dtype=np.float64)
    cells = np.array([[0, 1, 2], [1, 0, 3], [0, 1, 4]], dtype=np.int32)
    with pytest.raises(dg.DgcError, match="dgc error -2"):
        dg.Discretization(meshes.Mesh(xy=xy, cells=cells), "advection", 2, dg.F32)
    # the same meshes through the host sort give the same verdict
    with pytest.raises(dg.DgcError, match="dgc error -2"):
        dg.host_mesh(bad, 2)


def test_gpu_topology_results_unchanged(force_gpu):
    """A handle built on the GPU path steps exactly like one built on the host path."""
    m = meshes.jittered_square(16, 4)
    a = dg.Discretization(m, "maxwell_te", 4, dg.F64)
    os.environ["DGC_GPU_TOPOLOGY_MIN"] = str(1 << 40)
    try:
        b = dg.Discretization(m, "maxwell_te", 4, dg.F64)
    finally:
        os.environ["DGC_GPU_TOPOLOGY_MIN"] = "0"
    x, y = a.node_xy()
    q = np.concatenate([np.sin(np.pi * x).ravel(), np.cos(y).ravel(), (x * y).ravel()])
    ra = a.download(a.rhs(a.upload(q), 0.0))
    rb = b.download(b.rhs(b.upload(q), 0.0))
    assert np.array_equal(ra, rb)
