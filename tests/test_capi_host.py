"""C-ABI library checks that need no GPU: it builds, loads, exports every
symbol declared in include/*.h, and its host-side set-up (nodes, operator
matrices, mesh topology, geometry) agrees with the reference's goldens."""
import glob
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

import dgc_gb300 as dg
from dgc_gb300 import build, meshes


@pytest.fixture(scope="module")
def L():
    build.build()
    return dg.lib()


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names.update(re.findall(r"\b(dgc_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_exports_every_declared_symbol(L):
    syms = declared_symbols()
    assert len(syms) >= 19
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def relerr(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


@pytest.mark.parametrize("N", range(1, 7))
def test_nodes_and_operators_match_reference(L, N):
    d = np.load(os.path.join(GOLDEN, f"ref_jit4_N{N}.npz"))
    r, s = dg.ref_nodes(N)
    assert relerr(r, d["r"]) < 1e-14 and relerr(s, d["s"]) < 1e-14
    assert relerr(dg.ref_operator(N, dg.OP_V), d["V"]) < 1e-13
    for which, key in ((dg.OP_DR_WEAK, "Drw"), (dg.OP_DS_WEAK, "Dsw"), (dg.OP_LIFT, "Lw"),
                       (dg.OP_DR_STRONG, "Drs"), (dg.OP_DS_STRONG, "Dss")):
        assert relerr(dg.ref_operator(N, which), d[key]) < 1e-13, key


@pytest.mark.parametrize("N", (7, 8))
def test_high_order_operators_against_oracle(L, N):
    """Orders 7, 8: no reference pin (its Gauss-Lobatto table stops at 7
    points); agree with the oracle's independent restatement."""
    import oracle
    r, s = dg.ref_nodes(N)
    ro, so = oracle.nodes(N)
    assert relerr(r, ro) < 1e-13 and relerr(s, so) < 1e-13
    Dr, Ds, Lf, _ = oracle.operators(N, oracle.WEAK)
    assert relerr(dg.ref_operator(N, dg.OP_DR_WEAK), Dr) < 1e-12
    assert relerr(dg.ref_operator(N, dg.OP_LIFT), Lf) < 1e-12


@pytest.mark.parametrize("case", ["jit4_N4", "coarse_N3", "cells4_N2"])
def test_host_mesh_matches_reference_discretisation(L, case):
    d = np.load(os.path.join(GOLDEN, f"ref_{case}.npz"))
    N = int(case.split("_N")[1])
    m = meshes.Mesh(xy=d["mesh_xy"].reshape(-1, 2), cells=d["mesh_cells"].reshape(-1, 3))
    geom, nbr, nb = dg.host_mesh(m, N)
    K = m.num_cells
    inv = d["invJ"].reshape(K, 4)
    assert np.allclose(geom[:, 0:4], inv, rtol=1e-13, atol=1e-13)
    assert np.allclose(geom[:, 4], d["J"], rtol=1e-14)
    assert np.allclose(geom[:, 5:8], d["faceJ"].reshape(K, 3), rtol=1e-14)
    assert np.allclose(geom[:, 8:11], d["nx"].reshape(K, 3), atol=1e-15)
    assert np.allclose(geom[:, 11:14], d["ny"].reshape(K, 3), atol=1e-15)
    cell = d["nbCell"].reshape(K, 3)
    face = d["nbFace"].reshape(K, 3)
    bnd = cell == np.arange(K)[:, None]
    assert nb * (N + 1) == len(d["bx"])
    # interior: encoded twin; boundary: -(1 + b) with offset = b * Nfp
    exp = np.where(bnd, -(1 + face // (N + 1)), (cell << 2) | face)
    assert np.array_equal(nbr[:, :3], exp)


def test_mesh_validation_errors(L):
    m = meshes.jittered_square(2, 0)
    bad = meshes.Mesh(xy=m.xy, cells=m.cells[:, ::-1].copy())  # clockwise
    with pytest.raises(dg.DgcError, match="clockwise"):
        dg.host_mesh(bad, 2)
    bad = meshes.Mesh(xy=m.xy, cells=np.where(m.cells == 0, 99, m.cells).astype(np.int32))
    with pytest.raises(dg.DgcError, match="out of range"):
        dg.host_mesh(bad, 2)
    with pytest.raises(dg.DgcError, match="order"):
        dg.host_mesh(m, 9)
    three = meshes.Mesh(xy=np.array([[0, 0], [1, 0], [0, 1], [1, 1], [0.5, -1]], float),
                        cells=np.array([[0, 1, 2], [1, 3, 2], [0, 4, 1], [1, 2, 0]], np.int32))
    with pytest.raises(dg.DgcError):
        dg.host_mesh(three, 1)


def test_jittered_mesh_properties():
    m = meshes.jittered_square(32, 5)
    assert m.num_cells == 2048
    p = m.xy[m.cells]
    area = 0.5 * ((p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) -
                  (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1]))
    assert (area > 0).all() and abs(area.sum() - 4.0) < 1e-12
    onb = (np.abs(np.abs(m.xy) - 1.0) < 1e-15).any(axis=1)
    assert onb.sum() == 4 * 32
    m2 = meshes.jittered_square(32, 5)
    assert np.array_equal(m.xy, m2.xy)


def test_create_from_arrays_rejects_inconsistent_interfaces(L):
    """The reference-array path validates the interface map before it touches a
    GPU: an asymmetric twin or an out-of-sequence boundary offset is refused."""
    d = dict(np.load(os.path.join(GOLDEN, "ref_jit4_N2.npz")))
    K = d["J"].size
    cell = d["nbCell"].reshape(K, 3).copy()
    k, f = next((k, f) for k in range(K) for f in range(3) if cell[k, f] != k)
    cell[k, f] = (cell[k, f] + 1) % K if (cell[k, f] + 1) % K != k else (cell[k, f] + 2) % K
    bad = dict(d, nbCell=cell.reshape(-1))
    with pytest.raises(dg.DgcError, match="interface map|boundary node"):
        dg.Discretization.from_arrays(bad, "advection", 2)
    face = d["nbFace"].reshape(K, 3).copy()
    kb, fb = next((k, f) for k in range(K) for f in range(3) if d["nbCell"].reshape(K, 3)[k, f] == k and face[k, f] > 0)
    face[kb, fb] += 1
    with pytest.raises(dg.DgcError, match="offset"):
        dg.Discretization.from_arrays(dict(d, nbFace=face.reshape(-1)), "advection", 2)
