"""GPU parity of the weak-form gradient and divergence (dgc_grad_apply,
dgc_div_apply; grad_2d / div_2d) through the C ABI.

FP64: the reference's own grad_2d / div_2d outputs (tests/golden/, boundary
data u+ = 2 g - u- and u+ = u-) at 1e-12 relative, and the oracle at orders 7
and 8.  FP32: the oracle at 2e-5.  At 32768 elements: exactness on linear
fields with exact boundary data (a size-independent property).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import dgc_gb300 as dg  # noqa: E402
from dgc_gb300 import meshes  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def built():
    from dgc_gb300 import build
    build.build()


def relerr(a, b):
    a, b = np.ravel(a), np.ravel(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def golden_mesh(d):
    return meshes.Mesh(xy=d["mesh_xy"].reshape(-1, 2), cells=d["mesh_cells"].reshape(-1, 3))


def bdata(D):
    b = D.boundary_nodes()
    return 2 * np.sin(b[:, 0]) * np.cos(b[:, 1]), 2 * b[:, 0] * b[:, 1]


@pytest.mark.parametrize("physics", ["advection", "laplace"])
@pytest.mark.parametrize("case", [f"{m}_N{n}" for m in ("jit4", "coarse") for n in range(1, 7)] +
                         ["cells4_N1", "cells4_N2", "cells4_N3"])
def test_grad_div_match_reference(case, physics):
    d = np.load(os.path.join(GOLDEN, f"ref_{case}.npz"))
    N = int(case.split("_N")[1])
    D = dg.Discretization(golden_mesh(d), physics, N, dg.F64)
    gs, gv = bdata(D)
    u, v = D.upload(d["gd_u"]), D.upload(d["gd_v"])
    gx, gy = D.grad(u, gs, -1.0)
    assert relerr(D.download(gx), d["grad_dir_x"]) < 1e-12
    assert relerr(D.download(gy), d["grad_dir_y"]) < 1e-12
    gx, gy = D.grad(u, None, 1.0)
    assert relerr(D.download(gx), d["grad_mir_x"]) < 1e-12
    assert relerr(D.download(gy), d["grad_mir_y"]) < 1e-12
    assert relerr(D.download(D.div(u, v, gs, gv, -1.0)), d["div_dir"]) < 1e-12


@pytest.mark.parametrize("N", range(1, 9))
def test_grad_div_match_oracle(N):
    m = meshes.jittered_square(6, 90 + N)
    o = oracle.Oracle(m.xy, m.cells, N)
    rng = np.random.default_rng(N)
    u, v = rng.standard_normal(o.K * o.Np), rng.standard_normal(o.K * o.Np)
    for prec, tol in ((dg.F64, 1e-12), (dg.F32, 2e-5)):
        D = dg.Discretization(m, "advection", N, prec)
        gs, gv = bdata(D)
        gx, gy = D.grad(D.upload(u), gs, -1.0)
        rx, ry = o.grad(u, gs, -1.0)
        assert relerr(D.download(gx), rx) < tol and relerr(D.download(gy), ry) < tol
        dd = D.div(D.upload(u), D.upload(v), gs, gv, -1.0)
        assert relerr(D.download(dd), o.div(u, v, gs, gv, -1.0)) < tol
        D.check()


def test_linear_fields_exact_at_scale():
    m = meshes.jittered_square(128, 5)   # K = 32768
    D = dg.Discretization(m, "laplace", 4, dg.F64)
    x, y = D.node_xy()
    b = D.boundary_nodes()
    a1, a2, a3 = 0.7, -1.3, 0.25
    u = a1 * x + a2 * y + a3
    gx, gy = D.grad(D.upload(u), 2 * (a1 * b[:, 0] + a2 * b[:, 1] + a3), -1.0)
    assert np.max(np.abs(D.download(gx) - a1)) < 1e-9
    assert np.max(np.abs(D.download(gy) - a2)) < 1e-9
    dv = D.div(D.upload(x), D.upload(y), 2 * b[:, 0], 2 * b[:, 1], -1.0)
    assert np.max(np.abs(D.download(dv) - 2.0)) < 1e-9


def test_grad_div_reject_vector_handles():
    m = meshes.jittered_square(3, 1)
    D = dg.Discretization(m, "maxwell_te", 3, dg.F32)
    q = D.empty_state()
    with pytest.raises(dg.DgcError):
        D.grad(q)


def test_checkpoint_round_trip_and_rejection(tmp_path):
    m = meshes.jittered_square(10, 3)
    D = dg.Discretization(m, "maxwell_te", 5, dg.F32)
    q = torch.randn(D.state_len, device="cuda")
    path = str(tmp_path / "state.bin")
    D.save_state(path, q, 0.375)
    r, t = D.load_state(path)
    assert t == 0.375 and torch.equal(r, q)
    with pytest.raises(dg.DgcError):                      # another order
        dg.Discretization(m, "maxwell_te", 4, dg.F32).load_state(path)
    with pytest.raises(dg.DgcError):                      # another precision
        dg.Discretization(m, "maxwell_te", 5, dg.F64).load_state(path)
    raw = bytearray(open(path, "rb").read())
    raw[-1] ^= 0xFF
    open(path, "wb").write(bytes(raw))
    with pytest.raises(dg.DgcError):                      # corrupted payload
        D.load_state(path)
