"""GPU parity of the fused DG RHS / time-stage kernels, through the C ABI.

FP64 path: the reference's own outputs (tests/golden/) and the oracle, at
1e-12 relative L2 per time step (the parity bar).  FP32 path: the oracle at a
stated tolerance (FP32 contractions; 2e-5 relative per step).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import dgc_gb300 as dg  # noqa: E402
from dgc_gb300 import meshes  # noqa: E402

TOL64 = 1e-12
TOL32 = 2e-5


def relerr(a, b):
    a, b = np.ravel(a), np.ravel(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module", autouse=True)
def built():
    from dgc_gb300 import build
    build.build()
    assert torch.cuda.is_available()


def golden_mesh(d):
    """The case's mesh; read from the reference's own .msh file by dgc_msh_read
    when the case has one (so those cases also test the importer end to end)."""
    if "msh_source" in d.files:
        import tempfile
        with tempfile.TemporaryDirectory() as tmp:
            path = os.path.join(tmp, "mesh.msh")
            with open(path, "wb") as f:
                f.write(bytes(d["msh_source"]))
            return dg.read_msh(path)
    return meshes.Mesh(xy=d["mesh_xy"].reshape(-1, 2), cells=d["mesh_cells"].reshape(-1, 3))


CASES = [f"{m}_N{n}" for m in ("jit4", "coarse") for n in range(1, 7)] + ["fine_N1"]


@pytest.mark.parametrize("case", CASES)
def test_advection_matches_reference(case):
    d = np.load(os.path.join(GOLDEN, f"ref_{case}.npz"))
    N = int(case.split("_N")[1])
    D = dg.Discretization(golden_mesh(d), "advection", N, dg.F64, ax=1.0, ay=1.0, bc=dg.BC_SINSIN)
    u0 = D.upload(d["adv_u0"])
    assert relerr(D.download(D.rhs(u0, 0.05)), d["adv_rhs"]) < TOL64
    dt = float(d["dt"][0])
    work = [D.empty_state() for _ in range(3)]
    q = u0.clone()
    t = 0.0
    for i in range(10):
        D.rk4_step(q, t, dt, work)
        t += dt
        if i == 0:
            assert relerr(D.download(q), d["adv_rk4_1"]) < TOL64
    assert relerr(D.download(q), d["adv_rk4_10"]) < TOL64
    D.check()


@pytest.mark.parametrize("case", CASES)
def test_maxwell_tm_matches_reference(case):
    d = np.load(os.path.join(GOLDEN, f"ref_{case}.npz"))
    N = int(case.split("_N")[1])
    D = dg.Discretization(golden_mesh(d), "maxwell_tm", N, dg.F64)
    q0 = D.upload(d["mx_q0"])
    assert relerr(D.download(D.rhs(q0, 0.0)), d["mx_rhs"]) < TOL64
    dt = float(d["dt"][0])
    work = [D.empty_state() for _ in range(3)]
    q = q0.clone()
    for i in range(10):
        D.rk4_step(q, i * dt, dt, work)
        if i == 0:
            assert relerr(D.download(q), d["mx_rk4_1"]) < TOL64
    assert relerr(D.download(q), d["mx_rk4_10"]) < TOL64


def test_reference_matrices_injected_bitwise_path():
    """dgc_set_operators with the reference's own m_Dr/m_Ds/m_L."""
    d = np.load(os.path.join(GOLDEN, "ref_jit4_N5.npz"))
    D = dg.Discretization(golden_mesh(d), "advection", 5, dg.F64)
    Np = 21
    D.set_operators(0, d["Drw"].reshape(Np, Np), d["Dsw"].reshape(Np, Np), d["Lw"].reshape(Np, 18))
    u0 = D.upload(d["adv_u0"])
    assert relerr(D.download(D.rhs(u0, 0.05)), d["adv_rhs"]) < 1e-13


PROBLEMS = [
    ("adv_gauss", oracle.ADVECTION, dict(ax=1.0, ay=0.5, bc=dg.BC_GAUSS)),
    ("adv_sinsin_general_a", oracle.ADVECTION, dict(ax=-0.7, ay=0.4, bc=dg.BC_SINSIN)),
    ("maxwell_te", oracle.MAXWELL_TE, {}),
    ("maxwell_tm", oracle.MAXWELL_TM, {}),
]


def make_pair(n, seed, N, kind, kw, prec=dg.F64):
    m = meshes.jittered_square(n, seed)
    phys = {oracle.ADVECTION: "advection", oracle.MAXWELL_TE: "maxwell_te", oracle.MAXWELL_TM: "maxwell_tm"}[kind]
    D = dg.Discretization(m, phys, N, prec, **kw)
    o = oracle.Oracle(m.xy, m.cells, N)
    p = oracle.problem(kind, kw.get("ax", 1.0), kw.get("ay", 1.0), kw.get("bc", 0))
    return m, D, o, p


@pytest.mark.parametrize("N", range(1, 9))
@pytest.mark.parametrize("name,kind,kw", PROBLEMS, ids=[p[0] for p in PROBLEMS])
def test_lserk4_matches_oracle_all_orders(N, name, kind, kw):
    _, D, o, p = make_pair(5, 11 + N, N, kind, kw)
    q0 = o.exact(p, 0.13)
    dt = 0.5 * D.info.min_edge / ((N + 1) ** 2)
    # single RHS
    q = D.upload(q0)
    assert relerr(D.download(D.rhs(q, 0.21)), o.rhs(p, 0.21, q0)) < TOL64
    # three LSERK4 steps, per-step comparison
    res = D.empty_state()
    qb = D.empty_state()
    qo, ro = q0.copy(), np.zeros_like(q0)
    t = 0.13
    for _ in range(3):
        D.lserk4_step(q, qb, res, t, dt)
        q, qb = qb, q
        qo, ro = o.lserk4_step(p, t, dt, qo, ro)
        t += dt
        assert relerr(D.download(q), qo) < TOL64
    D.check()


@pytest.mark.parametrize("name,kind,kw", PROBLEMS, ids=[p[0] for p in PROBLEMS])
@pytest.mark.parametrize("N", (2, 4, 6, 8))
def test_fp32_matches_oracle(N, name, kind, kw):
    _, D, o, p = make_pair(6, 3 + N, N, kind, kw, prec=dg.F32)
    q0 = o.exact(p, 0.05)
    q = D.upload(q0)
    r32 = D.download(D.rhs(q, 0.05))
    assert relerr(r32, o.rhs(p, 0.05, q0)) < TOL32
    dt = 0.5 * D.info.min_edge / ((N + 1) ** 2)
    res, qb = D.empty_state(), D.empty_state()
    qo, ro = q0.copy(), np.zeros_like(q0)
    for s in range(4):
        D.lserk4_step(q, qb, res, 0.05 + s * dt, dt)
        q, qb = qb, q
        qo, ro = o.lserk4_step(p, 0.05 + s * dt, dt, qo, ro)
    assert relerr(D.download(q), qo) < TOL32


def test_config1_advection_parity_and_error():
    """2D advection a = (1, 0.5), 32x32 jittered mesh (K = 2048), N = 4, FP64,
    Gaussian pulse, LSERK4 with dt = 0.5 min(h) / ((N+1)^2 |a|): per-step match
    to the oracle at 1e-12 and the same L2 error against the exact solution."""
    N = 4
    kw = dict(ax=1.0, ay=0.5, bc=dg.BC_GAUSS)
    m, D, o, p = make_pair(32, 2024, N, oracle.ADVECTION, kw)
    dt0 = 0.5 * meshes.min_edge_length(m) / ((N + 1) ** 2 * np.hypot(1.0, 0.5))
    nsteps = 40
    q0 = o.exact(p, 0.0)
    qa, qb, res = D.upload(q0), D.empty_state(), D.empty_state()
    qo, ro = q0.copy(), np.zeros_like(q0)
    t = 0.0
    worst = 0.0
    for s in range(nsteps):
        D.lserk4_step(qa, qb, res, t, dt0)
        qa, qb = qb, qa
        qo, ro = o.lserk4_step(p, t, dt0, qo, ro)
        t += dt0
        if s % 8 == 7:
            worst = max(worst, relerr(D.download(qa), qo))
    assert worst < TOL64
    ex = o.exact(p, t)
    e_gpu = relerr(D.download(qa), ex)
    e_orc = relerr(qo, ex)
    assert abs(e_gpu - e_orc) <= 1e-9 * e_orc + 1e-14


def test_graph_run_equals_step_loop():
    _, D, o, p = make_pair(8, 5, 5, oracle.ADVECTION, dict(ax=1.0, ay=0.5, bc=dg.BC_GAUSS))
    q0 = o.exact(p, 0.0)
    dt = 0.5 * D.info.min_edge / 36.0
    a1, b1, r1 = D.upload(q0), D.empty_state(), D.empty_state()
    a2, b2, r2 = D.upload(q0), D.empty_state(), D.empty_state()
    fin1 = D.lserk4_run(a1, b1, r1, 0.0, dt, 45, graph=True)
    fin2 = D.lserk4_run(a2, b2, r2, 0.0, dt, 45, graph=False)
    assert torch.equal(fin1, fin2)
    qo, _ = o.run(p, oracle.LSERK4, 0.0, dt, 45, q0)
    assert relerr(D.download(fin1), qo) < TOL64


def test_layout_roundtrip_and_reference_gpu_layout():
    _, D, o, p = make_pair(4, 1, 3, oracle.MAXWELL_TE, {})
    q0 = o.exact(p, 0.3)
    q = D.upload(q0)
    back = D.download(q)
    assert np.array_equal(back, q0)
    ref_gpu = D.from_native(q, dg.LAYOUT_REF_GPU).cpu().numpy().reshape(3, D.Np, D.K)
    assert np.array_equal(ref_gpu, q0.reshape(3, D.K, D.Np).transpose(0, 2, 1))
    q2 = D.to_native(torch.from_numpy(ref_gpu.copy().reshape(-1)).cuda(), dg.LAYOUT_REF_GPU)
    assert torch.equal(q2, q)


def test_axpy_matches_reference_axpy():
    _, D, o, p = make_pair(3, 2, 2, oracle.ADVECTION, {})
    x = torch.randn(D.state_len, dtype=torch.float64, device="cuda")
    y = torch.randn(D.state_len, dtype=torch.float64, device="cuda")
    out = D.empty_state()
    D.axpy(0.37, x, y, out)
    # the kernel contracts a*x + y into one FMA; torch rounds the product first
    assert torch.allclose(out, 0.37 * x + y, rtol=4e-16, atol=4e-16)


def test_argument_errors():
    _, D, o, p = make_pair(3, 2, 2, oracle.MAXWELL_TE, {})
    q = D.empty_state()
    with pytest.raises(dg.DgcError, match="alias"):
        D.rhs(q, 0.0, out=q)
    big = torch.zeros(D.state_len + 4, dtype=torch.float64, device="cuda")
    with pytest.raises(dg.DgcError, match="aligned"):
        D.rhs(big[1:], 0.0)
    with pytest.raises(dg.DgcError, match="distinct"):
        D.lserk4_step(q, q, D.empty_state(), 0.0, 0.1)
    with pytest.raises(dg.DgcError):
        dg.Discretization(meshes.jittered_square(2, 0), "maxwell_te", 9)


@pytest.mark.parametrize("case", ["jit4_N4", "coarse_N3", "cells4_N2", "coarse_N6"])
def test_create_from_reference_arrays_matches_reference(case):
    """dgc_create_from_arrays with the reference's own fill_* arrays (the goldens
    hold what simple_discretization_2d produced): RHS and RK4 steps of both
    examples against the reference at 1e-12."""
    d = np.load(os.path.join(GOLDEN, f"ref_{case}.npz"))
    N = int(case.split("_N")[1])
    D = dg.Discretization.from_arrays(d, "advection", N, dg.F64, ax=1.0, ay=1.0, bc=dg.BC_SINSIN)
    u0 = D.upload(d["adv_u0"])
    assert relerr(D.download(D.rhs(u0, 0.05)), d["adv_rhs"]) < TOL64
    dt = float(d["dt"][0])
    work = [D.empty_state() for _ in range(3)]
    q = u0.clone()
    for i in range(10):
        D.rk4_step(q, i * dt, dt, work)
    assert relerr(D.download(q), d["adv_rk4_10"]) < TOL64
    M = dg.Discretization.from_arrays(d, "maxwell_tm", N, dg.F64)
    q0 = M.upload(d["mx_q0"])
    assert relerr(M.download(M.rhs(q0, 0.0)), d["mx_rhs"]) < TOL64
    with pytest.raises(dg.DgcError, match="vertex coordinates"):
        M.node_xy()
    D.check()
    M.check()
