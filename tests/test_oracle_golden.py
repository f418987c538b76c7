"""Pin the C oracle against the reference's own outputs (tests/golden/).

The goldens were produced by the reference's USE_CPU_ONLY code compiled from
its sources (tests/golden/make_golden.py).  Matrices and geometry must agree to
1e-13 relative; RHS and time steps to 1e-12 relative L2 (the parity bar).
"""
import glob
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, oracle

CASES = sorted(p for p in glob.glob(os.path.join(GOLDEN, "ref_*_N*.npz")) if "adv1d" not in p and "stokes" not in p)


def relerr(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def case_id(p):
    return os.path.basename(p)[4:-4]


@pytest.fixture(scope="module", params=CASES, ids=case_id)
def golden(request):
    d = dict(np.load(request.param))
    N = int(case_id(request.param).split("_N")[1])
    o = oracle.Oracle(d["mesh_xy"].reshape(-1, 2), d["mesh_cells"].reshape(-1, 3), N)
    return N, d, o


def test_golden_cases_exist():
    assert len(CASES) >= 15


def test_reference_element(golden):
    N, d, _ = golden
    r, s = oracle.nodes(N)
    assert relerr(r, d["r"]) < 1e-14 and relerr(s, d["s"]) < 1e-14
    F = oracle.face_nodes(N)
    for f in range(3):
        assert np.array_equal(F[f], d[f"F{f}"])
    V, Vr, Vs = oracle.vandermonde(N)
    assert relerr(V, d["V"]) < 1e-13
    assert relerr(Vr, d["Vr"]) < 1e-13 and relerr(Vs, d["Vs"]) < 1e-13


def test_operator_matrices(golden):
    N, d, _ = golden
    Dr, Ds, L, _ = oracle.operators(N, oracle.WEAK)
    assert relerr(Dr, d["Drw"]) < 1e-13 and relerr(Ds, d["Dsw"]) < 1e-13 and relerr(L, d["Lw"]) < 1e-13
    Dr, Ds, L, _ = oracle.operators(N, oracle.STRONG)
    assert relerr(Dr, d["Drs"]) < 1e-13 and relerr(Ds, d["Dss"]) < 1e-13 and relerr(L, d["Ls"]) < 1e-13


def test_discretisation_arrays(golden):
    N, d, o = golden
    a = o.arrays()
    for k in ("invJ", "J", "faceJ", "nx", "ny", "bx", "by"):
        assert relerr(a[k], d[k]) < 1e-14, k
    assert np.array_equal(a["nbCell"], d["nbCell"])
    assert np.array_equal(a["nbFace"], d["nbFace"])


def test_twin_half_facets(golden):
    """get_face_mapping: encoded (cell << 2 | face) twin of every half-facet
    (src/mesh/simple_triangular_mesh_2d.h:124-133, encoded_integer.h:49)."""
    N, d, o = golden
    a = o.arrays()
    K = o.K
    cell = np.repeat(np.arange(K), 3)
    face = np.tile(np.arange(3), K)
    bnd = a["nbCell"] == cell
    twin_cell = np.where(bnd, cell, a["nbCell"])
    twin_face = np.where(bnd, face, a["nbFace"])
    assert np.array_equal((twin_cell << 2) | twin_face, d["twin_hf"])


def test_advection_rhs_and_rk4(golden):
    N, d, o = golden
    p = oracle.problem(oracle.ADVECTION, 1.0, 1.0, oracle.BC_SINSIN)
    u0 = d["adv_u0"]
    assert relerr(o.exact(p, 0.0), u0) < 1e-15
    assert relerr(o.rhs(p, 0.05, u0), d["adv_rhs"]) < 1e-12
    dt = float(d["dt"][0])
    u1 = o.rk4_step(p, 0.0, dt, u0)
    assert relerr(u1, d["adv_rk4_1"]) < 1e-12
    u10, _ = o.run(p, oracle.RK4, 0.0, dt, 10, u0)
    assert relerr(u10, d["adv_rk4_10"]) < 1e-12


def test_maxwell_tm_rhs_and_rk4(golden):
    N, d, o = golden
    p = oracle.problem(oracle.MAXWELL_TM)
    q0 = d["mx_q0"]
    assert relerr(o.exact(p, 0.0), q0) < 1e-15
    assert relerr(o.rhs(p, 0.0, q0), d["mx_rhs"]) < 1e-12
    dt = float(d["dt"][0])
    assert relerr(o.rk4_step(p, 0.0, dt, q0), d["mx_rk4_1"]) < 1e-12
    q10, _ = o.run(p, oracle.RK4, 0.0, dt, 10, q0)
    assert relerr(q10, d["mx_rk4_10"]) < 1e-12


def test_laplace_apply(golden):
    N, d, o = golden
    out = o.laplace(d["lap_u"], dirichlet=True, tau_mode=0)
    assert relerr(out, d["lap_out"]) < 1e-12
    assert relerr(out, d["lap2_out"]) < 1e-12


def mixed_bc(bx, by):
    """The reference harness's mixed_bc object at boundary nodes: Dirichlet where
    x + 0.3 y < 0.2; exterior_val(x, y, 0) = 2 sin(x + y), exterior_grad_n(x, y, 0) = 2 cos(x y)."""
    return bx + 0.3 * by < 0.2, 2 * np.sin(bx + by), 2 * np.cos(bx * by)


def test_laplace_mixed_conditions_and_boundary_data(golden):
    N, d, o = golden
    a = o.arrays()
    isd, g, h = mixed_bc(a["bx"], a["by"])
    assert 0 < isd.sum() < isd.size      # both condition types present
    hom = o.laplace_bc(d["lapm_u"], isd)
    assert relerr(hom, d["lapm_hom"]) < 1e-12
    rhs = o.laplace_bc_rhs(isd, g, h)
    assert relerr(rhs, d["lapm_rhs"]) < 1e-12
    # operator() = apply_homogeneous - (the data contribution) (laplace_2d.h:121-128)
    assert relerr(hom - rhs, d["lapm_full"]) < 1e-12


def boundary_data(o):
    """The reference harness's boundary functions at the oracle's boundary nodes:
    grad / div exterior values 2 g - u with g = sin x cos y (and x y for div)."""
    a = o.arrays()
    bx, by = a["bx"], a["by"]
    return 2 * np.sin(bx) * np.cos(by), 2 * bx * by


def test_grad_and_div(golden):
    N, d, o = golden
    gs, gv = boundary_data(o)
    gx, gy = o.grad(d["gd_u"], gs, -1.0)
    assert relerr(gx, d["grad_dir_x"]) < 1e-12 and relerr(gy, d["grad_dir_y"]) < 1e-12
    gx, gy = o.grad(d["gd_u"], None, 1.0)
    assert relerr(gx, d["grad_mir_x"]) < 1e-12 and relerr(gy, d["grad_mir_y"]) < 1e-12
    assert relerr(o.div(d["gd_u"], d["gd_v"], gs, gv, -1.0), d["div_dir"]) < 1e-12


def test_known_answers_coarse_mesh():
    """The reference drivers' error norms on its own coarse mesh (K = 16)."""
    with open(os.path.join(GOLDEN, "ref_known_answers.json")) as f:
        known = json.load(f)
    d = dict(np.load(os.path.join(GOLDEN, "ref_coarse_N1.npz")))
    xy, cells = d["mesh_xy"].reshape(-1, 2), d["mesh_cells"].reshape(-1, 3)
    K = cells.shape[0]
    for N in (1, 2, 3, 4):
        rec = known["advection_10000_steps"][str(N)]
        o = oracle.Oracle(xy, cells, N)
        p = oracle.problem(oracle.ADVECTION, 1.0, 1.0, oracle.BC_SINSIN)
        l = 2.0 / np.sqrt(K)
        dt = (2.0 / 3.0) * (l / N) * (l / (2.0 + np.sqrt(2.0)))
        u, t = o.run(p, oracle.RK4, 0.0, dt, rec["steps"], o.exact(p, 0.0))
        mse = np.mean((o.exact(p, t) - u) ** 2)
        assert abs(t - rec["t_final"]) < 1e-9
        assert abs(mse - rec["mse"]) <= 1e-9 * rec["mse"]
    for N in (1, 2, 3, 4, 5, 6):
        rec = known["maxwell_T1"][str(N)]
        o = oracle.Oracle(xy, cells, N)
        p = oracle.problem(oracle.MAXWELL_TM)
        l = 2.0 / np.sqrt(K)
        dt = (2.0 / 3.0) * (l / N) * (l / (2.0 + np.sqrt(2.0)))
        q = o.exact(p, 0.0)
        t = 0.0
        for _ in range(rec["steps"]):
            h = min(dt, 1.0 - t)
            q = o.rk4_step(p, t, h, q)
            t += h
        n = o.K * o.Np
        mse = np.sum((o.exact(p, t) - q) ** 2) / n
        assert abs(mse - rec["mse"]) <= 1e-8 * rec["mse"]
