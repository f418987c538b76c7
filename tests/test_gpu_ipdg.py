"""GPU parity of the matrix-free laplace_2d (IPDG) operator and the
block-Jacobi PCG solvers, through the C ABI.

FP64 applies: the reference's own laplace_2d outputs (tests/golden/, tau = 1,
homogeneous Dirichlet; mixed Dirichlet / Neumann node types with boundary data
through apply_homogeneous, apply_inhomogeneous_as_rhs and operator()) and the
oracle (scaled tau, Neumann, mixed types) at 1e-12 relative.  FP32 applies: the
oracle at 2e-5.  Solvers: both methods reach the requested true FP64 residual
and agree with the oracle's FP64 PCG solution.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import dgc_gb300 as dg  # noqa: E402
from dgc_gb300 import meshes  # noqa: E402


def relerr(a, b):
    a, b = np.ravel(a), np.ravel(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module", autouse=True)
def built():
    from dgc_gb300 import build
    build.build()


def golden_mesh(d):
    return meshes.Mesh(xy=d["mesh_xy"].reshape(-1, 2), cells=d["mesh_cells"].reshape(-1, 3))


@pytest.mark.parametrize("case", [f"{m}_N{n}" for m in ("jit4", "coarse") for n in range(1, 7)] +
                         ["cells4_N1", "cells4_N2", "cells4_N3"])
def test_laplace_matches_reference(case):
    d = np.load(os.path.join(GOLDEN, f"ref_{case}.npz"))
    N = int(case.split("_N")[1])
    D = dg.Discretization(golden_mesh(d), "laplace", N, dg.F64, tau=dg.TAU_ONE, dirichlet=True)
    out = D.download(D.laplace(D.upload(d["lap_u"])))
    assert relerr(out, d["lap_out"]) < 1e-12
    # the FP32 kernels read their own penalty copy, also 1 here
    D32 = dg.Discretization(golden_mesh(d), "laplace", N, dg.F32, tau=dg.TAU_ONE, dirichlet=True)
    assert relerr(D32.download(D32.laplace(D32.upload(d["lap_u"]))), d["lap_out"]) < 2e-5


@pytest.mark.parametrize("N", range(1, 9))
@pytest.mark.parametrize("dirichlet", (True, False))
def test_laplace_scaled_tau_matches_oracle(N, dirichlet):
    m = meshes.jittered_square(5, 40 + N)
    o = oracle.Oracle(m.xy, m.cells, N)
    rng = np.random.default_rng(N)
    u = rng.standard_normal(o.K * o.Np)
    D = dg.Discretization(m, "laplace", N, dg.F64, tau=dg.TAU_SCALED, dirichlet=dirichlet)
    assert relerr(D.download(D.laplace(D.upload(u))), o.laplace(u, dirichlet, 1)) < 1e-12
    D32 = dg.Discretization(m, "laplace", N, dg.F32, tau=dg.TAU_SCALED, dirichlet=dirichlet)
    assert relerr(D32.download(D32.laplace(D32.upload(u))), o.laplace(u, dirichlet, 1)) < 2e-5


@pytest.mark.parametrize("N", (1, 2, 4, 6))
def test_spd_form_and_block_jacobi(N):
    m = meshes.jittered_square(4, 7 + N)
    o = oracle.Oracle(m.xy, m.cells, N)
    D = dg.Discretization(m, "laplace", N, dg.F64, tau=dg.TAU_SCALED)
    u = np.random.default_rng(3).standard_normal(o.K * o.Np)
    assert relerr(D.download(D.spd(D.upload(u))), o.spd(u, 1)) < 1e-12
    binv = D.block_jacobi().cpu().numpy()
    blocks = o.spd_blocks(1)
    ref = np.linalg.inv(blocks)
    assert relerr(binv, ref) < 1e-10
    # symmetric positive definite blocks
    assert np.allclose(blocks, blocks.transpose(0, 2, 1), atol=1e-10 * np.abs(blocks).max())
    assert (np.linalg.eigvalsh(0.5 * (blocks + blocks.transpose(0, 2, 1))) > 0).all()


def poisson_rhs(D, x, y):
    """b = M_J f for -laplace(u) = f, u = sin(pi x) sin(pi y)."""
    f = 2 * np.pi ** 2 * np.sin(np.pi * x) * np.sin(np.pi * y)
    fn = D.upload(f.reshape(-1))
    return D.mass(fn), np.sin(np.pi * x) * np.sin(np.pi * y)


@pytest.mark.parametrize("N", (2, 4))
def test_pcg_fp64_and_mixed_match_oracle(N):
    m = meshes.jittered_square(8, 100 + N)
    o = oracle.Oracle(m.xy, m.cells, N)
    D = dg.Discretization(m, "laplace", N, dg.F64, tau=dg.TAU_SCALED)
    x, y = D.node_xy()
    b, uex = poisson_rhs(D, x, y)
    b_ref = o.mass(2 * np.pi ** 2 * np.sin(np.pi * x) * np.sin(np.pi * y))
    assert relerr(D.download(b), b_ref) < 1e-13
    x64, st64 = D.pcg(b, mode=dg.SOLVE_FP64_PCG, rtol=1e-10)
    xmx, stmx = D.pcg(b, mode=dg.SOLVE_MIXED_IR, rtol=1e-10, inner_rtol=1e-4)
    assert st64["converged"] and st64["final_relres"] <= 1e-10
    assert stmx["converged"] and stmx["final_relres"] <= 1e-10 and stmx["outer_iterations"] >= 2
    xo, it, rel = o.pcg(b_ref, rtol=1e-12, tau_mode=1)
    assert it > 0 and rel <= 1e-12
    u64, umx = D.download(x64), D.download(xmx)
    assert relerr(u64, xo) < 1e-8
    assert relerr(umx, xo) < 1e-8
    # the discrete solution approximates sin(pi x) sin(pi y)
    assert relerr(u64, uex) < (0.02 if N == 2 else 2e-4)


def test_pcg_graph_and_plain_agree():
    m = meshes.jittered_square(10, 3)
    D = dg.Discretization(m, "laplace", 3, dg.F64, tau=dg.TAU_SCALED)
    x, y = D.node_xy()
    b, _ = poisson_rhs(D, x, y)
    xa, sa = D.pcg(b, rtol=1e-9, graph=True)
    xb, sb = D.pcg(b, rtol=1e-9, graph=False)
    # dot products are reduced with atomics, so runs agree to rounding only
    assert abs(sa["iterations"] - sb["iterations"]) <= 1
    assert relerr(xa.cpu().numpy(), xb.cpu().numpy()) < 1e-8


def test_pcg_reports_non_convergence():
    m = meshes.jittered_square(10, 3)
    D = dg.Discretization(m, "laplace", 3, dg.F64)
    x, y = D.node_xy()
    b, _ = poisson_rhs(D, x, y)
    _, st = D.pcg(b, rtol=1e-12, maxit=5, check=False)
    assert not st["converged"] and st["iterations"] <= 5
    with pytest.raises(dg.DgcError, match="tolerance"):
        D.pcg(b, rtol=1e-12, maxit=5)


def test_laplace_handle_rejects_time_stepping():
    m = meshes.jittered_square(3, 3)
    D = dg.Discretization(m, "laplace", 2, dg.F64)
    q = D.empty_state()
    with pytest.raises(dg.DgcError, match="laplace"):
        D.rhs(q, 0.0)
    A = dg.Discretization(m, "advection", 2, dg.F64)
    with pytest.raises(dg.DgcError, match="LAPLACE"):
        A.laplace(A.empty_state())


@pytest.mark.parametrize("prec", [dg.F64, dg.F32])
def test_apply_repeatable_at_scale(prec):
    """Many CTAs, several tiles each: repeated applies are bitwise identical and
    no barrier wait expires (a barrier re-armed before every warp had observed
    its previous phase used to leave CTAs waiting out their time limit)."""
    m = meshes.jittered_square(128, 7)   # K = 32768
    D = dg.Discretization(m, "laplace", 4, prec, tau=dg.TAU_SCALED)
    x, _ = D.node_xy()
    u = np.random.default_rng(1).standard_normal(x.size)
    U = D.upload(u.astype(np.float32) if prec == dg.F32 else u)
    first = D.download(D.spd(U))
    for _ in range(30):
        assert np.array_equal(D.download(D.spd(U)), first)
    lap = D.download(D.laplace(U))
    for _ in range(10):
        assert np.array_equal(D.download(D.laplace(U)), lap)
    D.check()


def test_mixed_ir_converges_at_scale():
    m = meshes.jittered_square(128, 7)   # K = 32768, N = 4
    D = dg.Discretization(m, "laplace", 4, dg.F64, tau=dg.TAU_SCALED)
    x, y = D.node_xy()
    f = 2 * np.pi ** 2 * np.sin(np.pi * x) * np.sin(np.pi * y)
    b = D.mass(D.upload(f.reshape(-1)))
    xs, st = D.pcg(b, mode=dg.SOLVE_MIXED_IR, rtol=1e-10, inner_rtol=1e-4, maxit=20000)
    assert st["converged"] and st["final_relres"] <= 1e-10
    ex = (np.sin(np.pi * x) * np.sin(np.pi * y)).reshape(-1)
    assert relerr(D.download(xs).reshape(-1), ex) < 1e-6
    D.check()


def mixed_bc(D):
    """The reference harness's mixed_bc at the handle's boundary nodes (Dirichlet where
    x + 0.3 y < 0.2; exterior_val(x, y, 0) = 2 sin(x + y), exterior_grad_n(x, y, 0) = 2 cos(x y))."""
    b = D.boundary_nodes()
    bx, by = b[:, 0], b[:, 1]
    return bx + 0.3 * by < 0.2, 2 * np.sin(bx + by), 2 * np.cos(bx * by)


@pytest.mark.parametrize("case", [f"{m}_N{n}" for m in ("jit4", "coarse") for n in range(1, 7)] +
                         ["cells4_N2", "fine_N1"])
def test_laplace_mixed_conditions_and_boundary_data_match_reference(case):
    d = np.load(os.path.join(GOLDEN, f"ref_{case}.npz"))
    N = int(case.split("_N")[1])
    D = dg.Discretization(golden_mesh(d), "laplace", N, dg.F64, tau=dg.TAU_ONE, dirichlet=True)
    isd, g, h = mixed_bc(D)
    D.set_bc_types(isd)
    hom = D.download(D.laplace(D.upload(d["lapm_u"])))
    assert relerr(hom, d["lapm_hom"]) < 1e-12
    rhs = D.download(D.laplace_bc_rhs(g, h))
    assert relerr(rhs, d["lapm_rhs"]) < 1e-12
    assert relerr(hom - rhs, d["lapm_full"]) < 1e-12      # laplace_2d::operator()
    with pytest.raises(dg.DgcError):                         # CG needs uniform Dirichlet
        D.pcg(D.upload(d["lapm_u"]))
    D.set_bc_types(None)
    D.check()


@pytest.mark.parametrize("N", (1, 3, 4, 6, 8))
def test_laplace_mixed_conditions_match_oracle(N):
    m = meshes.jittered_square(6, 70 + N)
    o = oracle.Oracle(m.xy, m.cells, N)
    rng = np.random.default_rng(N)
    u = rng.standard_normal(o.K * o.Np)
    for prec, tol in ((dg.F64, 1e-12), (dg.F32, 2e-5)):
        D = dg.Discretization(m, "laplace", N, prec, tau=dg.TAU_SCALED, dirichlet=True)
        isd, g, h = mixed_bc(D)
        D.set_bc_types(isd)
        assert relerr(D.download(D.laplace(D.upload(u))), o.laplace_bc(u, isd, tau_mode=1)) < tol
        assert relerr(D.download(D.laplace_bc_rhs(g, h)), o.laplace_bc_rhs(isd, g, h, tau_mode=1)) < tol


def dense_spd(D):
    """S (FP64, through dgc_laplace_spd_apply) as a dense matrix over the valid nodes."""
    K, Np, NpP = D.K, D.Np, D.NpP
    idx = [k * NpP + i for k in range(K) for i in range(Np)]
    cols = []
    for j in idx:
        e = torch.zeros(D.state_len, dtype=torch.float64, device="cuda")
        e[j] = 1.0
        cols.append(D.spd(e).cpu().numpy()[idx])
    return np.stack(cols, 1), idx


def test_shifted_spd_form_and_helmholtz_solve():
    m = meshes.jittered_square(4, 12)
    D = dg.Discretization(m, "laplace", 3, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    u = torch.from_numpy(np.random.default_rng(0).standard_normal(D.state_len)).cuda()
    s0 = D.spd(u).cpu().numpy()
    mu = D.mass(u).cpu().numpy()
    gamma = 37.5
    D.set_shift(gamma)
    assert relerr(D.spd(u).cpu().numpy(), s0 + gamma * mu) < 1e-12
    S, idx = dense_spd(D)
    assert np.allclose(S, S.T, atol=1e-10 * np.abs(S).max())
    b = D.mass(u)
    x, st = D.pcg(b, rtol=1e-12)
    xd = np.linalg.solve(S, b.cpu().numpy()[idx])
    assert st["converged"] and relerr(x.cpu().numpy()[idx], xd) < 1e-9
    xm, stm = D.pcg(b, mode=dg.SOLVE_MIXED_IR, rtol=1e-11)
    assert stm["converged"] and relerr(xm.cpu().numpy()[idx], xd) < 1e-8
    D.set_shift(0.0)
    assert relerr(D.spd(u).cpu().numpy(), s0) < 1e-15


def test_graphed_solve_after_shift_change_uses_new_operator():
    # the CG chunk graph captures the shift by value: a graphed solve, a new
    # shift, and a second graphed solve must solve the second system
    m = meshes.jittered_square(4, 14)
    D = dg.Discretization(m, "laplace", 3, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    u = torch.from_numpy(np.random.default_rng(3).standard_normal(D.state_len)).cuda()
    b = D.mass(u)
    for gamma in (0.0, 250.0, 11.0):
        D.set_shift(gamma)
        S, idx = dense_spd(D)
        xd = np.linalg.solve(S, b.cpu().numpy()[idx])
        for mode, tol in ((dg.SOLVE_FP64_PCG, 1e-9), (dg.SOLVE_MIXED_IR, 1e-8)):
            x, st = D.pcg(b, mode=mode, rtol=1e-12 if mode == dg.SOLVE_FP64_PCG else 1e-11, graph=True)
            assert st["converged"], (gamma, mode)
            assert relerr(x.cpu().numpy()[idx], xd) < tol, (gamma, mode)
    D.set_shift(0.0)


def test_all_neumann_pcg_solves_the_consistent_system():
    m = meshes.jittered_square(4, 13)
    D = dg.Discretization(m, "laplace", 2, dg.F64, tau=dg.TAU_SCALED, dirichlet=False)
    S, idx = dense_spd(D)
    w = np.linalg.eigvalsh(0.5 * (S + S.T))
    assert abs(w[0]) < 1e-8 * w[-1] and w[1] > 1e-8 * w[-1]     # one-dimensional null space
    rng = np.random.default_rng(1)
    bv = np.zeros(D.state_len)
    bv[idx] = rng.standard_normal(len(idx))
    b = torch.from_numpy(bv).cuda()
    for mode in (dg.SOLVE_FP64_PCG, dg.SOLVE_MIXED_IR):
        x, st = D.pcg(b, mode=mode, rtol=1e-10)
        assert st["converged"]
        xs = x.cpu().numpy()[idx]
        bp = bv[idx] - bv[idx].mean()
        ref = np.linalg.lstsq(S, bp, rcond=None)[0]
        assert abs(xs.mean()) < 1e-10 * np.abs(xs).max()
        assert relerr(xs, ref - ref.mean()) < 1e-7
