"""Coarse space of the two-level learned preconditioner (csrc/coarse.cu).

* dgc_coarse_apply equals P A_c^-1 P^T r formed densely in NumPy from the
  oracle's SPD matrix, the library's aggregates and its smoothing weight
  (P = (I - omega Binv S) P0, Binv the inverse of S's diagonal blocks), with
  and without a shift, at 1e-10: this checks the colour-probed assembly of
  A_c and its GPU inversion.
* Aggregates: every cell in exactly one, each face-connected.
* Flexible CG with M = Binv + coarse (zero network) reaches the same solution
  as block-Jacobi PCG in several times fewer iterations, and the learned solve
  with the coarse term never needs its fallback.
"""
import numpy as np
import pytest

from conftest import oracle

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


def poisson_rhs(D):
    x, y = D.node_xy()
    f = 2 * np.pi ** 2 * np.sin(np.pi * x) * np.sin(np.pi * y) + 3 * np.cos(5 * x * y)
    return D.mass(D.upload(f.reshape(-1)))


@pytest.mark.parametrize("n_side,N,size,shift", [(6, 1, 3, 0.0), (6, 2, 4, 0.0), (6, 3, 7, 0.0), (6, 2, 5, 40.0),
                                                  (26, 1, 3, 0.0)])
def test_coarse_apply_matches_dense(n_side, N, size, shift):
    """(26, 1, 3): 1352 cells, ~450 aggregates sharing colours (the probe
    separates them); the 6 x 6 cases have one aggregate per colour."""
    m = meshes.jittered_square(n_side, 2)
    D = dg.Discretization(m, "laplace", N, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    if shift:
        D.set_shift(shift)
    D.coarse_build(size)
    agg, na, nc, om = D.coarse_info()
    assert agg.min() == 0 and agg.max() == na - 1 and nc >= 1 and 0.0 < om < 2.0
    if n_side > 6:
        assert nc < na / 4
    check_dense(D, m, N, shift, 1e-10, 1e-4)


def check_dense(D, m, N, shift, tol64, tol32):
    """D.coarse_apply against P A_c^-1 P^T r formed densely from the oracle's S."""
    agg, na, _, om = D.coarse_info()
    O = oracle.Oracle(m.xy, m.cells, N)
    n = D.K * D.Np
    S = np.stack([O.spd(e) for e in np.eye(n)], axis=1)
    if shift:
        S = S + shift * np.stack([O.mass(e) for e in np.eye(n)], axis=1)
    P0 = np.zeros((n, na))
    Binv = np.zeros((n, n))
    for k in range(D.K):
        b = slice(k * D.Np, (k + 1) * D.Np)
        P0[b, agg[k]] = 1.0
        Binv[b, b] = np.linalg.inv(S[b, b])
    P = P0 - om * Binv @ S @ P0
    Ac = P.T @ S @ P
    rng = np.random.default_rng(N)
    for _ in range(2):
        r = rng.standard_normal(n)
        ref = P @ np.linalg.solve(Ac, P.T @ r)
        assert relerr(D.download(D.coarse_apply(D.upload(r))), ref) < tol64
        assert relerr(D.download(D.coarse_apply(D.upload(r), precision=dg.F32)), ref) < tol32


@pytest.mark.parametrize("N", [5, 6, 7, 8])
def test_coarse_apply_high_orders(N):
    """Orders whose padded element (NpP = 24, 28, 36, 48) gives CTAs of 240-252
    threads in the block-Jacobi apply."""
    m = meshes.jittered_square(4, 2)
    D = dg.Discretization(m, "laplace", N, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    D.coarse_build(4)
    check_dense(D, m, N, 0.0, 1e-9, 1e-3)


@pytest.mark.parametrize("size", [4, 16, 32])
def test_aggregates_cover_and_connect(size):
    m = meshes.jittered_square(32, 5)
    D = dg.Discretization(m, "laplace", 2, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    D.coarse_build(size)
    agg, na, _, _ = D.coarse_info()
    nbr, _ = D.neighbors()
    counts = np.bincount(agg, minlength=na)
    assert counts.min() >= 1 and counts.sum() == D.K
    assert np.median(counts) >= size * 0.5
    for a in range(na):
        cells = np.flatnonzero(agg == a)
        seen, stack = {cells[0]}, [cells[0]]
        while stack:
            k = stack.pop()
            for f in range(3):
                nb = nbr[k, f]
                if nb >= 0 and agg[nb >> 2] == a and (nb >> 2) not in seen:
                    seen.add(nb >> 2)
                    stack.append(nb >> 2)
        assert len(seen) == len(cells), a


def test_two_level_fcg_cuts_iterations():
    m = meshes.jittered_square(48, 3)
    D = dg.Discretization(m, "laplace", 3, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    b = poisson_rhs(D)
    xp, stp = D.pcg(b, rtol=1e-10)
    base = dg.MPNN(D, layers=1, seed=0)    # zero output layer
    base.set_coarse(16)
    xf, stf = base.fpcg(b, rtol=1e-10)
    assert stf["converged"] and stf["final_relres"] <= 1e-10
    print(f"two-level FCG {stf['iterations']} vs block-Jacobi PCG {stp['iterations']} iterations")
    assert stf["iterations"] * 4 < stp["iterations"], (stf["iterations"], stp["iterations"])
    assert relerr(D.download(xf), D.download(xp)) < 1e-8
    # the coarse term off again: back to block-Jacobi's iteration count
    base.set_coarse(0)
    _, st0 = base.fpcg(b, rtol=1e-10)
    assert abs(st0["iterations"] - stp["iterations"]) <= max(2, 0.05 * stp["iterations"])


def test_learned_solve_two_level_needs_no_fallback():
    m = meshes.jittered_square(32, 8)
    D = dg.Discretization(m, "laplace", 4, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    b = poisson_rhs(D)
    xp, stp = D.pcg(b, rtol=1e-10)
    net = dg.MPNN(D, layers=4, seed=3)
    net.set_coarse(16)
    x, st = net.solve(b, rtol=1e-10, fcg_maxit=stp["iterations"] // 2)
    assert not st["fell_back"] and st["final_relres"] <= 1e-10
    assert relerr(D.download(x), D.download(xp)) < 1e-8


def test_coarse_apply_neumann_is_pseudo_inverse():
    """All-Neumann: A_c is singular (P 1 = 1); on zero-sum residuals the
    regularised inverse equals A_c's pseudo-inverse."""
    m = meshes.jittered_square(6, 4)
    D = dg.Discretization(m, "laplace", 2, dg.F64, tau=dg.TAU_ONE, dirichlet=False)
    D.coarse_build(4)
    agg, na, _, om = D.coarse_info()
    O = oracle.Oracle(m.xy, m.cells, 2)
    n = D.K * D.Np
    S = np.stack([O.laplace(e, dirichlet=False) for e in np.eye(n)], axis=1)
    S = -np.stack([O.mass(c) for c in S.T], axis=1)       # -J M A
    P0 = np.zeros((n, na))
    Binv = np.zeros((n, n))
    for k in range(D.K):
        b = slice(k * D.Np, (k + 1) * D.Np)
        P0[b, agg[k]] = 1.0
        Binv[b, b] = np.linalg.inv(S[b, b])
    P = P0 - om * Binv @ S @ P0
    Ac = P.T @ S @ P
    r = np.random.default_rng(0).standard_normal(n)
    r -= r.mean()
    ref = P @ np.linalg.pinv(Ac, rcond=1e-12) @ P.T @ r
    assert relerr(D.download(D.coarse_apply(D.upload(r))), ref) < 1e-9


@pytest.mark.parametrize("mode", [dg.SOLVE_TWO_LEVEL, dg.SOLVE_TWO_LEVEL_MIXED])
@pytest.mark.parametrize("dirichlet", [True, False])
def test_two_level_mode_matches_fp64_pcg(dirichlet, mode):
    m = meshes.jittered_square(40, 6)
    D = dg.Discretization(m, "laplace", 3, dg.F64, tau=dg.TAU_SCALED if dirichlet else dg.TAU_ONE,
                          dirichlet=dirichlet)
    b = poisson_rhs(D)
    xp, stp = D.pcg(b, rtol=1e-10)
    D.coarse_build(8)
    xt, stt = D.pcg(b, mode=mode, rtol=1e-10)
    print(f"dirichlet={dirichlet} mode={mode}: two-level {stt['iterations']} vs block-Jacobi "
          f"{stp['iterations']} iterations")
    assert stt["converged"] and stt["final_relres"] <= 1e-10
    assert stt["iterations"] * 2 < stp["iterations"]
    assert relerr(D.download(xt), D.download(xp)) < 1e-8


def test_two_level_mode_needs_coarse_space():
    m = meshes.jittered_square(4, 1)
    D = dg.Discretization(m, "laplace", 2, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    with pytest.raises(dg.DgcError):
        D.pcg(poisson_rhs(D), mode=dg.SOLVE_TWO_LEVEL)


def test_coarse_space_refusals():
    m = meshes.jittered_square(4, 1)
    D32 = dg.Discretization(m, "laplace", 2, dg.F32, tau=dg.TAU_SCALED, dirichlet=True)
    with pytest.raises(dg.DgcError):
        D32.coarse_build(4)
    Dm = dg.Discretization(m, "laplace", 2, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    Dm.set_bc_types((Dm.boundary_nodes()[:, 0] > 0).astype(np.uint8))
    with pytest.raises(dg.DgcError):
        Dm.coarse_build(4)                              # per-node boundary types
    D = dg.Discretization(m, "laplace", 2, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    with pytest.raises(dg.DgcError):
        D.coarse_apply(D.upload(np.ones(D.K * D.Np)))   # not built
    D.coarse_build(4)
    D.set_shift(3.0)
    with pytest.raises(dg.DgcError):
        D.coarse_apply(D.upload(np.ones(D.K * D.Np)))   # built for shift 0


@pytest.mark.parametrize("prec", [dg.F64, dg.F32])
@pytest.mark.parametrize("N", [1, 2, 3, 4, 5, 8])
def test_spd_apply_writes_zero_padding(N, prec):
    """Solvers sum whole vectors: S u must leave 0, not stale memory, in the
    padded node slots of its output (orders where NpP > Np)."""
    m = meshes.jittered_square(5, 1)
    D = dg.Discretization(m, "laplace", N, prec, tau=dg.TAU_SCALED, dirichlet=True)
    assert D.NpP > D.Np
    u = D.upload(np.random.default_rng(N).standard_normal(D.K * D.Np))
    out = torch.full((D.state_len,), float("nan"), dtype=D.torch_dtype, device="cuda")
    D.spd(u, out=out)
    pad = out.view(D.K, D.NpP)[:, D.Np:]
    assert torch.all(pad == 0)
    assert torch.isfinite(out).all()
