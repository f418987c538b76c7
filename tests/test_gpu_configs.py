"""Parity at the benchmark workloads' own sizes, through the C ABI.

* Advection, jittered 32x32 mesh (K = 2048), N = 4, a = (1, 0.5), Gaussian
  pulse exp(-((x+0.3)^2 + y^2)/0.02), exact inflow, LSERK4 with
  dt = 0.5 min(h) / ((N+1)^2 |a|) to T = 0.5: every step against the oracle at
  1e-12 (FP64), and the L2 error against the exact translated pulse equal to
  the oracle's (examples/advection_2d/advection_2d.h:132-154 is the reference's
  exact solution for its own velocity).
* Maxwell TE cavity, jittered 128x128 mesh (K = 32768), N = 6: three LSERK4
  steps against the oracle, FP64 per step at 1e-12, FP32 at 2e-5 with the
  autotuned stage kernel and with the tensor-core pipeline (variant 9).
* IPDG Poisson, jittered 256x256 mesh (K = 131072), N = 4, tau = (N+1)^2/h:
  the mixed-precision solution's residual recomputed on the CPU with the
  oracle's operator (FP64) is at the solver's 1e-10, and it agrees with the
  FP64 PCG solution and with sin(pi x) sin(pi y) to the same tolerance.
"""
import numpy as np
import pytest

from conftest import oracle

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


def test_advection_k2048_n4_to_t05_every_step():
    N, T = 4, 0.5
    ax, ay = 1.0, 0.5
    m = meshes.jittered_square(32, 2026)
    D = dg.Discretization(m, "advection", N, dg.F64, ax=ax, ay=ay, bc=dg.BC_GAUSS)
    assert D.K == 2048
    o = oracle.Oracle(m.xy, m.cells, N)
    p = oracle.problem(oracle.ADVECTION, ax, ay, oracle.BC_GAUSS)
    dt0 = 0.5 * D.info.min_edge / ((N + 1) ** 2 * np.hypot(ax, ay))
    nsteps = int(np.ceil(T / dt0))
    dt = T / nsteps
    q = o.exact(p, 0.0)
    res = np.zeros_like(q)
    a, b, r = D.upload(q), D.empty_state(), D.empty_state()
    worst = 0.0
    for n in range(nsteps):
        t = n * dt
        q, res = o.lserk4_step(p, t, dt, q, res)
        D.lserk4_step(a, b, r, t, dt)
        a, b = b, a
        e = relerr(D.download(a), q)
        worst = max(worst, e)
        assert e < TOL64, (n, e)
    D.check()
    ex = o.exact(p, T)
    err_gpu = relerr(D.download(a), ex)
    err_orc = relerr(q, ex)
    assert abs(err_gpu - err_orc) <= 1e-9 * err_orc, (err_gpu, err_orc)
    # the discretisation error of this workload: a resolved pulse at N = 4
    assert err_orc < 1e-2
    print(f"advection K=2048 N=4: {nsteps} steps, worst per-step {worst:.2e}, L2 error {err_orc:.4e}")


@pytest.fixture(scope="module")
def cavity():
    N = 6
    m = meshes.jittered_square(128, 2026)
    o = oracle.Oracle(m.xy, m.cells, N)
    p = oracle.problem(oracle.MAXWELL_TE)
    D64 = dg.Discretization(m, "maxwell_te", N, dg.F64)
    assert D64.K == 32768
    dt = 0.5 * D64.info.min_edge / (N + 1) ** 2
    q = o.exact(p, 0.0)
    res = np.zeros_like(q)
    states = [q]
    for n in range(3):
        q, res = o.lserk4_step(p, n * dt, dt, q, res)
        states.append(q)
    return m, N, dt, D64, states


def _run_steps(D, states, dt, tol):
    a, b, r = D.upload(states[0]), D.empty_state(), D.empty_state()
    errs = []
    for n in range(3):
        D.lserk4_step(a, b, r, n * dt, dt)
        a, b = b, a
        errs.append(relerr(D.download(a), states[n + 1]))
        assert errs[-1] < tol, (n, errs)
    D.check()
    return errs


def test_maxwell_te_k32768_n6_fp64_steps(cavity):
    m, N, dt, D64, states = cavity
    _run_steps(D64, states, dt, TOL64)


@pytest.mark.parametrize("variant", ["autotuned", 9])
def test_maxwell_te_k32768_n6_fp32_steps(cavity, variant):
    m, N, dt, _, states = cavity
    D = dg.Discretization(m, "maxwell_te", N, dg.F32)
    if variant == "autotuned":
        D.autotune(reps=5)
    else:
        D.set_variant(variant)
    _run_steps(D, states, dt, TOL32)


def test_poisson_k131072_n4_mixed_solution_residual_on_cpu():
    N = 4
    m = meshes.jittered_square(256, 4242)
    D = dg.Discretization(m, "laplace", N, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    assert D.K == 131072
    o = oracle.Oracle(m.xy, m.cells, N)
    x, y = D.node_xy()
    f = 2 * np.pi ** 2 * np.sin(np.pi * x) * np.sin(np.pi * y)
    b = D.mass(D.upload(f.reshape(-1)))
    sol = {}
    for mode in (dg.SOLVE_MIXED_IR, dg.SOLVE_FP64_PCG):
        xs, st = D.pcg(b, mode=mode, rtol=1e-10, maxit=40000)
        assert st["converged"] and st["final_relres"] <= 1e-10
        sol[mode] = D.download(xs).reshape(-1)
    D.check()
    # residual with the oracle's own FP64 operator (reference CPU layout)
    bo = o.mass(f.reshape(-1))
    r = bo - o.spd(sol[dg.SOLVE_MIXED_IR], tau_mode=1)
    assert np.linalg.norm(r) <= 2e-10 * np.linalg.norm(bo)
    ex = (np.sin(np.pi * x) * np.sin(np.pi * y)).reshape(-1)
    # at this resolution the discretisation error (~1e-12) is below the solves'
    # algebraic error, so both solutions sit within the 1e-10 tolerance of the
    # exact solution and of each other
    e_mixed, e_fp64 = relerr(sol[dg.SOLVE_MIXED_IR], ex), relerr(sol[dg.SOLVE_FP64_PCG], ex)
    assert e_mixed < 1e-10 and e_fp64 < 1e-10, (e_mixed, e_fp64)
    assert relerr(sol[dg.SOLVE_MIXED_IR], sol[dg.SOLVE_FP64_PCG]) < 1e-10
