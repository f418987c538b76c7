"""GPU parity of the Stokes example's pieces through the C ABI.

* dgc_laplace_bc_rhs in both boundary-data modes against the oracle (FP64 at
  1e-12 relative, FP32 at 2e-5), uniform and mixed condition types; the
  CONSISTENT mode exact on polynomials at 131072 elements (a size-independent
  property).
* dgc_stokes_step against the dense restatement of advance_timestep
  (oracle/stokes_oracle.py, direct solves), three steps from the example's
  initial data, both modes: velocity to 1e-9 relative (the GPU solves run to
  a 1e-11 relative residual), pressure to 1e-7.
* The example driver with the consistent data term reaches the analytic
  solution; with the reference's term it does not (as the oracle shows).
"""
import numpy as np
import pytest

from conftest import oracle  # noqa: F401

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import stokes_oracle as so  # noqa: E402
import dgc_gb300 as dg  # noqa: E402
from dgc_gb300 import meshes  # noqa: E402
from dgc_gb300 import stokes as st  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def built():
    from dgc_gb300 import build
    build.build()


def relerr(a, b):
    a, b = np.ravel(a), np.ravel(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("prec", [dg.F64, dg.F32])
@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("N", [1, 2, 3, 4, 6, 8])
def test_bc_rhs_modes_match_oracle(N, mixed, prec):
    m = meshes.jittered_square(5, 3)
    D = dg.Discretization(m, "laplace", N, prec, tau=dg.TAU_ONE)
    O = oracle.Oracle(m.xy, m.cells, N)
    b = D.boundary_nodes()
    nb = b.shape[0]
    flags = (b[:, 0] > 0.2).astype(np.uint8) if mixed else np.ones(nb, np.uint8)
    if mixed:
        D.set_bc_types(flags)
    g = np.sin(b[:, 0] + 2 * b[:, 1]) + 1.5
    h = np.cos(3 * b[:, 0]) - b[:, 1]
    for mode in (dg.BC_DATA_REFERENCE, dg.BC_DATA_CONSISTENT):
        D.set_bc_data_mode(mode)
        out = D.laplace_bc_rhs(g, h)
        ref = O.laplace_bc_rhs(flags, g, h, consistent=mode == dg.BC_DATA_CONSISTENT)
        assert relerr(D.download(out), ref) < (1e-12 if prec == dg.F64 else 2e-5), mode
    # the jump term accumulates into out like the rest
    base = D.upload(np.full(D.K * D.Np, 0.25))
    out = D.laplace_bc_rhs(g, h, out=base)
    ref = O.laplace_bc_rhs(flags, g, h, out=np.full(D.K * D.Np, 0.25), consistent=True)
    assert relerr(D.download(out), ref) < (1e-12 if prec == dg.F64 else 2e-5)


@pytest.mark.parametrize("N", [2, 4])
def test_consistent_operator_exact_at_scale(N):
    """laplace(u) - bc_rhs(consistent) = lap u for u = x y - x^2 + y/2 on 131072 cells."""
    m = meshes.jittered_square(256, 5)
    D = dg.Discretization(m, "laplace", N, dg.F64, tau=dg.TAU_ONE)
    D.set_bc_data_mode(dg.BC_DATA_CONSISTENT)
    x, y = (a.reshape(-1) for a in D.node_xy())
    b = D.boundary_nodes()
    f = lambda x, y: x * y - x * x + 0.5 * y  # noqa: E731
    u = D.upload(f(x, y))
    Au = D.laplace(u)
    r = D.download(Au) - D.download(D.laplace_bc_rhs(2.0 * f(b[:, 0], b[:, 1])))
    scale = np.abs(D.download(Au)).max()
    assert np.abs(r + 2.0).max() < 1e-9 * scale
    D.set_bc_data_mode(dg.BC_DATA_REFERENCE)
    r = D.download(Au) - D.download(D.laplace_bc_rhs(2.0 * f(b[:, 0], b[:, 1])))
    assert np.abs(r + 2.0).max() > 1.0


@pytest.mark.parametrize("mode", [dg.SOLVE_MIXED_IR, dg.SOLVE_TWO_LEVEL, dg.SOLVE_TWO_LEVEL_MIXED])
@pytest.mark.parametrize("consistent", [False, True])
@pytest.mark.parametrize("N", [2, 3])
def test_stokes_step_matches_dense_restatement(N, consistent, mode):
    m = meshes.jittered_square(4, 1)
    S = st.Stokes(m, N, consistent=consistent, rtol=1e-11, mode=mode)
    O = so.StokesOracle(m.xy, m.cells, N, consistent=consistent)
    vs = S.velocity_space
    x, y = (a.reshape(-1) for a in vs.node_xy())
    ox, oy = (a.reshape(-1) for a in O.o.node_xy())
    assert np.array_equal(x, ox) and np.array_equal(y, oy)
    bxy = vs.boundary_nodes()
    assert np.allclose(bxy[:, 0], O.arr["bx"], rtol=0, atol=0) and np.allclose(bxy[:, 1], O.arr["by"], rtol=0, atol=0)
    ux, uy = st.exact_velocity(x, y, 0.0)
    h = [ux.copy(), uy.copy(), ux.copy(), uy.copy()]  # u^(n-1), u^n on the host (oracle)
    d = [vs.upload(ux), vs.upload(uy), vs.upload(ux), vs.upload(uy)]
    p = S.empty()
    t_prev = t = 0.0
    dt = 0.002
    for k in range(3):
        bc = st.example_boundary_data(O.arr["bx"], O.arr["by"], t, t_prev, dt)
        hx, hy, hp = O.step(h[0], h[1], h[2], h[3], dt, bc)
        gx, gy, stats = S.step(d[0], d[1], d[2], d[3], dt, S.boundary_data(t, t_prev, dt), p_out=p)
        assert stats["converged"] == 1 and stats["final_relres"] <= 1e-11
        assert relerr(vs.download(gx), hx) < 1e-9, k
        assert relerr(vs.download(gy), hy) < 1e-9, k
        assert relerr(vs.download(p), hp) < 1e-7, k
        h = [h[2], h[3], hx, hy]
        d = [d[2], d[3], gx, gy]
        t_prev, t = t, t + dt


def test_stokes_outputs_may_alias_previous_state():
    m = meshes.jittered_square(3, 2)
    S = st.Stokes(m, 3, consistent=True)
    vs = S.velocity_space
    x, y = (a.reshape(-1) for a in vs.node_xy())
    ux, uy = st.exact_velocity(x, y, 0.0)
    bc = S.boundary_data(0.0, 0.0, 0.001)
    a = S.step(vs.upload(ux), vs.upload(uy), vs.upload(ux), vs.upload(uy), 0.001, bc)
    up = [vs.upload(ux), vs.upload(uy)]
    b = S.step(up[0], up[1], vs.upload(ux), vs.upload(uy), 0.001, bc, out=(up[0], up[1]))
    # the pressure solve warm-starts from the previous step's p: equal to the solver tolerance
    assert relerr(vs.download(a[0]), vs.download(b[0])) < 1e-9
    assert relerr(vs.download(a[1]), vs.download(b[1])) < 1e-9
    u = vs.upload(ux)
    with pytest.raises(dg.DgcError):
        S.step(up[0], up[1], u, vs.upload(uy), 0.001, bc, out=(u, up[1]))


def test_stokes_example_converges_with_consistent_data():
    """examples/stokes_2d/main.cpp's loop (u^(-1) = u^0, T, dt) on a small mesh."""
    m = meshes.jittered_square(6, 1)
    errs = {}
    for cons in (False, True):
        S = st.Stokes(m, 4, consistent=cons)
        _, _, t, err, iters = S.run_example(T=0.02, dt=0.001)
        assert abs(t - 0.02) < 1e-12 and iters > 0
        errs[cons] = err
    O = so.StokesOracle(m.xy, m.cells, 4, consistent=True)
    _, _, _, oerr = O.run(T=0.02, dt=0.001)
    assert errs[True] < 1e-5
    assert abs(errs[True] - oerr) < 1e-3 * oerr
    assert errs[False] > 1e-2


@pytest.mark.parametrize("N", [2, 3, 4])
def test_stokes_step_matches_reference_golden(N):
    """dgc_stokes_step from the reference's own step inputs (tests/golden/
    ref_stokes_jit4_N*.npz: stokes_2d probed up to its solves, solved densely):
    velocity at 1e-9, pressure at 1e-7, both steps."""
    import os
    from conftest import GOLDEN
    d = np.load(os.path.join(GOLDEN, f"ref_stokes_jit4_N{N}.npz"))
    m = meshes.Mesh(xy=d["mesh_xy"].reshape(-1, 2), cells=d["mesh_cells"].reshape(-1, 3))
    S = st.Stokes(m, N, rtol=1e-11)
    vs = S.velocity_space
    b = vs.boundary_nodes()
    assert np.array_equal(b[:, 0], d["bx"]) and np.array_equal(b[:, 1], d["by"])
    dt = float(d["dt"][0])
    p = S.empty()
    for k in range(2):
        g = {key[3:]: d[key] for key in d.files if key.startswith(f"s{k}_")}
        u = [vs.upload(g[c]) for c in ("u0x", "u0y", "u1x", "u1y")]
        ux, uy, stats = S.step(*u, dt, S.boundary_data(float(g["t"][0]), float(g["t_prev"][0]), dt), p_out=p)
        assert stats["converged"] == 1
        assert relerr(vs.download(ux), g["ux"]) < 1e-9, k
        assert relerr(vs.download(uy), g["uy"]) < 1e-9, k
        assert relerr(vs.download(p), g["p"]) < 1e-7, k
