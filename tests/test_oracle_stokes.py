"""The Stokes example's pieces on the CPU: the boundary-data term of
laplace_2d and the dual-splitting step restated in oracle/stokes_oracle.py.

apply_inhomogeneous_as_rhs (src/laplace_2d.h:253-348) lifts the Dirichlet
data into q_d on the boundary cells but adds only its boundary-face terms; the
jumps of q_d across interior faces (which apply_homogeneous's second pass has
for the same lift) are missing.  With non-zero Dirichlet data the reference's
`operator()` is then not the affine operator of its scheme, and the Stokes
example (the one caller with such data) does not converge to its analytic
solution.  The oracle's bc_jump term restores them; these tests pin both
forms."""
import numpy as np
import pytest

from conftest import oracle  # noqa: F401  (puts oracle/ on sys.path)
import stokes_oracle as so
from dgc_gb300 import meshes

POLYS = [
    ("one", lambda x, y: 1.0 + 0 * x, lambda x, y: 0 * x, 1),
    ("quad", lambda x, y: x * y - x * x + 0.5 * y, lambda x, y: -2.0 + 0 * x, 2),
    ("cubic", lambda x, y: x * x * y + 0.3 * y ** 3, lambda x, y: 2.0 * y + 1.8 * y, 3),
]


def _setup(n, N, seed=2):
    m = meshes.jittered_square(n, seed)
    return m, so.StokesOracle(m.xy, m.cells, N)


@pytest.mark.parametrize("N", [1, 2, 3, 4])
def test_consistent_data_term_exact_on_polynomials(N):
    """laplace_apply(u) - bc_rhs(2 u|bdry) - bc_jump = lap u for deg u <= N
    (exterior_val = 2 g - interior, the Stokes example's velocity condition)."""
    _, s = _setup(4, N)
    x, y = (a.reshape(-1) for a in s.o.node_xy())
    bx, by = s.arr["bx"], s.arr["by"]
    for name, f, lap, deg in POLYS:
        if deg > N:
            continue
        u = f(x, y)
        d = s.o.laplace_bc_rhs(np.ones(s.nb, np.uint8), 2.0 * f(bx, by), None, consistent=True)
        F = s.A_D @ u - d
        assert np.abs(F - lap(x, y)).max() < 1e-9 * max(1.0, np.abs(s.A_D @ u).max()), name


def test_reference_data_term_misses_interior_jumps():
    """For u = 1, g = 1 the reference's operator() leaves a residual, and only
    on boundary cells and their face neighbours."""
    _, s = _setup(6, 2)
    K, Np = s.K, s.Np
    u = np.ones(K * Np)
    d_ref = s.o.laplace_bc_rhs(np.ones(s.nb, np.uint8), 2.0 * np.ones(s.nb), None)
    d_con = s.o.laplace_bc_rhs(np.ones(s.nb, np.uint8), 2.0 * np.ones(s.nb), None, consistent=True)
    r_ref = (s.A_D @ u - d_ref).reshape(K, Np)
    r_con = (s.A_D @ u - d_con).reshape(K, Np)
    assert np.abs(r_con).max() < 1e-9
    nc = s.arr["nbCell"].reshape(K, 3)
    isb = np.array([any(nc[c, f] == c for f in range(3)) for c in range(K)])
    near = isb | np.array([any(isb[nc[c, f]] for f in range(3)) for c in range(K)])
    assert np.abs(r_ref).max() > 10.0
    assert np.abs(r_ref[~near]).max() < 1e-9


def test_jump_term_zero_without_dirichlet_data():
    _, s = _setup(3, 3)
    h = np.linspace(-1, 1, s.nb)
    a = s.o.laplace_bc_rhs(np.zeros(s.nb, np.uint8), None, h)
    b = s.o.laplace_bc_rhs(np.zeros(s.nb, np.uint8), None, h, consistent=True)
    assert np.array_equal(a, b)


def test_hp_matches_analytic_curl_free_case():
    """hp = dgdt.n + (curl curl term).n: for u^n = u^(n-1) = a gradient field
    (curl 0) the curl-curl term vanishes and hp = dgdt.n exactly."""
    _, s = _setup(3, 3)
    x, y = (a.reshape(-1) for a in s.o.node_xy())
    ux, uy = 2 * x * y, x * x - y * y  # grad(x^2 y - y^3/3)
    ddx = np.linspace(0, 1, s.nb)
    ddy = np.linspace(1, 2, s.nb)
    hp = s.hp(ux, uy, ux, uy, ddx, ddy)
    nxb, nyb = [], []
    nx, ny = s.arr["nx"].reshape(s.K, 3), s.arr["ny"].reshape(s.K, 3)
    for c in range(s.K):
        for f in range(3):
            if s._is_boundary(c, f):
                nxb += [nx[c, f]] * s.Nfp
                nyb += [ny[c, f]] * s.Nfp
    assert np.abs(hp - (ddx * np.array(nxb) + ddy * np.array(nyb))).max() < 1e-10


def test_step_convergence_consistent_only():
    """The dual-splitting step (stokes_2d.h:393-423) reaches the example's
    analytic solution with the consistent data term, not with the reference's."""
    m = meshes.jittered_square(4, 1)
    errs = {}
    for cons in (False, True):
        s = so.StokesOracle(m.xy, m.cells, 3, consistent=cons)
        _, _, t, err = s.run(T=0.01, dt=0.001)
        assert abs(t - 0.01) < 1e-12
        errs[cons] = err
    assert errs[True] < 1e-4
    assert errs[False] > 1e-2


def test_step_error_decreases_with_order():
    m = meshes.jittered_square(4, 1)
    e = [so.StokesOracle(m.xy, m.cells, N, consistent=True).run(T=0.01, dt=0.001)[3] for N in (2, 3, 4)]
    assert e[0] > 10 * e[1] and e[1] > 2 * e[2]


# ------------------------------------------------------------------ reference goldens
# tests/golden/ref_stokes_jit4_N*.npz: the reference's stokes_2d probed up to its
# linear solves (oracle/ref_harness/ref_stokes.cpp), solved densely (make_golden.py)
import os  # noqa: E402

from conftest import GOLDEN  # noqa: E402

STOKES_CASES = [2, 3, 4]


def _golden(N):
    d = np.load(os.path.join(GOLDEN, f"ref_stokes_jit4_N{N}.npz"))
    s = so.StokesOracle(d["mesh_xy"].reshape(-1, 2), d["mesh_cells"].reshape(-1, 3), N)
    return d, s


def _rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300)


@pytest.mark.parametrize("N", STOKES_CASES)
def test_stokes_pieces_match_reference(N):
    """hp, the pressure right-hand side, grad p, the projected u~ and the viscous
    right-hand sides of the oracle equal the reference's at 1e-12."""
    d, s = _golden(N)
    x, y = (a.reshape(-1) for a in s.o.node_xy())
    assert _rel(x, d["x"]) < 1e-15 and _rel(y, d["y"]) < 1e-15
    assert _rel(s.arr["bx"], d["bx"]) < 1e-15 and _rel(s.arr["by"], d["by"]) < 1e-15
    dt = float(d["dt"][0])
    for k in range(2):
        g = {key[3:]: d[key] for key in d.files if key.startswith(f"s{k}_")}
        t_prev, t = float(g["t_prev"][0]), float(g["t"][0])
        bc = so.boundary_data(s.arr["bx"], s.arr["by"], t, t_prev, dt)
        assert _rel((4 * g["u1x"] - g["u0x"]) / 3, g["ut_x"]) < 1e-15
        hp = s.hp(g["u0x"], g["u0y"], g["u1x"], g["u1y"], bc["dgdt_x"], bc["dgdt_y"])
        assert _rel(2 * hp, g["hp2"]) < 1e-12
        w = s.o.div(g["ut_x"], g["ut_y"], bc["ut_x"], bc["ut_y"], -1.0) * (1.5 / dt)
        assert _rel(w, g["div_ut"]) < 1e-12
        w = s.o.laplace_bc_rhs(np.zeros(s.nb, np.uint8), None, g["hp2"], out=w)
        assert _rel(w, g["p_rhs"]) < 1e-12
        gx, gy = s.o.grad(g["p"], None, 1.0)
        assert _rel(gx, g["grad_p_x"]) < 1e-12 and _rel(gy, g["grad_p_y"]) < 1e-12
        assert _rel(g["ut_x"] - 2 * dt * gx / 3, g["utp_x"]) < 1e-12
        for c, gd in (("x", bc["g_x"]), ("y", bc["g_y"])):
            v = s.o.laplace_bc_rhs(np.ones(s.nb, np.uint8), gd, None, out=-1.5 * g[f"utp_{c}"] / dt)
            assert _rel(v, g[f"v_rhs_{c}"]) < 1e-12


@pytest.mark.parametrize("N", STOKES_CASES)
def test_stokes_step_matches_reference(N):
    """The whole restated step from the reference's inputs: velocity at 1e-10,
    pressure (same null-space convention) at 1e-9."""
    d, s = _golden(N)
    dt = float(d["dt"][0])
    for k in range(2):
        g = {key[3:]: d[key] for key in d.files if key.startswith(f"s{k}_")}
        bc = so.boundary_data(s.arr["bx"], s.arr["by"], float(g["t"][0]), float(g["t_prev"][0]), dt)
        ux, uy, p = s.step(g["u0x"], g["u0y"], g["u1x"], g["u1y"], dt, bc)
        assert _rel(ux, g["ux"]) < 1e-10 and _rel(uy, g["uy"]) < 1e-10, k
        assert _rel(p, g["p"]) < 1e-9, k


def test_product_example_data_matches_oracle():
    """The Stokes example's boundary data and exact velocity are written twice,
    in the product module and in the oracle: they must agree."""
    from dgc_gb300 import stokes as st
    rng = np.random.default_rng(3)
    x, y = rng.uniform(-1, 1, 50), rng.uniform(-1, 1, 50)
    for t, tp, dt in ((0.0, 0.0, 1e-3), (0.02, 0.019, 1e-3), (0.5, 0.49, 0.01)):
        a = st.example_boundary_data(x, y, t, tp, dt)
        b = so.boundary_data(x, y, t, tp, dt)
        assert a.keys() == b.keys()
        for k in a:
            assert np.array_equal(a[k], b[k]), k
        for u, v in zip(st.exact_velocity(x, y, t), so.exact(x, y, t)):
            assert np.array_equal(u, v)
