"""GPU parity of the 1D advection example (dgc_adv1d_*) through the C ABI:
operators, RHS and RK4 states against the reference's own advection_1d
(tests/golden/ref_adv1d_*.npz) at 1e-12 in FP64, including the driver's
10000-step error norm; orders 7-8 and FP32 against the oracle."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import dgc_gb300 as dg  # noqa: E402

CASES = sorted(glob.glob(os.path.join(GOLDEN, "ref_adv1d_K*_N*.npz")))


@pytest.fixture(scope="module", autouse=True)
def built():
    from dgc_gb300 import build
    build.build()


def relerr(a, b):
    a, b = np.ravel(a), np.ravel(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def kn(path):
    k, n = os.path.basename(path)[10:-4].split("_")
    return int(k[1:]), int(n[1:])


def run(A, u0, dt, steps):
    q = A.upload(u0)
    work = [A.empty_state() for _ in range(3)]
    t = 0.0
    for _ in range(steps):
        A.rk4_step(q, t, dt, work)
        t += dt
    return q.double().cpu().numpy(), t


@pytest.mark.parametrize("path", CASES, ids=lambda p: os.path.basename(p)[4:-4])
def test_matches_reference(path):
    d = np.load(path)
    K, N = kn(path)
    A = dg.Advection1D(K, N, dg.F64)
    assert relerr(A.operator(0), d["D"]) < 1e-13 and relerr(A.operator(1), d["L"]) < 1e-13
    assert relerr(A.node_x(), d["x"]) < 1e-15
    assert relerr(A.rhs(A.upload(d["u0"]), 0.1).cpu().numpy(), d["rhs"]) < 1e-12
    dt = float(d["dt"][0])
    assert relerr(run(A, d["u0"], dt, 1)[0], d["rk4_1"]) < 1e-12
    steps = int(d["steps"][0])
    u, t = run(A, d["u0"], dt, steps)
    if steps == 10:
        assert relerr(u, d["rk4_10"]) < 1e-12
    else:   # the driver's run: state and mean-square error at its final time
        assert relerr(u, d["rk4_final"]) < 1e-10
        o = oracle.Oracle1D(K, N)
        mse = float(np.mean((o.exact(float(d["t_final"][0])) - u) ** 2))
        # this error is round-off (~1e-26): the same order, not the same bits
        assert mse <= 10.0 * float(d["error_norm"][0]) + 1e-28
    assert A.launch_count() == 1 + 4 * (1 + steps)


@pytest.mark.parametrize("N", [7, 8])
def test_high_orders_match_oracle(N):
    K = 40
    o = oracle.Oracle1D(K, N)
    A = dg.Advection1D(K, N, dg.F64)
    D, L = o.operators()
    assert relerr(A.operator(0), D) < 1e-13 and relerr(A.operator(1), L) < 1e-13
    u0 = o.exact(0.0)
    dt = 0.25 / N / N * A.min_elem_size / A.wave_speed
    assert relerr(run(A, u0, dt, 10)[0], o.rk4(u0, 0.0, dt, 10)) < 1e-12


@pytest.mark.parametrize("N", range(1, 9))
def test_fp32_matches_oracle(N):
    K = 64
    o = oracle.Oracle1D(K, N)
    A = dg.Advection1D(K, N, dg.F32)
    u0 = o.exact(0.0)
    dt = 0.25 / N / N * A.min_elem_size / A.wave_speed
    assert relerr(run(A, u0, dt, 10)[0], o.rk4(u0, 0.0, dt, 10)) < 2e-5


def test_bad_arguments():
    with pytest.raises(dg.DgcError):
        dg.Advection1D(0, 3)
    with pytest.raises(dg.DgcError):
        dg.Advection1D(8, 9)
