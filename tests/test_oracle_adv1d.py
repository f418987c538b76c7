"""Pin the 1D advection oracle (oracle.Oracle1D) against the reference's own
examples/advection_1d/advection_1d.h (tests/golden/ref_adv1d_*.npz): operators
to 1e-13, RHS and RK4 states to 1e-12 relative, and the driver's error norm
after 10000 steps."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, oracle

CASES = sorted(glob.glob(os.path.join(GOLDEN, "ref_adv1d_K*_N*.npz")))


def relerr(a, b):
    a, b = np.ravel(a), np.ravel(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def kn(path):
    name = os.path.basename(path)[10:-4]          # K<K>_N<N>
    k, n = name.split("_")
    return int(k[1:]), int(n[1:])


def test_cases_exist():
    assert len(CASES) >= 7


@pytest.mark.parametrize("path", CASES, ids=lambda p: os.path.basename(p)[4:-4])
def test_oracle_matches_reference_1d(path):
    d = np.load(path)
    K, N = kn(path)
    o = oracle.Oracle1D(K, N)
    D, L = o.operators()
    assert relerr(D, d["D"]) < 1e-13 and relerr(L, d["L"]) < 1e-13
    assert relerr(o.node_x(), d["x"]) < 1e-15
    assert relerr(o.exact(0.0), d["u0"]) < 1e-15
    assert relerr(o.rhs(d["u0"], 0.1), d["rhs"]) < 1e-12
    dt = float(d["dt"][0])
    assert relerr(o.rk4(d["u0"], 0.0, dt, 1), d["rk4_1"]) < 1e-12
    steps = int(d["steps"][0])
    if steps == 10:
        assert relerr(o.rk4(d["u0"], 0.0, dt, 10), d["rk4_10"]) < 1e-12
    else:   # the driver's run: error norm (mean square nodal error) at its final time
        u = o.rk4(d["u0"], 0.0, dt, steps)
        t = steps * dt
        assert abs(t - float(d["t_final"][0])) < 1e-12
        mse = float(np.mean((o.exact(float(d["t_final"][0])) - u) ** 2))
        assert relerr(u, d["rk4_final"]) < 1e-10
        assert abs(mse - float(d["error_norm"][0])) <= 1e-6 * float(d["error_norm"][0])
