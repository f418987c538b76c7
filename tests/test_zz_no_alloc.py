"""dgc_rk4_step_static: the RK4 step for callers that cannot allocate device
memory (global-mode graph capture, allocator-free real-time loops, plugins
whose memory belongs to the host application).  Called through the C ABI and
compared, on two calls in a row, with dgc_rk4_step given explicit work
vectors; sizes beyond the 2 MiB per-vector limit are rejected.

This file is collected last on purpose (a failure here leaves every other test
already run), and passes both alone in a fresh process and after the rest."""
import ctypes as C

import numpy as np
import pytest

from conftest import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import dgc_gb300 as dg  # noqa: E402
from dgc_gb300 import meshes  # noqa: E402

TOL = 1e-13  # same kernels and operation order as dgc_rk4_step


@pytest.fixture(scope="module")
def L():
    from dgc_gb300 import build
    build.build()
    L = dg.lib()
    L.dgc_rk4_step_static.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_void_p]
    return L


def relerr(a, b):
    a, b = np.ravel(a), np.ravel(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("phys,kind,prec", [("advection", oracle.ADVECTION, dg.F64),
                                            ("maxwell_te", oracle.MAXWELL_TE, dg.F32)])
def test_static_rk4_matches_rk4_with_work(L, phys, kind, prec):
    m = meshes.jittered_square(8, 12)
    D = dg.Discretization(m, phys, 4, prec, ax=1.0, ay=0.5, bc=dg.BC_GAUSS)
    o = oracle.Oracle(m.xy, m.cells, 4)
    p = oracle.problem(kind, 1.0, 0.5, oracle.BC_GAUSS)
    q0 = o.exact(p, 0.0)
    qs = D.upload(q0)
    qw = D.upload(q0)
    work = [D.empty_state() for _ in range(3)]
    dt = 0.4 * D.info.min_edge / 25.0
    stream = torch.cuda.current_stream().cuda_stream
    t = 0.0
    for _ in range(2):
        rc = L.dgc_rk4_step_static(D._h, qs.data_ptr(), t, dt, stream)
        assert rc == 0, L.dgc_last_error().decode()
        D.rk4_step(qw, t, dt, work)
        t += dt
        torch.cuda.synchronize()
        assert relerr(D.download(qs), D.download(qw)) <= TOL
    D.check()


def test_static_rk4_rejects_oversized_state(L):
    m = meshes.jittered_square(40, 1)            # K = 3200, N = 6, 3 fields, FP64: 2.15 MB
    D = dg.Discretization(m, "maxwell_te", 6, dg.F64)
    assert D.state_len * 8 > 2 * 1024 * 1024
    q = D.empty_state()
    rc = L.dgc_rk4_step_static(D._h, q.data_ptr(), 0.0, 1e-4, torch.cuda.current_stream().cuda_stream)
    assert rc == -1
    assert "2 MiB" in L.dgc_last_error().decode()
