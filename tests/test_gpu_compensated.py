"""The compensated FP32 state (DGC_F32C): FP32 arithmetic, the state carried as
hi + lo FP32 pairs, strong-form stage kernel with jump-based surface terms.

* operator values against the oracle (FP64) at every order and physics,
  within FP32 round-off (2e-5, as for DGC_F32);
* one LSERK4 step against the oracle's step at 5e-7 relative: the update is
  compensated, so only dt times the operator's FP32 round-off remains;
* a TE cavity run to T = 1 (jittered 32x32, N = 6) lands within 1e-6 of the
  FP64 run and of the exact mode, where the plain FP32 state stops near 5e-6;
* reference-layout round trips keep FP64 values to 2^-47; graph replay is
  bitwise equal to the launch-by-launch run; the operations that are not
  offered for these handles say so.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import dgc_gb300 as dg  # noqa: E402
from dgc_gb300 import meshes  # noqa: E402

PHYS = [("advection", oracle.ADVECTION), ("maxwell_tm", oracle.MAXWELL_TM), ("maxwell_te", oracle.MAXWELL_TE)]


def relerr(a, b):
    a, b = np.ravel(a), np.ravel(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module", autouse=True)
def built():
    from dgc_gb300 import build
    build.build()


def make(m, phys, kind, N, prec):
    kw = dict(ax=1.0, ay=0.5, bc=dg.BC_GAUSS) if kind == oracle.ADVECTION else {}
    D = dg.Discretization(m, phys, N, prec, **kw)
    p = oracle.problem(kind, kw.get("ax", 1.0), kw.get("ay", 1.0), kw.get("bc", 0))
    return D, p


@pytest.mark.parametrize("N", range(1, 9))
@pytest.mark.parametrize("phys,kind", PHYS)
def test_rhs_and_step_match_oracle(N, phys, kind):
    m = meshes.jittered_square(9, 80 + N)   # K = 162: several tiles, ragged last tile
    D, p = make(m, phys, kind, N, dg.F32C)
    o = oracle.Oracle(m.xy, m.cells, N)
    assert D.num_variants() == 1
    q0 = o.exact(p, 0.07)
    q = D.upload(q0)
    assert relerr(D.download(q), q0) < 2.0 ** -47
    ref = o.rhs(p, 0.07, q0)
    assert relerr(D.download(D.rhs(q, 0.07)), ref) < 2e-5
    dt = 0.3 * D.info.min_edge / (N + 1) ** 2
    qb, res = D.empty_state(), D.empty_state()
    D.lserk4_step(q.clone(), qb, res, 0.07, dt)
    qo, ro = o.lserk4_step(p, 0.07, dt, q0, np.zeros_like(q0))
    assert relerr(D.download(qb), qo) < 5e-7
    D.check()


def test_cavity_run_to_t1_reaches_fp64_accuracy():
    N, T = 6, 1.0
    m = meshes.jittered_square(32, 2026)
    o = oracle.Oracle(m.xy, m.cells, N)
    p = oracle.problem(oracle.MAXWELL_TE)
    q0 = o.exact(p, 0.0)
    ex = o.exact(p, T)
    out = {}
    for prec in (dg.F64, dg.F32, dg.F32C):
        D = dg.Discretization(m, "maxwell_te", N, prec)
        dt0 = 0.5 * D.info.min_edge / (N + 1) ** 2
        ns = int(np.ceil(T / dt0))
        fin = D.lserk4_run(D.upload(q0), D.empty_state(), D.empty_state(), 0.0, T / ns, ns, graph=True)
        out[prec] = D.download(fin)
        D.check()
    e64, e32, e32c = (relerr(out[k], ex) for k in (dg.F64, dg.F32, dg.F32C))
    d32c = relerr(out[dg.F32C], out[dg.F64])
    print(f"T=1 errors vs exact: fp64 {e64:.3e}  fp32 {e32:.3e}  fp32c {e32c:.3e} (vs fp64 {d32c:.3e})")
    assert e64 < 1e-9
    assert d32c < 1e-6 and e32c < 1e-6
    assert e32c < 0.25 * e32


def test_graph_replay_is_bitwise_and_layouts_round_trip():
    m = meshes.jittered_square(12, 3)
    D, p = make(m, "maxwell_tm", oracle.MAXWELL_TM, 5, dg.F32C)
    o = oracle.Oracle(m.xy, m.cells, 5)
    q0 = o.exact(p, 0.2)
    dt = 0.3 * D.info.min_edge / 36.0
    res = {}
    for graph in (True, False):
        qa, qb, r = D.upload(q0), D.empty_state(), D.empty_state()
        res[graph] = D.lserk4_run(qa, qb, r, 0.2, dt, 24, graph=graph).clone()
    assert torch.equal(res[True], res[False])
    for layout in (dg.LAYOUT_REF_CPU, dg.LAYOUT_REF_GPU):
        src = torch.from_numpy(np.random.default_rng(layout).standard_normal(q0.size)).cuda()
        back = D.from_native(D.to_native(src, layout), layout)
        assert relerr(back.cpu().numpy(), src.cpu().numpy()) < 2.0 ** -47
    D.check()


def test_operations_not_offered_for_compensated_state():
    m = meshes.jittered_square(4, 1)
    D, _ = make(m, "advection", oracle.ADVECTION, 3, dg.F32C)
    q = D.empty_state()
    work = [D.empty_state() for _ in range(3)]
    with pytest.raises(dg.DgcError):
        D.rk4_step(q, 0.0, 1e-3, work)
    with pytest.raises(dg.DgcError):
        D.axpy(1.0, q, work[0], work[1])
    with pytest.raises(dg.DgcError):
        D.grad(q)
    with pytest.raises(dg.DgcError):
        dg.Batch([D])
    with pytest.raises(dg.DgcError):
        dg.Discretization(m, "laplace", 3, dg.F32C)
