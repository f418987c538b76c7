"""Batched persistent launches (dgc_batch_*): many independent FP32 advection /
Maxwell problems with mixed orders and mesh sizes, one launch per LSERK4
stage.  A batched step runs the tile code of each handle's variant (variant 0,
or the register-blocked one-element-per-thread variant: 5 at orders 1..6, 1
at orders 7, 8), so results must be bitwise equal to per-instance
dgc_lserk4_step with that variant, and the per-instance results agree with the
oracle at the FP32 tolerance."""
import numpy as np
import pytest

from conftest import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import dgc_gb300 as dg  # noqa: E402
from dgc_gb300 import meshes  # noqa: E402

TOL32 = 2e-5

# (physics, oracle kind, order, squares per side, seed)
CASES = [("advection", oracle.ADVECTION, 2, 5, 11), ("maxwell_te", oracle.MAXWELL_TE, 6, 9, 12),
         ("maxwell_tm", oracle.MAXWELL_TM, 3, 4, 13), ("advection", oracle.ADVECTION, 8, 3, 14),
         ("maxwell_te", oracle.MAXWELL_TE, 1, 12, 15), ("maxwell_tm", oracle.MAXWELL_TM, 7, 6, 16),
         ("advection", oracle.ADVECTION, 5, 7, 17), ("maxwell_te", oracle.MAXWELL_TE, 4, 2, 18)]


@pytest.fixture(scope="module", autouse=True)
def built():
    from dgc_gb300 import build
    build.build()


def make(case):
    phys, kind, N, n, seed = case
    m = meshes.jittered_square(n, seed)
    kw = dict(ax=0.8, ay=-0.6, bc=dg.BC_GAUSS) if kind == oracle.ADVECTION else {}
    D = dg.Discretization(m, phys, N, dg.F32, **kw)
    o = oracle.Oracle(m.xy, m.cells, N)
    p = oracle.problem(kind, kw.get("ax", 1.0), kw.get("ay", 1.0), kw.get("bc", 0))
    dt = 0.3 * D.info.min_edge / (N + 1) ** 2
    return D, o, p, dt


def blk_variant(N):
    return 5 if N <= 6 else 1


@pytest.mark.parametrize("codes", ["v0", "blocked", "mixed"])
def test_batched_steps_equal_per_instance_steps(codes):
    insts = [make(c) for c in CASES]
    for i, (D, *_) in enumerate(insts):
        blocked = codes == "blocked" or (codes == "mixed" and i % 2 == 1)
        D.set_variant(blk_variant(D.N) if blocked else 0)
    t0 = [0.05 * i for i in range(len(insts))]
    q0 = [o.exact(p, t) for (D, o, p, dt), t in zip(insts, t0)]
    B = dg.Batch([D for D, _, _, _ in insts])
    dts = [dt for *_, dt in insts]
    # reference: per-instance steps with each handle's variant
    ref = []
    for (D, o, p, dt), q, t in zip(insts, q0, t0):
        a, b, r = D.upload(q), D.empty_state(), D.empty_state()
        for s in range(3):
            D.lserk4_step(a, b, r, t + s * dt, dt)
            a, b = b, a
        ref.append(a.clone())
    # batched: three single steps
    qa = [D.upload(q) for (D, *_), q in zip(insts, q0)]
    qb = [D.empty_state() for D, *_ in insts]
    rs = [D.empty_state() for D, *_ in insts]
    l0 = B.launch_count()
    for s in range(3):
        B.lserk4_step(qa, qb, rs, [t + s * dt for t, dt in zip(t0, dts)], dts)
        qa, qb = qb, qa
    torch.cuda.synchronize()
    assert B.launch_count() - l0 == 15
    for i, (a, r) in enumerate(zip(qa, ref)):
        assert torch.equal(a, r), CASES[i]
    # batched run, graph-replayed (odd step count: results in qb)
    qa = [D.upload(q) for (D, *_), q in zip(insts, q0)]
    qb = [D.empty_state() for D, *_ in insts]
    rs = [D.empty_state() for D, *_ in insts]
    fin = B.lserk4_run(qa, qb, rs, t0, dts, 3, graph=True)
    assert fin[0] is qb[0]
    for i, (a, r) in enumerate(zip(fin, ref)):
        assert torch.equal(a, r), CASES[i]
    for D, *_ in insts:
        D.check()
    # and the per-instance path agrees with the oracle
    for (D, o, p, dt), q, t, a in zip(insts, q0, t0, ref):
        qo, res = q, np.zeros_like(q)
        for s in range(3):
            qo, res = o.lserk4_step(p, t + s * dt, dt, qo, res)
        err = np.linalg.norm(D.download(a) - qo) / np.linalg.norm(qo)
        assert err < TOL32


def test_batch_rejects_unsupported_handles():
    m = meshes.jittered_square(3, 1)
    D64 = dg.Discretization(m, "maxwell_te", 3, dg.F64)
    with pytest.raises(dg.DgcError):
        dg.Batch([D64])
    L = dg.Discretization(m, "laplace", 3, dg.F32)
    with pytest.raises(dg.DgcError):
        dg.Batch([L])
