"""Tile-shape variants of the fused RHS kernel and the autotuner.

Every compiled variant computes the same operator (parity with the oracle at
the FP32 tolerance); the autotuner picks one of them, and a cached choice is
reused without timing."""
import numpy as np
import pytest

from conftest import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import dgc_gb300 as dg  # noqa: E402
from dgc_gb300 import meshes  # noqa: E402

TOL32 = 2e-5


def relerr(a, b):
    a, b = np.ravel(a), np.ravel(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module", autouse=True)
def built():
    from dgc_gb300 import build
    build.build()


@pytest.mark.parametrize("N", range(1, 9))
@pytest.mark.parametrize("phys,kind", [("maxwell_te", oracle.MAXWELL_TE), ("advection", oracle.ADVECTION)])
def test_every_variant_matches_oracle(N, phys, kind):
    m = meshes.jittered_square(9, 60 + N)   # K = 162: several tiles, ragged last tile
    kw = dict(ax=1.0, ay=0.5, bc=dg.BC_GAUSS) if kind == oracle.ADVECTION else {}
    D = dg.Discretization(m, phys, N, dg.F32, **kw)
    o = oracle.Oracle(m.xy, m.cells, N)
    p = oracle.problem(kind, kw.get("ax", 1.0), kw.get("ay", 1.0), kw.get("bc", 0))
    q0 = o.exact(p, 0.07)
    ref = o.rhs(p, 0.07, q0)
    nv = D.num_variants()
    assert nv == (10 if N <= 6 else 4)
    q = D.upload(q0)
    for v in range(nv):
        D.set_variant(v)
        assert relerr(D.download(D.rhs(q, 0.07)), ref) < TOL32, v
        dt = 0.3 * D.info.min_edge / (N + 1) ** 2
        qb, res = D.empty_state(), D.empty_state()
        D.lserk4_step(q.clone(), qb, res, 0.07, dt)
        qo, _ = o.lserk4_step(p, 0.07, dt, q0, np.zeros_like(q0))
        assert relerr(D.download(qb), qo) < TOL32, v
    D.check()


def test_autotune_selects_and_caches(tmp_path, monkeypatch):
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("DGC_TUNE_CACHE", str(cache))
    m = meshes.jittered_square(24, 1)
    D = dg.Discretization(m, "maxwell_te", 6, dg.F32)
    chosen, times = D.autotune(reps=5)
    assert 0 <= chosen < D.num_variants()
    assert len(times) == D.num_variants() and all(t > 0 for t in times)
    assert times[chosen] == min(times)
    txt = cache.read_text().strip().split()
    assert txt[-1] == str(chosen)
    D2 = dg.Discretization(m, "maxwell_te", 6, dg.F32)
    c2, t2 = D2.autotune(measure=False)
    assert c2 == chosen and t2 is None
    assert D2.info.rhs_tile == D.info.rhs_tile


@pytest.mark.parametrize("prec", [dg.F32, dg.F64])
def test_variants_repeatable_at_scale(prec):
    """K = 32768, N = 6: every variant gives bitwise-repeatable RHS values over
    many launches (persistent CTAs over several tiles each) and no barrier
    wait expires."""
    m = meshes.jittered_square(128, 5)
    D = dg.Discretization(m, "maxwell_te", 6, prec)
    o = oracle.Oracle(m.xy, m.cells, 6)
    q = D.upload(o.exact(oracle.problem(oracle.MAXWELL_TE, 1.0, 1.0, 0), 0.1))
    for v in range(D.num_variants()):
        D.set_variant(v)
        ref = D.rhs(q, 0.1).clone()
        out = D.empty_state()
        for _ in range(40):
            D.rhs(q, 0.1, out=out)
            assert torch.equal(out, ref), v
        D.check()


def test_graphed_run_follows_variant_change():
    """A graphed dgc_lserk4_run, a variant change, and a second graphed run on
    the same buffers and dt: the second run replays the new variant (bitwise
    equal to its launch-by-launch run), not the graph of the first."""
    m = meshes.jittered_square(16, 7)
    D = dg.Discretization(m, "maxwell_te", 5, dg.F32)
    o = oracle.Oracle(m.xy, m.cells, 5)
    q0 = o.exact(oracle.problem(oracle.MAXWELL_TE, 1.0, 1.0, 0), 0.0)
    dt = 0.3 * D.info.min_edge / 36.0
    qa, qb, res = D.empty_state(), D.empty_state(), D.empty_state()
    out = {}
    for v in (0, 5, 0):
        D.set_variant(v)
        for graph in (True, False):
            qa.copy_(D.upload(q0))
            res.zero_()
            fin = D.lserk4_run(qa, qb, res, 0.0, dt, 20, graph=graph)
            out[(v, graph)] = fin.clone()
        assert torch.equal(out[(v, True)], out[(v, False)]), v
    D.check()
