"""Programmatic dependent launch changes timing only: the stage kernels and
the batch kernel give bit-identical results with the launch attribute on
(default) and off (DGC_STAGE_OVERLAP=0), and the solves through the FP32 CG
kernels agree to their tolerance (their FP64 atomic reductions are not
ordered, with or without the attribute).

The switch is read once per process, so each setting runs in its own child
process; the children write their results to .npz files that the test
compares.  Cases: 12 LSERK4 steps launch by launch and 20 from a
CUDA graph on a Maxwell TE cavity (jittered 16x16, N = 6) with the blocked
FP32 kernel (variant 5), the tensor-core pipeline (variant 9) and the
compensated state; one batched step of two instances; the two-level mixed
Poisson solve (jittered 16x16, N = 4).
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))

CHILD = r"""
import os, sys
import numpy as np
sys.path.insert(0, os.path.join(sys.argv[1], "dg-on-cuda_gb300"))
import torch
import dgc_gb300 as dg
from dgc_gb300 import meshes
out = sys.argv[2]
m = meshes.jittered_square(16, 7)
res = {}
for tag, prec, var in (("v5", dg.F32, 5), ("v9", dg.F32, 9), ("f32c", dg.F32C, None)):
    D = dg.Discretization(m, "maxwell_te", 6, prec)
    if var is not None:
        D.set_variant(var)
    x, y = D.node_xy()
    q0 = np.concatenate([np.sin(np.pi * x).reshape(-1) * 0.3, np.cos(np.pi * y).reshape(-1) * 0.2,
                         (np.cos(np.pi * x) * np.cos(np.pi * y)).reshape(-1)])
    dt = 0.3 * D.info.min_edge / 49.0
    a, b, r = D.upload(q0), D.empty_state(), D.empty_state()
    for n in range(12):
        D.lserk4_step(a, b, r, n * dt, dt)
        a, b = b, a
    res[tag + "_eager"] = a.cpu().numpy()
    fin = D.lserk4_run(D.upload(q0), D.empty_state(), D.empty_state(), 0.0, dt, 20, graph=True)
    res[tag + "_graph"] = fin.cpu().numpy()
    D.check()
insts = []
for n, N in ((10, 3), (12, 5)):
    D = dg.Discretization(meshes.jittered_square(n, n), "maxwell_tm", N, dg.F32)
    D.set_variant(5)
    x, y = D.node_xy()
    q = np.concatenate([np.zeros(x.size), np.zeros(x.size), (np.sin(np.pi * x) * np.sin(np.pi * y)).reshape(-1)])
    insts.append((D, D.upload(q), D.empty_state(), D.empty_state(), 0.2 * D.info.min_edge / (N + 1) ** 2))
B = dg.Batch([i[0] for i in insts])
fin = B.lserk4_run([i[1] for i in insts], [i[2] for i in insts], [i[3] for i in insts], [0.0, 0.0],
                   [i[4] for i in insts], 2, graph=True)
for k, f in enumerate(fin):
    res["batch%d" % k] = f.cpu().numpy()
m = meshes.jittered_square(16, 11)
D = dg.Discretization(m, "laplace", 4, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
x, y = D.node_xy()
D.block_jacobi()
D.coarse_build(8)
b = D.mass(D.upload((2 * np.pi ** 2 * np.sin(np.pi * x) * np.sin(np.pi * y)).reshape(-1)))
xs, st = D.pcg(b, mode=dg.SOLVE_TWO_LEVEL_MIXED, rtol=1e-10, maxit=4000)
res["poisson"] = xs.cpu().numpy()
xs, st = D.pcg(b, mode=dg.SOLVE_MIXED_IR, rtol=1e-10, maxit=40000)
res["poisson_ir"] = xs.cpu().numpy()
D.check()
np.savez(out, **res)
"""


@pytest.fixture(scope="module", autouse=True)
def built():
    from dgc_gb300 import build
    build.build()


def run_child(tmp_path, overlap):
    out = os.path.join(str(tmp_path), "overlap%d.npz" % overlap)
    env = dict(os.environ, DGC_STAGE_OVERLAP=str(overlap))
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT, out], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    return np.load(out)


def test_results_with_and_without_launch_overlap(tmp_path):
    on, off = run_child(tmp_path, 1), run_child(tmp_path, 0)
    assert sorted(on.files) == sorted(off.files)
    for k in on.files:
        assert on[k].shape == off[k].shape, k
        assert np.all(np.isfinite(on[k])), k
        if k.startswith("poisson"):
            # the solvers' dot products end in FP64 atomics, whose order varies
            # from run to run: the solutions agree to the solve tolerance
            d = np.linalg.norm(on[k] - off[k]) / np.linalg.norm(off[k])
            assert d < 1e-9, (k, d)
        else:
            assert np.array_equal(on[k].view(np.uint8), off[k].view(np.uint8)), k
