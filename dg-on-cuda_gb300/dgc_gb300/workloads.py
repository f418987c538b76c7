"""Small, self-contained workloads of single kernels, for profiling runs.

    python -m dgc_gb300.workloads <name> [--reps R]

Each workload builds its inputs, runs its kernel a few times untimed (graph
capture, autotuning and first-touch costs), synchronises, then launches the
kernel of interest R more times and checks the handle's device status.  The
sizes are the benchmark's own where they fit a profiler capture (inputs of
tens of MB, larger than L2 where DRAM figures matter) and smaller otherwise.
The kernel each workload targets, and how many launches precede the measured
ones, are printed on the first line, so that a profiler's kernel filter and
skip count can be read off.

    stage_x2     dg_rhs_x2_kernel<6, TE>: Maxwell TE, jittered 128x128 (K = 32768),
                 N = 6, compensated FP32 state, one LSERK4 stage per launch
    stage_fp64   dg_rhs_kernel<double, 6, TE>: the same workload in FP64
    stage_fp32   the autotuned FP32 stage kernel of the same workload
    batch        dg_batch_kernel: 24 seeded instances (advection / Maxwell TE / TM,
                 n in [8, 160], N in 2..8), each on its faster batch tile code
    mpnn_fwd     k_fwd_layer_tc: the 4-layer, width-64 network over a jittered
                 128x128 mesh (K = 32768), N = 4
    bj_apply     k_bj_apply<float>: block-Jacobi application inside the two-level
                 mixed PCG, jittered 256x256 mesh (K = 131072), N = 4
    grad_div     k_grad_div: weak-form gradient and divergence, K = 131072, N = 4, FP64
"""
from __future__ import annotations

import argparse
import sys

import numpy as np


def _sync():
    import torch
    torch.cuda.synchronize()


def stage(prec_name: str, reps: int):
    import dgc_gb300 as dg
    from dgc_gb300 import meshes
    prec = {"x2": dg.F32C, "fp64": dg.F64, "fp32": dg.F32}[prec_name]
    m = meshes.jittered_square(128, 2026)
    D = dg.Discretization(m, "maxwell_te", 6, prec)
    if prec == dg.F32:
        D.autotune(reps=5)
    x, y = D.node_xy()
    q = np.zeros((3,) + x.shape)
    q[2] = np.cos(np.pi * x) * np.cos(np.pi * y)
    a, b, r = D.upload(q), D.empty_state(), D.empty_state()
    dt = 0.5 * D.info.min_edge / 49.0
    warm = 15
    print(f"kernel: stage kernel ({prec_name}), warm-up launches {warm}, measured {reps}", flush=True)
    for s in range(warm):
        D.lserk4_stage(s % 5, a if s % 2 == 0 else b, b if s % 2 == 0 else a, r, 0.0, dt)
    _sync()
    for s in range(reps):
        D.lserk4_stage(s % 5, a if s % 2 == 0 else b, b if s % 2 == 0 else a, r, 0.0, dt)
    _sync()
    D.check()


def batch(reps: int):
    import dgc_gb300 as dg
    from dgc_gb300 import meshes
    rng = np.random.default_rng(777)
    insts = []
    for i in range(24):
        n = int(round(np.exp(rng.uniform(np.log(8), np.log(160)))))
        N = int(rng.integers(2, 9))
        kind = ["advection", "maxwell_te", "maxwell_tm"][int(rng.integers(0, 3))]
        D = dg.Discretization(meshes.jittered_square(n, 777 + i), kind, N, dg.F32, ax=0.6, ay=0.8,
                              bc=dg.BC_GAUSS)
        _, times = D.autotune(reps=5)
        blk = 5 if N <= 6 else 1
        D.set_variant(blk if times[blk] < times[0] else 0)
        x, y = D.node_xy()
        q = np.exp(-((x + 0.3) ** 2 + y ** 2) / 0.02)[None].repeat(D.Nf, 0)
        insts.append((D, q, 0.5 * D.info.min_edge / (N + 1) ** 2))
    B = dg.Batch([D for D, *_ in insts])
    qa = [D.upload(q) for D, q, _ in insts]
    qb = [D.empty_state() for D, *_ in insts]
    rs = [D.empty_state() for D, *_ in insts]
    dts = [dt for *_, dt in insts]
    print(f"kernel: dg_batch_kernel, warm-up launches 10, measured {5 * reps}", flush=True)
    B.lserk4_run(qa, qb, rs, [0.0] * len(insts), dts, 2, graph=False)
    _sync()
    B.lserk4_run(qa, qb, rs, [0.0] * len(insts), dts, reps, graph=False)
    _sync()
    for D, *_ in insts:
        D.check()


def mpnn_fwd(reps: int):
    import torch
    import dgc_gb300 as dg
    from dgc_gb300 import meshes
    D = dg.Discretization(meshes.jittered_square(128, 5151), "laplace", 4, dg.F64, tau=dg.TAU_SCALED,
                          dirichlet=True)
    net = dg.MPNN(D, layers=4, seed=3)
    w = net.get_weights()
    w[:] = np.random.default_rng(1).standard_normal(w.size).astype(np.float32) * 0.05
    net.set_weights(w)
    xin = torch.randn(D.K * D.NpP, dtype=torch.float32, device="cuda")
    print(f"kernel: k_fwd_layer_tc, warm-up forward passes 3, measured {reps}", flush=True)
    for _ in range(3):
        net.forward(xin)
    _sync()
    for _ in range(reps):
        net.forward(xin)
    _sync()


def bj_apply(reps: int):
    import dgc_gb300 as dg
    from dgc_gb300 import meshes
    D = dg.Discretization(meshes.jittered_square(256, 4242), "laplace", 4, dg.F64, tau=dg.TAU_SCALED,
                          dirichlet=True)
    x, y = D.node_xy()
    D.block_jacobi()
    D.coarse_build(32)
    b = D.mass(D.upload((2 * np.pi ** 2 * np.sin(np.pi * x) * np.sin(np.pi * y)).reshape(-1)))
    print(f"kernel: k_bj_apply (two-level mixed PCG iterations), solves 1 + {reps}", flush=True)
    D.pcg(b, mode=dg.SOLVE_TWO_LEVEL_MIXED, rtol=1e-10, maxit=40, check=False)
    _sync()
    for _ in range(reps):
        D.pcg(b, mode=dg.SOLVE_TWO_LEVEL_MIXED, rtol=1e-10, maxit=40, check=False)
    _sync()
    D.check()


def grad_div(reps: int):
    import dgc_gb300 as dg
    from dgc_gb300 import meshes
    D = dg.Discretization(meshes.jittered_square(256, 4242), "laplace", 4, dg.F64, tau=dg.TAU_SCALED,
                          dirichlet=True)
    x, y = D.node_xy()
    u = D.upload((np.sin(np.pi * x) * np.cos(np.pi * y)).reshape(-1))
    print(f"kernel: k_grad_div, warm-up launches 4, measured {2 * reps}", flush=True)
    for _ in range(2):
        gx, gy = D.grad(u)
        D.div(gx, gy)
    _sync()
    for _ in range(reps):
        gx, gy = D.grad(u)
        D.div(gx, gy)
    _sync()
    D.check()


WORKLOADS = {
    "stage_x2": lambda r: stage("x2", r),
    "stage_fp64": lambda r: stage("fp64", r),
    "stage_fp32": lambda r: stage("fp32", r),
    "batch": batch,
    "mpnn_fwd": mpnn_fwd,
    "bj_apply": bj_apply,
    "grad_div": grad_div,
}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("name", choices=sorted(WORKLOADS))
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args(argv)
    import torch
    torch.cuda.set_device(0)
    WORKLOADS[a.name](a.reps)
    print("workload ok", flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
