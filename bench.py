#!/usr/bin/env python
"""Headline benchmark: 2D Maxwell TE in a PEC cavity, mixed precision.

Workload (one "step" = one LSERK4 time step = 5 fused RHS+stage launches):
  jittered 128x128 square mesh (K = 32768 triangles), order N = 6 (Np = 28),
  TE cavity mode Hz = cos(pi x) cos(pi y), Ex = Ey = 0 at t = 0,
  dt = 0.5 min(edge) / (N+1)^2.  State and element contractions in FP32;
  geometric factors computed in FP64 on the host and stored rounded to FP32
  for the FP32 kernels.  Metric: GDOF/s = 3 Np K RHS-evaluations per second / 1e9.

Timing: W warm-up steps, then K timed steps; before every timed step L2 is
flushed by writing a 512 MiB buffer (outside the timed events); each stage
launch is bracketed by CUDA events on the launching stream; max over ranks.
Replicas only: under torchrun every rank runs the same workload on its own GPU
and `value` is the sum of the ranks' throughput at the slowest rank's time.

--impl reference times the reference's CPU implementation of the same path
(the oracle's serial C port of maxwell_2d + LSERK4, one core) on this host.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "dg-on-cuda_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

ORDER = 6
NSIDE = 128
SEED = 2026
METRIC = "GDOF/s (Maxwell TE N=6 K=32768, LSERK4, mixed FP32 vs FP64 plain)"
UNIT = "GDOF/s"
WORKLOAD = "maxwell_te_pec_cavity_k32768_n6_lserk4"
# FP32 stage-kernel variants at order 6 (dgc_set_variant / dgc_autotune)
STAGE_KERNELS = {
    0: "dgk::dg_rhs_kernel<float,6,PHYS_TE>",
    1: "dgk::dg_rhs_v2_kernel<6,PHYS_TE,8,4>",
    2: "dgk::dg_rhs_v2_kernel<6,PHYS_TE,4,8>",
    3: "dgk::dg_rhs_v2_kernel<6,PHYS_TE,4,4>",
    4: "dgk::dg_rhs_tc_kernel<6,PHYS_TE> (tcgen05, split TF32)",
    5: "dgk::dg_rhs_blk_kernel<6,PHYS_TE,1>",
    6: "dgk::dg_rhs_blk_kernel<6,PHYS_TE,2>",
    7: "dgk::dg_rhs_blk_kernel<6,PHYS_TE,1> (warp-uniform operator loads)",
    8: "dgk::dg_rhs_tct_kernel<6,PHYS_TE> (tcgen05, A in TMEM, split TF32)",
    9: "dgk::dg_rhs_tcp_kernel<6,PHYS_TE> (tcgen05, A in TMEM, warp-specialized pipeline)",
}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def te_initial(x, y):
    q = np.zeros((3,) + x.shape)
    q[2] = np.cos(np.pi * x) * np.cos(np.pi * y)
    return q


def te_exact(x, y, t):
    s2 = np.sqrt(2.0)
    q = np.zeros((3,) + x.shape)
    q[0] = -np.cos(np.pi * x) * np.sin(np.pi * y) * np.sin(s2 * np.pi * t) / s2
    q[1] = np.sin(np.pi * x) * np.cos(np.pi * y) * np.sin(s2 * np.pi * t) / s2
    q[2] = np.cos(np.pi * x) * np.cos(np.pi * y) * np.cos(s2 * np.pi * t)
    return q


def config_dict(n_gpus):
    return {"workload": WORKLOAD, "mesh": f"jittered {NSIDE}x{NSIDE} squares split into triangles",
            "num_cells": 2 * NSIDE * NSIDE, "order": ORDER, "fields": 3,
            "integrator": "LSERK4 (Carpenter-Kennedy 5-stage), one fused launch per stage",
            "precision": "fp32 state and contractions; geometric factors computed in fp64, stored fp32",
            "l2": "flushed between timed steps (512 MiB write)",
            "parallelism": f"replicas x{n_gpus}"}


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def oracle_sample(steps: int, warm: int):
    """Serial oracle (C port of the reference CPU path): LSERK4 steps on the
    full workload.  Returns (GDOF/s, seconds per step)."""
    import oracle
    from dgc_gb300 import meshes
    m = meshes.jittered_square(NSIDE, SEED)
    o = oracle.Oracle(m.xy, m.cells, ORDER)
    p = oracle.problem(oracle.MAXWELL_TE)
    x, y = o.node_xy()
    q = te_initial(x, y).reshape(-1)
    res = np.zeros_like(q)
    dt = 0.5 * meshes.min_edge_length(m) / (ORDER + 1) ** 2
    for _ in range(warm):
        q, res = o.lserk4_step(p, 0.0, dt, q, res)
    t0 = time.perf_counter()
    for _ in range(steps):
        q, res = o.lserk4_step(p, 0.0, dt, q, res)
    sec = (time.perf_counter() - t0) / max(steps, 1)
    dofs = 3 * o.Np * o.K
    return dofs * 5 / sec / 1e9, sec


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thr = threading.Thread(target=self._read, daemon=True)
            self.thr.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) < 9:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# committed ncu summaries of the stage-kernel variants on this workload
PROFILES = {5: "dg_rhs_blk_maxwell_te_n6_fp32.md", 9: "dg_rhs_tcp_maxwell_te_n6_fp32.md",
            "x2": "dg_rhs_x2_maxwell_te_n6_fp32c.md"}


def read_traffic(variant):
    """DRAM bytes per launch of the chosen stage kernel from its committed ncu
    summary (None when no summary covers that variant)."""
    if variant not in PROFILES:
        return None
    path = os.path.join(ROOT, "profiles", PROFILES[variant])
    try:
        txt = open(path).read()
        m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", txt)
        return float(m.group(1)) if m else None
    except OSError:
        return None


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


POISSON_NSIDE, POISSON_ORDER, POISSON_SEED = 256, 4, 4242
POISSON_AGGREGATE = 32                          # cells per aggregate of the two-level line


def fourier_rhs(x, y, seed: int, modes: int = 32):
    """Sum of `modes` sine modes sin(kx pi (x+1)/2) sin(ky pi (y+1)/2), kx, ky in
    1..8 drawn from `seed`, amplitudes ~ N(0, |k|^-3) (zero on the boundary)."""
    rng = np.random.default_rng(seed)
    f = np.zeros_like(x)
    for _ in range(modes):
        kx, ky = rng.integers(1, 9, size=2)
        a = rng.normal(0.0, (kx * kx + ky * ky) ** -0.75)
        f += a * np.sin(kx * np.pi * (x + 1) / 2) * np.sin(ky * np.pi * (y + 1) / 2)
    return f


def measure_poisson(dg, meshes):
    """IPDG Poisson -lap u = f, Dirichlet u = 0, jittered 256x256 mesh (K = 131072),
    N = 4, tau = (N+1)^2 / h: FP64 block-Jacobi PCG against FP32 inner PCG in
    FP64 iterative refinement, both to 1e-10 relative FP64 residual, for the
    manufactured solution sin(pi x) sin(pi y) and a 32-mode Fourier right-hand side.
    An extra line (no counterpart in the workload's definition): the two-level PCG
    (block-Jacobi + smoothed-aggregation coarse space of POISSON_AGGREGATE cells)."""
    import torch
    m = meshes.jittered_square(POISSON_NSIDE, POISSON_SEED)
    D = dg.Discretization(m, "laplace", POISSON_ORDER, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    x, y = D.node_xy()
    D.block_jacobi()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    D.coarse_build(POISSON_AGGREGATE)
    torch.cuda.synchronize()
    _, n_agg, n_col, omega = D.coarse_info()
    out = {"workload": f"ipdg_poisson_dirichlet_k{D.K}_n{POISSON_ORDER}", "num_cells": D.K,
           "order": POISSON_ORDER, "rtol": 1e-10,
           "two_level": {"cells_per_aggregate": POISSON_AGGREGATE, "aggregates": n_agg, "colours": n_col,
                         "omega": omega, "build_s": time.perf_counter() - t0},
           "cases": {}}
    cases = {"manufactured": 2 * np.pi ** 2 * np.sin(np.pi * x) * np.sin(np.pi * y),
             "fourier32": fourier_rhs(x, y, POISSON_SEED)}
    for name, f in cases.items():
        b = D.mass(D.upload(f.reshape(-1)))
        res = {}
        sols = {}
        for mode, tag in ((dg.SOLVE_FP64_PCG, "fp64_pcg"), (dg.SOLVE_MIXED_IR, "mixed_ir"),
                          (dg.SOLVE_TWO_LEVEL, "two_level"), (dg.SOLVE_TWO_LEVEL_MIXED, "two_level_mixed")):
            D.pcg(b, mode=mode, rtol=1e-10, maxit=40000, check=False)  # warm-up (graphs, preconditioner)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            xs, st = D.pcg(b, mode=mode, rtol=1e-10, maxit=40000, check=False)
            torch.cuda.synchronize()
            st["wall_s"] = time.perf_counter() - t0
            sols[tag] = D.download(xs).reshape(-1)
            res[tag] = {k: st[k] for k in ("iterations", "outer_iterations", "converged", "final_relres", "wall_s")}
        ref = sols["fp64_pcg"]
        res["rel_l2_mixed_vs_fp64"] = float(np.linalg.norm(sols["mixed_ir"] - ref) / np.linalg.norm(ref))
        res["rel_l2_two_level_vs_fp64"] = float(np.linalg.norm(sols["two_level"] - ref) / np.linalg.norm(ref))
        res["rel_l2_two_level_mixed_vs_fp64"] = float(np.linalg.norm(sols["two_level_mixed"] - ref) /
                                                      np.linalg.norm(ref))
        if name == "manufactured":
            ex = (np.sin(np.pi * x) * np.sin(np.pi * y)).reshape(-1)
            for tag in sols:
                res[tag]["rel_l2_vs_exact"] = float(np.linalg.norm(sols[tag] - ex) / np.linalg.norm(ex))
        res["speedup_mixed_vs_fp64"] = res["fp64_pcg"]["wall_s"] / res["mixed_ir"]["wall_s"]
        res["speedup_two_level_vs_fp64"] = res["fp64_pcg"]["wall_s"] / res["two_level"]["wall_s"]
        res["speedup_two_level_vs_mixed"] = res["mixed_ir"]["wall_s"] / res["two_level"]["wall_s"]
        res["speedup_two_level_mixed_vs_mixed"] = res["mixed_ir"]["wall_s"] / res["two_level_mixed"]["wall_s"]
        out["cases"][name] = res
    D.check()
    return out


STOKES_NSIDE, STOKES_ORDER, STOKES_SEED, STOKES_STEPS, STOKES_DT = 128, 4, 77, 10, 1e-3


def measure_stokes(dg, meshes):
    """The Stokes example's dual-splitting step (examples/stokes_2d) on a jittered
    128x128 mesh (K = 32768), N = 4, from its exact initial velocity (u^-1 = u^0),
    STOKES_STEPS steps of dt = 1e-3, the Dirichlet data in the consistent form:
    time per step and the error against the analytic solution, with the pressure
    system solved by block-Jacobi refinement and by the two-level PCG."""
    import torch
    from dgc_gb300 import stokes as st
    m = meshes.jittered_square(STOKES_NSIDE, STOKES_SEED)
    out = {"workload": f"stokes_dual_splitting_k{m.cells.shape[0]}_n{STOKES_ORDER}", "num_cells": m.cells.shape[0],
           "order": STOKES_ORDER, "dt": STOKES_DT, "steps": STOKES_STEPS,
           "data": "exact initial velocity, consistent Dirichlet data, rtol 1e-10 per solve"}
    for tag, mode in (("mixed_ir", dg.SOLVE_MIXED_IR), ("two_level", dg.SOLVE_TWO_LEVEL),
                      ("two_level_mixed", dg.SOLVE_TWO_LEVEL_MIXED)):
        S = st.Stokes(m, STOKES_ORDER, consistent=True, rtol=1e-10, mode=mode)
        S.run_example(T=2 * STOKES_DT, dt=STOKES_DT)                     # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, _, t, err, iters = S.run_example(T=STOKES_STEPS * STOKES_DT, dt=STOKES_DT)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        out[tag] = {"ms_per_step": wall / STOKES_STEPS * 1e3, "solver_iterations_per_step": iters / STOKES_STEPS,
                    "error_norm": err, "T": t}
        S.close()
    out["speedup_two_level_vs_mixed"] = out["mixed_ir"]["ms_per_step"] / out["two_level"]["ms_per_step"]
    return out


LEARN_NSIDE, LEARN_ORDER, LEARN_SEED = 128, 4, 5151
LEARN_TRAIN, LEARN_HELD = 1600, 400            # the full sequence: 2000 solves
LEARN_TRAIN_SAMPLE, LEARN_HELD_SAMPLE = 16, 24  # the bounded sample timed here
LEARN_FP64_HELD = 8                             # held-out solves also timed with plain FP64 PCG
LEARN_SNAPSHOTS = (4, 16, 64, 256, 1024)       # PCG iterates giving residual / error pairs
LEARN_AGGREGATE = 8                             # cells per aggregate of the coarse space


def smooth_rhs(x, y, index: int, modes: int = 24):
    """Right-hand side `index` of the learned-preconditioner sequence: `modes` sine
    modes sin(kx pi (x+1)/2) sin(ky pi (y+1)/2), kx, ky in 1..8, amplitudes
    ~ N(0, |k|^-2), seeded by the index (zero on the boundary)."""
    rng = np.random.default_rng(LEARN_SEED * 100003 + index)
    f = np.zeros_like(x)
    for _ in range(modes):
        kx, ky = rng.integers(1, 9, size=2)
        f += rng.normal(0.0, (kx * kx + ky * ky) ** -0.5) * np.sin(kx * np.pi * (x + 1) / 2) * \
            np.sin(ky * np.pi * (y + 1) / 2)
    return f


def measure_learned(dg, meshes, n_train=LEARN_TRAIN_SAMPLE, n_held=LEARN_HELD_SAMPLE, n_fp64=LEARN_FP64_HELD,
                    snapshots=LEARN_SNAPSHOTS, full=False, activation="relu", correction="additive"):
    """Learned preconditioner on IPDG Poisson (Dirichlet, jittered 128x128 mesh,
    K = 32768, N = 4), in two-level form: M r = Binv r + P A_c^-1 P^T r + network,
    the coarse space a smoothed aggregation of LEARN_AGGREGATE cells.  Residual /
    error pairs from plain block-Jacobi PCG iterates of the first training solves
    train the 4-layer width-64 message-passing network (BF16 weights, FP32
    accumulation, energy-norm loss, Adam) on what the two-level base leaves; on
    held-out solves the learned solve (truncated flexible CG, block-Jacobi PCG as
    fallback once its break-even budget is spent) is timed against plain
    FP64 block-Jacobi PCG, the mixed FP32/FP64 refinement and the same two-level
    flexible CG without the network, all to 1e-10 relative FP64 residual.  By
    default a bounded sample of the 2000-solve sequence (1600 train / 400 held
    out): the first n_train training and n_held held-out right-hand sides, plain
    FP64 PCG timed on the first n_fp64 of them.  With full=True (bench.py
    --learned-full) the whole sequence: pairs from plain PCG iterates of all 1600
    training solves (their errors against a two-level solve to 1e-11, the plain
    FP64 solve being the slowest part of the data generation) and all 400
    held-out solves."""
    import torch
    m = meshes.jittered_square(LEARN_NSIDE, LEARN_SEED)
    D = dg.Discretization(m, "laplace", LEARN_ORDER, dg.F64, tau=dg.TAU_SCALED, dirichlet=True)
    x, y = D.node_xy()
    D.block_jacobi()
    c = float(np.sqrt(D.K * D.Np))
    net = dg.MPNN(D, layers=4, seed=LEARN_SEED)
    if activation == "linear":   # a fixed linear correction: flexible CG sees a fixed preconditioner
        net.set_activation(dg.MPNN_ACT_LINEAR)
    if correction == "residual":  # the network acts on r' = r - S z0, the residual the two-level step leaves
        net.set_correction(dg.MPNN_CORR_RESIDUAL)
    bj = dg.MPNN(D, layers=1, seed=0)               # zero output layer: M(r) = Binv r + coarse
    # two-level form: the coarse space (smoothed aggregation) removes the smooth
    # mesh-wide error that a 4-hop network cannot see; the network learns the rest
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    bj.set_coarse(LEARN_AGGREGATE)
    torch.cuda.synchronize()
    coarse_s = time.perf_counter() - t0
    net.set_coarse(LEARN_AGGREGATE)
    _, n_agg, n_col, omega = D.coarse_info()

    def rhs(i):
        return D.mass(D.upload(smooth_rhs(x, y, i).reshape(-1)))

    def sync_time(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    # training pairs: x = r c/|r|, t = (e - M_0 r) c/|r| at PCG iterates x_k, e = x* - x_k,
    # M_0 = Binv + the coarse correction
    t0 = time.perf_counter()
    X, T, pcg_its = [], [], []
    for i in range(n_train):
        b = rhs(i)
        if full:
            xs, st = D.pcg(b, mode=dg.SOLVE_TWO_LEVEL, rtol=1e-11, maxit=40000, check=False)
            if i < n_fp64:
                pcg_its.append(D.pcg(b, rtol=1e-10)[1]["iterations"])
        else:
            xs, st = D.pcg(b, rtol=1e-10)
            pcg_its.append(st["iterations"])
        for k in snapshots:
            xk, _ = D.pcg(b, rtol=1e-30, maxit=k, check=False)
            r = b - D.spd(xk)
            z0 = bj.precondition(r)
            rin = r - D.spd(z0) if correction == "residual" else r
            nr = float(torch.linalg.norm(rin))
            X.append((rin * (c / nr)).float())
            T.append(((xs - xk - z0) * (c / nr)).float())
    torch.cuda.synchronize()
    datagen_s = time.perf_counter() - t0
    sigma = float(torch.sqrt(torch.mean(torch.stack([torch.mean(t.double() ** 2) for t in T]))))
    T = [t / sigma for t in T]
    rng = np.random.default_rng(LEARN_SEED)
    losses, batch, epochs, lr = [], 8, 30, 1e-4
    t0 = time.perf_counter()
    for ep in range(epochs):
        order = rng.permutation(len(X))
        el = [net.train_step(torch.cat([X[j] for j in order[i:i + batch]]),
                             torch.cat([T[j] for j in order[i:i + batch]]), lr=lr)[0]
              for i in range(0, len(X), batch)]
        losses.append(float(np.mean(el)))
    # step length of the network's correction: theta minimises sum_j |t_j - theta y_j|_S^2
    # over the training pairs (energy norm), so an output uncorrelated with the targets
    # is scaled towards zero instead of disturbing the flexible CG
    num = den = 0.0
    for xj, tj in zip(X, T):
        yj = net.forward(xj).double()
        syj = D.spd(yj)
        num += float(torch.dot(tj.double(), syj))
        den += float(torch.dot(yj, syj))
    theta = num / den if den > 0.0 else 0.0
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    w = net.get_weights()
    # targets were trained in units of sigma; the output layer also takes theta
    w[-(D.NpP * 64 + D.NpP):] *= sigma * theta
    net.set_weights(w)

    # per-iteration costs and the flexible-CG budget beyond which it cannot beat plain PCG
    b0 = rhs(0)
    (_, st_p), tp = sync_time(lambda: D.pcg(b0, rtol=1e-10))
    (_, st_f), tf = sync_time(lambda: net.fpcg(b0, rtol=1e-30, maxit=300, check=False))
    it_p, it_f = tp / st_p["iterations"], tf / max(st_f["iterations"], 1)
    budget = int(np.median(pcg_its) * it_p / it_f)
    _, t_fwd = sync_time(lambda: [net.forward(X[0]) for _ in range(20)])

    held = {"fp64_pcg": [], "mixed_ir": [], "two_level_no_network": [], "learned": []}
    fell = fell0 = 0
    agree = []
    for i in range(n_held):
        b = rhs(LEARN_TRAIN + i)
        if i < n_fp64:
            (xp, sp), tp = sync_time(lambda: D.pcg(b, rtol=1e-10))
            held["fp64_pcg"].append((sp["iterations"], tp, sp["final_relres"]))
        else:
            xp, _ = D.pcg(b, mode=dg.SOLVE_TWO_LEVEL, rtol=1e-11, maxit=40000, check=False)  # reference only
        (_, sm), tm = sync_time(lambda: D.pcg(b, mode=dg.SOLVE_MIXED_IR, rtol=1e-10))
        (_, s0), t0_ = sync_time(lambda: bj.solve(b, rtol=1e-10, fcg_maxit=budget))
        (xl, sl), tl = sync_time(lambda: net.solve(b, rtol=1e-10, fcg_maxit=budget))
        fell += int(sl["fell_back"])
        fell0 += int(s0["fell_back"])
        held["mixed_ir"].append((sm["iterations"], tm, sm["final_relres"]))
        held["two_level_no_network"].append((s0["iterations"], t0_, s0["final_relres"]))
        held["learned"].append((sl["iterations"], tl, sl["final_relres"], sl["inner_iterations"]))
        agree.append(float(torch.linalg.norm(xl - xp) / torch.linalg.norm(xp)))
    D.check()

    def summary(rows):
        its = [r[0] for r in rows]
        ts = [r[1] for r in rows]
        return {"iterations_median": float(np.median(its)), "wall_s_p50": float(np.percentile(ts, 50)),
                "wall_s_p95": float(np.percentile(ts, 95)), "wall_s_total": float(np.sum(ts)),
                "max_final_relres": float(max(r[2] for r in rows))}

    out = {"workload": f"ipdg_poisson_dirichlet_k{D.K}_n{LEARN_ORDER}_learned_precond", "activation": activation,
           "correction": correction,
           "num_cells": D.K, "order": LEARN_ORDER, "rtol": 1e-10,
           "sequence": {"solves": LEARN_TRAIN + LEARN_HELD, "train": LEARN_TRAIN, "held_out": LEARN_HELD,
                        "rhs": "24 Fourier modes, amplitudes ~ N(0, |k|^-2), seeded per solve"},
           "sample": {"train_solves": n_train, "held_out_solves": n_held, "fp64_pcg_timed_on": n_fp64,
                      "pairs": len(X), "snapshots": list(snapshots), "full_sequence": full},
           "network": {"layers": 4, "width": 64, "params": net.num_params, "weights": "bf16 (fp32 masters)",
                       "accumulate": "fp32", "loss": "energy norm |y - t|_S^2 / |t|_S^2",
                       "optimizer": f"Adam lr {lr:g}, batch {batch}, {epochs} epochs",
                       "theta": theta,
                       "forward_ms": t_fwd / 20 * 1e3},
           "coarse": {"cells_per_aggregate": LEARN_AGGREGATE, "aggregates": n_agg, "colours": n_col,
                      "omega": omega, "build_s": coarse_s,
                      "form": "M r = Binv r + P A_c^-1 P^T r + net, P = (I - omega Binv S) P0 (smoothed "
                              "aggregation), A_c = P^T S P inverted once; smoothing applies in FP32"},
           "datagen_s": datagen_s, "train_s": train_s, "loss_per_epoch": losses,
           "pcg_iteration_ms": it_p * 1e3, "fcg_iteration_ms": it_f * 1e3, "fcg_budget": budget,
           "held_out": {k: summary(v) for k, v in held.items()},
           "fallback_count": fell, "fallback_count_two_level_no_network": fell0,
           "max_rel_l2_learned_vs_fp64_pcg": float(max(agree))}
    ho = out["held_out"]
    # per-solve medians: the FP64 PCG arm is timed on the first n_fp64 solves only
    out["speedup_learned_vs_fp64_pcg"] = ho["fp64_pcg"]["wall_s_p50"] / ho["learned"]["wall_s_p50"]
    out["speedup_learned_vs_mixed_ir"] = ho["mixed_ir"]["wall_s_total"] / ho["learned"]["wall_s_total"]
    # what the trained network adds to the same two-level method without it
    out["network_gain"] = {
        "iterations": ho["two_level_no_network"]["iterations_median"] / ho["learned"]["iterations_median"],
        "wall_time": ho["two_level_no_network"]["wall_s_total"] / ho["learned"]["wall_s_total"]}
    return out


BATCH_INSTANCES, BATCH_SEED, BATCH_STEPS = 96, 777, 10


def batch_specs():
    """The batched workload's instances, drawn from BATCH_SEED: n log-uniform in
    [8, 160] squares per side, N uniform in {2..8}, physics uniform over advection
    (random direction, Gaussian pulse at a random centre) and Maxwell TE / TM."""
    rng = np.random.default_rng(BATCH_SEED)
    out = []
    for i in range(BATCH_INSTANCES):
        n = int(round(np.exp(rng.uniform(np.log(8), np.log(160)))))
        N = int(rng.integers(2, 9))
        kind = ["advection", "maxwell_te", "maxwell_tm"][int(rng.integers(0, 3))]
        sp = {"n": n, "N": N, "kind": kind, "seed": BATCH_SEED + i}
        if kind == "advection":
            th = rng.uniform(0, 2 * np.pi)
            sp.update(ax=float(np.cos(th)), ay=float(np.sin(th)), gx0=float(rng.uniform(-0.5, 0.5)),
                      gy0=float(rng.uniform(-0.5, 0.5)))
        out.append(sp)
    return out


def batch_initial(sp, x, y):
    """Initial state of a batch instance in the reference CPU layout [field][cell][node]."""
    if sp["kind"] == "advection":
        return np.exp(-((x - sp["gx0"]) ** 2 + (y - sp["gy0"]) ** 2) / 0.02)[None]
    q = np.zeros((3,) + x.shape)
    # TE: Hz = cos cos; TM: Ez = sin sin (both PEC cavity modes)
    q[2] = (np.cos(np.pi * x) * np.cos(np.pi * y) if sp["kind"] == "maxwell_te"
            else np.sin(np.pi * x) * np.sin(np.pi * y))
    return q


def _cpu_batch_worker(specs):
    """One host process: one LSERK4 step of each given instance with the oracle
    (the serial C port of the reference CPU operator, FP64); returns (DOF-stage
    evaluations, seconds of the steps alone)."""
    import oracle
    from dgc_gb300 import meshes
    work, sec = 0.0, 0.0
    kinds = {"advection": oracle.ADVECTION, "maxwell_te": oracle.MAXWELL_TE, "maxwell_tm": oracle.MAXWELL_TM}
    for sp in specs:
        m = meshes.jittered_square(sp["n"], sp["seed"])
        o = oracle.Oracle(m.xy, m.cells, sp["N"])
        if sp["kind"] == "advection":
            p = oracle.problem(oracle.ADVECTION, sp["ax"], sp["ay"], oracle.BC_GAUSS, sp["gx0"], sp["gy0"], 0.02)
        else:
            p = oracle.problem(kinds[sp["kind"]])
        x, y = o.node_xy()
        q = batch_initial(sp, x, y).reshape(-1)
        dt = 0.5 * meshes.min_edge_length(m) / (sp["N"] + 1) ** 2
        t0 = time.perf_counter()
        o.lserk4_step(p, 0.0, dt, q, np.zeros_like(q))
        sec += time.perf_counter() - t0
        work += q.size * 5
    return work, sec


def cpu_batched_baseline():
    """The batched workload on the host cores: one process per core (spawned, so
    no CUDA state is inherited), the instances dealt out longest first, one LSERK4
    step of each.  Aggregate GDOF/s over the slowest process's step time, and the
    same work on one core."""
    import multiprocessing as mp
    specs = batch_specs()
    cores = os.cpu_count() or 1
    cost = lambda sp: 2 * sp["n"] ** 2 * ((sp["N"] + 1) * (sp["N"] + 2) // 2) ** 2 * (1 if sp["kind"] == "advection" else 3)  # noqa: E731,E501
    bins = [[] for _ in range(cores)]
    load = [0.0] * cores
    for sp in sorted(specs, key=cost, reverse=True):
        j = int(np.argmin(load))
        bins[j].append(sp)
        load[j] += cost(sp)
    with mp.get_context("spawn").Pool(cores) as pool:
        res = pool.map(_cpu_batch_worker, [b for b in bins if b])
    work = sum(r[0] for r in res)
    span = max(r[1] for r in res)
    serial = sum(r[1] for r in res)
    return {"value": work / span / 1e9, "unit": UNIT, "cores": cores, "kind": "port",
            "single_core_gdofs": work / serial / 1e9,
            "sample": f"one LSERK4 step of each of the {len(specs)} instances (serial C port of the reference CPU "
                      f"operator, FP64), one spawned process per core, instances dealt longest first; "
                      f"host {cpu_model()}"}


def measure_batched(dg, meshes):
    """96 independent FP32 instances (advection with a random velocity direction
    and Gaussian pulse, or a Maxwell TE / TM cavity mode) on jittered meshes with
    n log-uniform in [8, 160] squares per side and N uniform in {2..8}.  Every
    instance is autotuned first.  Batched: one persistent launch per LSERK4
    stage for all instances, the step replayed from a CUDA graph, each instance
    on the faster of the two tile codes the batch offers (variant 0 or the
    register-blocked variant, by its autotune times).  Sequential: instance
    after instance, each with its own autotuned variant, its steps replayed
    from its own CUDA graph.  Aggregate GDOF/s of both."""
    import torch
    insts = []
    for sp in batch_specs():
        N, kind = sp["N"], sp["kind"]
        m = meshes.jittered_square(sp["n"], sp["seed"])
        if kind == "advection":
            D = dg.Discretization(m, kind, N, dg.F32, ax=sp["ax"], ay=sp["ay"], bc=dg.BC_GAUSS,
                                  gx0=sp["gx0"], gy0=sp["gy0"], gw=0.02)
        else:
            D = dg.Discretization(m, kind, N, dg.F32)
        x, y = D.node_xy()
        q = batch_initial(sp, x, y)
        tuned, times = D.autotune(reps=5)
        blk = 5 if N <= 6 else 1
        batch_v = blk if times[blk] < times[0] else 0
        insts.append((D, q.reshape(-1), 0.5 * D.info.min_edge / (N + 1) ** 2, tuned, batch_v))
    dofs = sum(D.Nf * D.Np * D.K for D, *_ in insts)
    for D, _, _, _, bv in insts:
        D.set_variant(bv)
    B = dg.Batch([D for D, *_ in insts])
    dts = [it[2] for it in insts]
    qa = [D.upload(q) for D, q, *_ in insts]
    qb = [D.empty_state() for D, *_ in insts]
    rs = [D.empty_state() for D, *_ in insts]
    B.lserk4_run(qa, qb, rs, [0.0] * len(insts), dts, 4, graph=True)  # warm-up (even: back in qa)
    for (D, q, *_), a in zip(insts, qa):                              # both arms start from the same state
        a.copy_(D.upload(q))
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = B.launch_count()
    ev0.record()
    fin = B.lserk4_run(qa, qb, rs, [0.0] * len(insts), dts, BATCH_STEPS, graph=True)
    ev1.record()
    torch.cuda.synchronize()
    batched_ms = ev0.elapsed_time(ev1)
    batch_launches = B.launch_count() - l0
    B.close()
    # sequential: the same steps, instance after instance, each with its autotuned variant
    for D, _, _, tv, _ in insts:
        D.set_variant(tv)
    sa = [D.upload(q) for D, q, *_ in insts]
    sb = [D.empty_state() for D, *_ in insts]
    sr = [D.empty_state() for D, *_ in insts]
    for (D, *_), a, b, r, dt in zip(insts, sa, sb, sr, dts):
        D.lserk4_run(a, b, r, 0.0, dt, 4, graph=True)                  # warm-up, graph capture
    for (D, q, *_), a in zip(insts, sa):                               # same buffers: the graphs are reused
        a.copy_(D.upload(q))
    torch.cuda.synchronize()
    seq_fin = []
    ev0.record()
    for (D, *_), a, b, r, dt in zip(insts, sa, sb, sr, dts):
        seq_fin.append(D.lserk4_run(a, b, r, 0.0, dt, BATCH_STEPS, graph=True))
    ev1.record()
    torch.cuda.synchronize()
    seq_ms = ev0.elapsed_time(ev1)
    # instances whose batch tile code is their tuned variant must agree bit for bit
    same = [i for i, it in enumerate(insts) if it[3] == it[4]]
    bitwise = all(torch.equal(fin[i], seq_fin[i]) for i in same)
    diff = max(float((f - g).abs().max()) / max(float(g.abs().max()), 1e-30) for f, g in zip(fin, seq_fin))
    for D, *_ in insts:
        D.check()
    Ks = [D.K for D, *_ in insts]
    codes = [it[4] for it in insts]
    return {"workload": f"batched_{len(insts)}_instances", "instances": len(insts),
            "dofs_total": dofs, "K_range": [min(Ks), max(Ks)],
            "orders": sorted({D.N for D, *_ in insts}), "steps": BATCH_STEPS,
            "geometry": "fp32 records rounded from fp64 set-up (rounding measured without effect on the "
                        "error floor)",
            "batched": {"gdofs": dofs * 5 * BATCH_STEPS / (batched_ms * 1e-3) / 1e9, "ms": batched_ms,
                        "launches_per_step": batch_launches / BATCH_STEPS, "graph": True,
                        "instances_on_blocked_tiles": sum(1 for c in codes if c != 0)},
            "sequential": {"gdofs": dofs * 5 * BATCH_STEPS / (seq_ms * 1e-3) / 1e9, "ms": seq_ms,
                           "launches_per_step": 5 * len(insts), "graph": True,
                           "variants": {str(v): sum(1 for it in insts if it[3] == v)
                                        for v in sorted({it[3] for it in insts})}},
            "speedup_batched_vs_sequential": seq_ms / batched_ms,
            "bitwise_equal_where_same_tile_code": bitwise, "instances_same_tile_code": len(same),
            "max_rel_diff_batched_vs_sequential": diff}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    gdofs, sec = None, None
    try:
        # each step is one full LSERK4 step of the workload on one core
        gdofs, sec = oracle_sample(args.steps, args.warmup)
    except Exception as e:  # pragma: no cover
        print(json.dumps({"impl": "reference", "unavailable": f"oracle port failed: {e}"}))
        return
    line = {"metric": METRIC, "value": gdofs, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config_dict(args.gpus),
            "impl": "reference",
            "cpu_baseline": {"value": gdofs, "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": f"{args.steps} full LSERK4 steps of the workload (serial C port of "
                                       "the reference CPU operator, FP64), host " + cpu_model()},
            "e2e": {"value": gdofs, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


E2E_STREAMS = 3  # CUDA streams the end-to-end loop issues its independent steps on
E2E_SETS = 9     # device buffer sets it rotates through (3 x 11 MB each; a multiple of E2E_STREAMS)


def measure_e2e(D32, bufs, res, flush, stream, t, dt, steps, ws, dofs, barrier):
    """End to end through the C ABI with pinned host buffers, every step: H2D of
    the step's input state, one LSERK4 step (dgc_lserk4_step), D2H of the new
    state.  Steps are independent (each starts from the host state), so they are
    issued round robin on E2E_STREAMS CUDA streams: one step's copies overlap the
    others' kernels, as a host application streaming states through the library
    would run it.  The device buffers rotate through E2E_SETS sets (297 MB in all,
    more than L2), so nothing a step reads stays in L2 from an earlier step except
    what its own host-to-device copy has just written.  The same calls on
    one stream, one step after another with an L2 flush between steps, are
    reported as `serial`."""
    import torch
    from dgc_gb300 import replicas
    n = D32.state_len
    h_state = torch.empty(n, dtype=torch.float32, pin_memory=True)
    h_state.copy_(bufs[0].cpu())
    # pinned as well (empty_like would not pin it): a pageable target is staged
    # through a bounce buffer and page-faults on its first write
    h_out = [torch.empty(n, dtype=torch.float32, pin_memory=True) for _ in range(E2E_STREAMS)]
    sets = [(D32.empty_state(), D32.empty_state(), D32.empty_state()) for _ in range(E2E_SETS)]
    streams = [torch.cuda.Stream() for _ in range(E2E_STREAMS)]

    def one(i):
        # step i and step i + E2E_SETS share a buffer set and a host output: same stream
        st = streams[i % E2E_STREAMS]
        qi, qo, rr = sets[i % E2E_SETS]
        with torch.cuda.stream(st):
            qi.copy_(h_state, non_blocking=True)
            D32.lserk4_step(qi, qo, rr, t, dt, stream=st.cuda_stream)
            h_out[i % E2E_STREAMS].copy_(qo, non_blocking=True)

    for i in range(4):  # warm-up: the same calls, untimed
        one(i)
    torch.cuda.synchronize()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for st in streams:
        st.wait_stream(stream)
    for i in range(steps):
        one(i)
    for st in streams:
        stream.wait_stream(st)
    e1.record(stream)
    barrier()
    ms = replicas.max_over_ranks(e0.elapsed_time(e1) / steps, device="cuda")
    # serial: one stream, step after step, L2 flushed in between (outside the events)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for it in range(steps):
        flush.fill_(float(it))
        evs[it][0].record(stream)
        bufs[0].copy_(h_state, non_blocking=True)
        D32.lserk4_step(bufs[0], bufs[1], res, t, dt)
        h_out[0].copy_(bufs[1], non_blocking=True)
        evs[it][1].record(stream)
    barrier()
    per = np.array([a.elapsed_time(b) for a, b in evs])
    ms_serial = replicas.max_over_ranks(float(np.mean(per)), device="cuda")
    nbytes = n * 4
    return {"value": replicas.job_throughput(dofs * 5, ms * 1e-3, ws) / 1e9, "unit": UNIT,
            "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes, "ms_per_step": ms,
            "path": "dgc_lserk4_step via ctypes, pinned host state in and out every step, independent steps "
                    f"on {E2E_STREAMS} streams, {E2E_SETS} device buffer sets (inputs larger than L2)",
            "serial": {"value": replicas.job_throughput(dofs * 5, ms_serial * 1e-3, ws) / 1e9,
                       "ms_per_step": ms_serial,
                       "ms_per_step_min_median_max": [float(per.min()), float(np.median(per)),
                                                      float(per.max())],
                       "path": "one stream, step after step, L2 flushed between steps"}}


def measure_fp64(dg, m, q_init, dt, flush, stream, steps, dofs):
    import torch
    D64 = dg.Discretization(m, "maxwell_te", ORDER, dg.F64)
    a, b, r = D64.upload(q_init), D64.empty_state(), D64.empty_state()
    for _ in range(3):
        D64.lserk4_step(a, b, r, 0.0, dt)
        a, b = b, a
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for it in range(steps):
        flush.fill_(float(it))
        evs[it][0].record(stream)
        D64.lserk4_step(a, b, r, 0.0, dt)
        evs[it][1].record(stream)
        a, b = b, a
    torch.cuda.synchronize()
    ms = float(np.mean([x.elapsed_time(y) for x, y in evs]))
    D64.check()
    return D64, {"value": dofs * 5 / (ms * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": ms, "steps": steps}


def measure_fp32c(dg, m, q_init, dt, flush, stream, steps, dofs):
    """The workload with the compensated FP32 state (DGC_F32C): per-step time of
    the 5 stage launches (L2 flushed before each step), GDOF/s and the stage
    kernel's roofline.  Algorithmic bytes per element: hi and lo state read and
    written, residual read and written (6 Nf Np x 4 B) + 14 FP32 geometric
    factors + 3 int32 neighbours."""
    import torch
    D = dg.Discretization(m, "maxwell_te", ORDER, dg.F32C)
    a, b, r = D.upload(q_init), D.empty_state(), D.empty_state()
    for _ in range(3):
        D.lserk4_step(a, b, r, 0.0, dt)
        a, b = b, a
    # events at the step boundaries only: the five launches of a step run back
    # to back, each overlapping its set-up with the previous one's end
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(steps)]
    for it in range(steps):
        flush.fill_(float(it))
        evs[it][0].record(stream)
        for st in range(5):
            D.lserk4_stage(st, a if st % 2 == 0 else b, b if st % 2 == 0 else a, r, 0.0, dt)
        evs[it][1].record(stream)
        a, b = b, a
    torch.cuda.synchronize()
    D.check()
    step_ms = float(np.mean([e[0].elapsed_time(e[1]) for e in evs]))
    stage_ms = step_ms / 5
    elem_bytes = 6 * 3 * D.Np * 4 + 14 * 4 + 3 * 4
    peak, peak_kind = measured_peak()
    achieved = elem_bytes * D.K / (stage_ms * 1e-3) / 1e9
    return {"value": dofs * 5 / (step_ms * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": step_ms, "steps": steps,
            "kernel": "dgk::dg_rhs_x2_kernel<6,PHYS_TE> (LSERK4 stage)",
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind, "launch_ms": stage_ms,
                         "alg_bytes_per_element": elem_bytes, "alg_bytes_per_launch": elem_bytes * D.K,
                         "traffic": read_traffic("x2")}}


def measure_accuracy(dg, D32, D64, q_init, x, y, dt):
    """Both precisions from the same initial data to T = 1 (graph-replayed
    LSERK4); relative L2 errors against the exact cavity mode and each other."""
    import torch
    nsteps = int(np.ceil(1.0 / dt))
    dtT = 1.0 / nsteps
    t0 = time.perf_counter()
    f32 = D32.lserk4_run(D32.upload(q_init), D32.empty_state(), D32.empty_state(), 0.0, dtT, nsteps, graph=True)
    torch.cuda.synchronize()
    t32 = time.perf_counter() - t0
    t0 = time.perf_counter()
    f64 = D64.lserk4_run(D64.upload(q_init), D64.empty_state(), D64.empty_state(), 0.0, dtT, nsteps, graph=True)
    torch.cuda.synchronize()
    t64 = time.perf_counter() - t0
    ex = te_exact(x, y, 1.0).reshape(-1)
    u32, u64 = D32.download(f32), D64.download(f64)
    nrm = np.linalg.norm(ex)
    return {"T": 1.0, "steps": nsteps, "rel_l2_fp32_vs_exact": float(np.linalg.norm(u32 - ex) / nrm),
            "rel_l2_fp64_vs_exact": float(np.linalg.norm(u64 - ex) / nrm),
            "rel_l2_fp32_vs_fp64": float(np.linalg.norm(u32 - u64) / np.linalg.norm(u64)),
            "fp32_run_s": t32, "fp64_run_s": t64}


def measure_advection(dg, meshes):
    """The advection workload: jittered 32x32 mesh (K = 2048), N = 4, a = (1, 0.5),
    Gaussian pulse exp(-((x+0.3)^2 + y^2)/0.02) with its exact translation as
    inflow data, LSERK4 with dt = 0.5 min(h) / ((N+1)^2 |a|) to T = 0.5.  The L2
    error against the exact pulse from the GPU (FP64 and compensated FP32,
    graphed runs, device time of the whole run) and from the oracle (the serial
    C port of the reference CPU operator, FP64, host time)."""
    import torch
    import oracle
    N, T, ax, ay = 4, 0.5, 1.0, 0.5
    m = meshes.jittered_square(32, SEED)
    o = oracle.Oracle(m.xy, m.cells, N)
    p = oracle.problem(oracle.ADVECTION, ax, ay, oracle.BC_GAUSS)
    q0, ex = o.exact(p, 0.0), o.exact(p, T)
    out = {"workload": "advection_gauss_k2048_n4_lserk4_t0.5", "num_cells": int(m.cells.shape[0]), "order": N}
    stream = torch.cuda.current_stream()
    for tag, prec in (("fp64", dg.F64), ("fp32c", dg.F32C)):
        D = dg.Discretization(m, "advection", N, prec, ax=ax, ay=ay, bc=dg.BC_GAUSS)
        dt0 = 0.5 * D.info.min_edge / ((N + 1) ** 2 * np.hypot(ax, ay))
        ns = int(np.ceil(T / dt0))
        qa, qb, r = D.upload(q0), D.empty_state(), D.empty_state()
        D.lserk4_run(qa, qb, r, 0.0, T / ns, 20, graph=True)            # warm-up, graph capture
        qa.copy_(D.upload(q0))
        r.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fin = D.lserk4_run(qa, qb, r, 0.0, T / ns, ns, graph=True)
        e1.record(stream)
        torch.cuda.synchronize()
        D.check()
        ms = e0.elapsed_time(e1)
        out["steps"] = ns
        out[tag] = {"rel_l2_vs_exact": float(np.linalg.norm(D.download(fin) - ex) / np.linalg.norm(ex)),
                    "ms_to_t": ms, "gdofs": D.Np * D.K * 5 * ns / (ms * 1e-3) / 1e9}
    t0 = time.perf_counter()
    qo, _ = o.run(p, 1, 0.0, T / out["steps"], out["steps"], q0)   # scheme 1: LSERK4
    cpu_s = time.perf_counter() - t0
    out["oracle_cpu"] = {"rel_l2_vs_exact": float(np.linalg.norm(qo - ex) / np.linalg.norm(ex)), "seconds": cpu_s,
                         "cores": 1}
    return out


EQ_MESHES = (16, 32, 64, 128)
EQ_ORDERS = (2, 3, 4, 5, 6)
EQ_TARGETS = (1e-4, 1e-5, 1e-6, 1e-7)


def measure_equal_error(dg, meshes):
    """Accuracy against time for the TE cavity to T = 1: every (mesh, order) of
    EQ_MESHES x EQ_ORDERS in FP64, FP32 and compensated FP32 (FP32 arithmetic,
    hi + lo state), graph-replayed LSERK4 with dt = 0.5 min(edge) / (N+1)^2,
    device time of the whole run (CUDA events), relative L2 error against the
    exact mode.  Two comparisons at equal error:
      * per configuration: where a mixed path's error equals FP64's (within 5 %),
        the ratio of their GDOF/s on that configuration;
      * per target error E: the fastest configuration of each precision whose
        error is <= E, and the ratio of their times to solution."""
    import torch
    stream = torch.cuda.current_stream()
    rows = []
    for n in EQ_MESHES:
        m = meshes.jittered_square(n, SEED)
        for N in EQ_ORDERS:
            row = {"n": n, "num_cells": 2 * n * n, "order": N}
            for tag, prec in (("fp64", dg.F64), ("fp32", dg.F32), ("fp32c", dg.F32C)):
                D = dg.Discretization(m, "maxwell_te", N, prec)
                variant = D.autotune(reps=5)[0] if prec == dg.F32 else None
                x, y = D.node_xy()
                dt0 = 0.5 * D.info.min_edge / (N + 1) ** 2
                ns = int(np.ceil(1.0 / dt0))
                qa, qb, res = D.upload(te_initial(x, y)), D.empty_state(), D.empty_state()
                D.lserk4_run(qa, qb, res, 0.0, 1.0 / ns, 20, graph=True)     # warm-up, graph capture
                qa.copy_(D.upload(te_initial(x, y)))                           # same buffers: the graph is reused
                res.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fin = D.lserk4_run(qa, qb, res, 0.0, 1.0 / ns, ns, graph=True)
                e1.record(stream)
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1)
                D.check()
                ex = te_exact(x, y, 1.0).reshape(-1)
                err = float(np.linalg.norm(D.download(fin) - ex) / np.linalg.norm(ex))
                row["steps"] = ns
                row[tag] = {"rel_l2": err, "ms_to_t1": ms,
                            "gdofs": 3 * D.Np * D.K * 5 * ns / (ms * 1e-3) / 1e9}
                if variant is not None:
                    row[tag]["variant"] = variant
                del D, qa, qb, res, fin
            rows.append(row)
    same = []
    for r in rows:
        for tag in ("fp32", "fp32c"):
            if abs(r[tag]["rel_l2"] - r["fp64"]["rel_l2"]) <= 0.05 * r["fp64"]["rel_l2"]:
                same.append({"n": r["n"], "order": r["order"], "precision": tag, "rel_l2": r[tag]["rel_l2"],
                             "gdofs": r[tag]["gdofs"], "fp64_gdofs": r["fp64"]["gdofs"],
                             "speedup": r[tag]["gdofs"] / r["fp64"]["gdofs"]})
    best = {}
    for tag in ("fp64", "fp32", "fp32c"):
        floor = min(r[tag]["rel_l2"] for r in rows)
        best[tag + "_min_error"] = floor
    targets = list(EQ_TARGETS) + [best["fp32c_min_error"] * 1.05]
    frontier = []
    for E in targets:
        ent = {"target_rel_l2": E}
        for tag in ("fp64", "fp32", "fp32c"):
            ok = [r for r in rows if r[tag]["rel_l2"] <= E]
            if ok:
                b = min(ok, key=lambda r: r[tag]["ms_to_t1"])
                ent[tag] = {"n": b["n"], "order": b["order"], "ms_to_t1": b[tag]["ms_to_t1"],
                            "rel_l2": b[tag]["rel_l2"]}
        for tag in ("fp32", "fp32c"):
            if tag in ent and "fp64" in ent:
                ent["speedup_" + tag] = ent["fp64"]["ms_to_t1"] / ent[tag]["ms_to_t1"]
        frontier.append(ent)
    return {"workload": "maxwell_te_pec_cavity to T=1, jittered n x n meshes, LSERK4",
            "meshes": list(EQ_MESHES), "orders": list(EQ_ORDERS), "rows": rows,
            "same_error_configs": same, "min_error": best, "time_to_error": frontier}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 plain-path timing")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end (host buffer) timing")
    ap.add_argument("--variant", type=int, default=-1, help="force an RHS kernel variant instead of autotuning")
    ap.add_argument("--no-poisson", action="store_true", help="skip the IPDG Poisson solver comparison")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-instances comparison")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-preconditioner comparison")
    ap.add_argument("--no-stokes", action="store_true", help="skip the Stokes dual-splitting timing")
    ap.add_argument("--no-advection", action="store_true", help="skip the advection (K = 2048) accuracy line")
    ap.add_argument("--no-equal-error", action="store_true", help="skip the accuracy-against-time sweep")
    ap.add_argument("--learned-activation", default="relu", choices=["relu", "linear"],
                    help="hidden-layer activation of the learned preconditioner's network")
    ap.add_argument("--learned-correction", default="additive", choices=["additive", "residual"],
                    help="where the learned preconditioner's network acts: on r, or on r - S z0")
    ap.add_argument("--learned-full", action="store_true",
                    help="run only the learned-preconditioner workload over its whole 1600 / 400 sequence "
                         "(about a quarter of an hour) and print its section as one JSON line")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.learned_full:
        import torch
        import dgc_gb300 as dg
        from dgc_gb300 import meshes
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        out = measure_learned(dg, meshes, n_train=LEARN_TRAIN, n_held=LEARN_HELD, n_fp64=40,
                              snapshots=(4, 16, 64), full=True, activation=args.learned_activation,
                              correction=args.learned_correction)
        print(json.dumps({"learned_precond_full": out}))
        return None

    import torch
    import dgc_gb300 as dg
    from dgc_gb300 import meshes, replicas

    ws, rank, local = dist_env()
    # host threads and pinned buffers next to this rank's GPU: the e2e copies then
    # take the GPU's own CPU link instead of crossing between sockets
    bound = replicas.bind_local_cpus(local)
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")

    def barrier():
        if ws > 1:
            import torch.distributed as tdist
            tdist.barrier()
        torch.cuda.synchronize()

    m = meshes.jittered_square(NSIDE, SEED)
    D32 = dg.Discretization(m, "maxwell_te", ORDER, dg.F32)
    if args.variant >= 0:
        D32.set_variant(args.variant)
        tuned, tune_ms = args.variant, None
    else:
        tuned, tune_ms = D32.autotune(reps=10)
    K, Np = D32.K, D32.Np
    x, y = D32.node_xy()
    q_init = te_initial(x, y)
    dt = 0.5 * D32.info.min_edge / (ORDER + 1) ** 2
    dofs = 3 * Np * K
    stream = torch.cuda.current_stream()
    qa = D32.upload(q_init)
    qb, res = D32.empty_state(), D32.empty_state()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step_stages(bufs, t, evs=None):
        for s in range(5):
            D32.lserk4_stage(s, bufs[s & 1], bufs[(s + 1) & 1], res, t, dt)
            if evs is not None:
                evs[s + 1].record(stream)

    bufs = [qa, qb]
    t = 0.0
    for _ in range(args.warmup):
        step_stages(bufs, t)
        bufs.reverse()
        t += dt
    barrier()
    sampler = ClockSampler(local)
    sampler.start()
    launches0 = D32.launch_count()
    # events at the step boundaries only: the five launches of a step run back
    # to back, each overlapping its set-up with the previous one's end
    events = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(args.steps)]
    wall0 = time.perf_counter()
    for it in range(args.steps):
        flush.fill_(float(it))
        events[it][0].record(stream)
        step_stages(bufs, t)
        events[it][1].record(stream)
        bufs.reverse()
        t += dt
    barrier()
    wall = time.perf_counter() - wall0
    launches = D32.launch_count() - launches0
    clocks = sampler.stop()
    step_ms = np.array([events[i][0].elapsed_time(events[i][1]) for i in range(args.steps)])
    # per-stage breakdown from separate steps with an event after every launch
    # (stage 1 reads the flushed state from DRAM, stages 2-5 find it in L2)
    nb = min(args.steps, 5)
    sevents = [[torch.cuda.Event(enable_timing=True) for _ in range(6)] for _ in range(nb)]
    for it in range(nb):
        flush.fill_(float(it))
        sevents[it][0].record(stream)
        step_stages(bufs, t, sevents[it])
        bufs.reverse()
        t += dt
    torch.cuda.synchronize()
    stage_ms = np.array([[sevents[i][s].elapsed_time(sevents[i][s + 1]) for s in range(5)] for i in range(nb)])
    D32.check()
    # replicas: every rank advances its own copy; slowest rank's time, all ranks' work
    my_ms = replicas.max_over_ranks(float(step_ms.mean()), device="cuda")
    value = replicas.job_throughput(dofs * 5, my_ms * 1e-3, ws) / 1e9

    # roofline of the dominant kernel (the fused RHS + LSERK4 stage): compulsory
    # bytes per element = read q, read res, write res, write q (3 fields x Np x 4 B
    # each) + 14 FP32 geometric factors + 3 int32 neighbour indices
    alg_bytes_elem = 4 * 3 * Np * 4 + 14 * 4 + 3 * 4
    alg_bytes = alg_bytes_elem * K
    launch_ms = float(step_ms.mean()) / 5
    achieved = alg_bytes / (launch_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": read_traffic(tuned), "peak_source": peak_kind,
                "kernel": STAGE_KERNELS.get(tuned, "variant %s" % tuned) + " (LSERK4 stage)",
                "alg_bytes_per_launch": alg_bytes, "alg_bytes_per_element": alg_bytes_elem,
                "launch_ms": launch_ms, "launch_ms_basis": "step time / 5 back-to-back launches",
                "stage_ms": [float(v) for v in stage_ms.mean(axis=0)],
                "tile": {"variant": tuned, "elements_per_tile": D32.info.rhs_tile,
                         "threads": D32.info.rhs_threads, "smem_bytes": D32.info.rhs_smem,
                         "ctas_per_sm": D32.info.rhs_blocks_per_sm, "autotune_ms": tune_ms}}

    e2e = None if args.no_e2e else measure_e2e(D32, bufs, res, flush, stream, t, dt, args.steps, ws, dofs, barrier)
    if e2e is not None:
        e2e["host_cpus"] = (f"{len(bound)} CPUs of the GPU's NUMA node ({bound[0]}-{bound[-1]})" if bound
                            else "unbound (GPU NUMA node not found)")
    D64, fp64 = (None, None) if args.no_fp64 else measure_fp64(dg, m, q_init, dt, flush, stream,
                                                                max(3, min(args.steps, 10)), dofs)
    fp32c = None if args.no_fp64 else measure_fp32c(dg, m, q_init, dt, flush, stream,
                                                    max(3, min(args.steps, 10)), dofs)
    equal_error = None
    if rank == 0 and not args.no_equal_error:
        equal_error = measure_equal_error(dg, meshes)
    accuracy = None
    if rank == 0 and equal_error is not None and not args.no_accuracy:
        # the sweep's run of this very workload (mesh, order, dt rule, T = 1)
        row = next(r for r in equal_error["rows"] if r["n"] == NSIDE and r["order"] == ORDER)
        accuracy = {"T": 1.0, "steps": row["steps"], "from": "equal_error sweep, same mesh / order / dt",
                    "rel_l2_fp32_vs_exact": row["fp32"]["rel_l2"], "rel_l2_fp64_vs_exact": row["fp64"]["rel_l2"],
                    "rel_l2_fp32c_vs_exact": row["fp32c"]["rel_l2"],
                    "gdofs_graphed_run": {k: row[k]["gdofs"] for k in ("fp64", "fp32", "fp32c")}}
    elif rank == 0 and D64 is not None and not args.no_accuracy:
        accuracy = measure_accuracy(dg, D32, D64, q_init, x, y, dt)
    poisson = None
    if rank == 0 and not args.no_poisson:
        poisson = measure_poisson(dg, meshes)
    batched = None
    if rank == 0 and not args.no_batched:
        batched = measure_batched(dg, meshes)
        if ws == 1 and not args.no_cpu_baseline:
            batched["cpu_baseline"] = cpu_batched_baseline()
    learned = None
    if rank == 0 and not args.no_learned:
        learned = measure_learned(dg, meshes, activation=args.learned_activation,
                                  correction=args.learned_correction)
    advection = None
    if rank == 0 and not args.no_advection:
        advection = measure_advection(dg, meshes)
    stokes = None
    if rank == 0 and not args.no_stokes:
        stokes = measure_stokes(dg, meshes)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        csteps = 10
        cg, csec = oracle_sample(csteps, 1)
        cpu = {"value": cg, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"{csteps} full LSERK4 steps of the workload (serial C port of the reference CPU "
                         f"operator, FP64, {csec:.2f} s/step), host {cpu_model()}"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": my_ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config_dict(ws),
                "e2e": e2e, "gpu_launches": int(launches), "roofline": roofline, "cpu_baseline": cpu,
                "clocks": clocks, "fp64_plain": fp64, "fp32c": fp32c,
                "speedup_mixed_vs_fp64": (value / ws / fp64["value"]) if fp64 else None,
                "accuracy": accuracy, "poisson": poisson, "batched": batched, "learned_precond": learned,
                "stokes": stokes, "advection": advection, "equal_error": equal_error, "wall_s_timed_region": wall}
        print(json.dumps(line))
    if ws > 1:
        import torch.distributed as tdist
        tdist.destroy_process_group()


if __name__ == "__main__":
    main()
