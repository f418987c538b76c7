"""The round-off model behind the compensated FP32 stage kernel (DGC_F32C),
checked with a NumPy emulation of FP32 arithmetic on the CPU (no GPU needed).

A Maxwell TE cavity run (jittered 12x12 mesh, N = 4, LSERK4 to T = 0.5) is
integrated four ways, every operation of the three FP32 variants rounded to
float32, and compared with the FP64 run of the same scheme:

  fp32       the weak form with a plain FP32 state (what DGC_F32 computes);
  x2         the strong form, surface terms from hi/lo jumps, volume term on
             hi - c, compensated state update (what dg_rhs_x2_kernel computes);
  x2_geo64   the same with the geometric factors kept in FP64.

The x2 arrangement lands an order of magnitude closer to the FP64 run, and
keeping the geometry in FP64 changes its error by less than a quarter: the
FP32 geometry records are not what limits the mixed path's accuracy.
"""
import numpy as np

from conftest import oracle
from dgc_gb300 import meshes

F32 = np.float32


def setup(n=12, N=4, seed=2026):
    m = meshes.jittered_square(n, seed)
    o = oracle.Oracle(m.xy, m.cells, N)
    K, Np, Nfp = o.K, o.Np, o.Nfp
    A = o.arrays()
    Drw, Dsw, Lw, _ = oracle.operators(N, oracle.WEAK)
    Drs, Dss, Ls, _ = oracle.operators(N, oracle.STRONG)
    fm = oracle.face_nodes(N)
    inv = A["invJ"].reshape(K, 4)
    g = dict(rx=inv[:, :1], ry=inv[:, 1:2], sx=inv[:, 2:3], sy=inv[:, 3:4],
             sc=-np.repeat(A["faceJ"].reshape(K, 3), Nfp, 1) / A["J"][:, None],
             nx=np.repeat(A["nx"].reshape(K, 3), Nfp, 1), ny=np.repeat(A["ny"].reshape(K, 3), Nfp, 1))
    nbc, nbf = A["nbCell"].reshape(K, 3), A["nbFace"].reshape(K, 3)
    bnd = nbc == np.arange(K)[:, None]
    nbf = np.where(bnd, 0, nbf)
    own = np.concatenate(fm)
    cell = np.repeat(nbc, Nfp, 1)
    node = np.stack([np.array(fm)[nbf[:, f], Nfp - 1 - d] for f in range(3) for d in range(Nfp)], 1)
    ops = dict(Drw=Drw, Dsw=Dsw, Lw=Lw, Drs=Drs, Dss=Dss, Ls=Ls)
    return m, o, dict(g=g, ops=ops, own=own, cell=cell, node=node, bnd=np.repeat(bnd, Nfp, 1), K=K, Np=Np)


def traces(q, t):
    a = q[:, :, t["own"]]
    b = q[:, t["cell"], t["node"]]
    return a, np.where(t["bnd"][None], np.stack([-a[0], -a[1], a[2]]), b)  # PEC: E+ = -E-, Hz+ = Hz-


def rhs_weak(q, t, dtype):
    c = lambda x: np.asarray(x, dtype=dtype)  # noqa: E731
    g, ops = t["g"], t["ops"]
    a, b = traces(q, t)
    nx, ny, h = c(g["nx"]), c(g["ny"]), dtype(0.5)
    w = (a[2] + b[2]) - ny * (a[0] - b[0]) + nx * (a[1] - b[1])
    f = [-h * ny * w, h * nx * w, h * (nx * (a[1] + b[1]) - ny * (a[0] + b[0]) + a[2] - b[2])]
    L, sc = c(ops["Lw"].T), c(g["sc"])
    ur, us = q @ c(ops["Drw"].T), q @ c(ops["Dsw"].T)
    rx, ry, sx, sy = (c(g[k]) for k in ("rx", "ry", "sx", "sy"))
    vol = [-(ry * ur[2] + sy * us[2]), rx * ur[2] + sx * us[2], (rx * ur[1] + sx * us[1]) - (ry * ur[0] + sy * us[0])]
    return np.stack([v + (fi * sc) @ L for v, fi in zip(vol, f)])


def rhs_x2(hi, lo, t, geo64=False):
    c = lambda x: np.asarray(x, dtype=F32)  # noqa: E731
    gc = (lambda x: x) if geo64 else c
    g, ops = t["g"], t["ops"]
    ah, bh = traces(hi, t)
    al, bl = traces(lo, t)
    d = (bh - ah) + (bl - al)
    nx, ny, h = c(g["nx"]), c(g["ny"]), F32(0.5)
    w = d[2] + ny * d[0] - nx * d[1]
    f = [-h * ny * w, h * nx * w, h * (nx * d[1] - ny * d[0] - d[2])]
    L, sc = c(ops["Ls"].T), gc(g["sc"])
    qv = hi - hi[:, :, :1]
    rx, ry, sx, sy = (gc(g[k]) for k in ("rx", "ry", "sx", "sy"))
    Dr, Ds = c(ops["Drs"].T), c(ops["Dss"].T)
    ur, us = qv[2] @ Dr, qv[2] @ Ds
    # the curl term as one product pair: Dr (ry Ex - rx Ey) + Ds (sy Ex - sx Ey)
    u, w = (ry * qv[0] - rx * qv[1]).astype(F32), (sy * qv[0] - sx * qv[1]).astype(F32)
    vol = [ry * ur + sy * us, -(rx * ur + sx * us), u @ Dr + w @ Ds]
    return np.stack([(v + (fi * sc) @ L).astype(F32) for v, fi in zip(vol, f)])


def two_sum_update(hi, lo, d):
    s = hi + d
    bb = s - hi
    e = (hi - (s - bb)) + (d - bb)
    lo = lo + e
    h2 = s + lo
    return h2, lo - (h2 - s)


def run(kind, q0, t, ns, dt):
    a, b, _ = oracle.lserk4_coeffs()
    if kind == "fp64":
        q, r = q0.copy(), np.zeros_like(q0)
        for _ in range(ns):
            for k in range(5):
                r = a[k] * r + dt * rhs_weak(q, t, np.float64)
                q = q + b[k] * r
        return q
    A, B, D = [F32(v) for v in a], [F32(v) for v in b], F32(dt)
    if kind == "fp32":
        q, r = q0.astype(F32), np.zeros(q0.shape, F32)
        for _ in range(ns):
            for k in range(5):
                r = A[k] * r + D * rhs_weak(q, t, F32)
                q = q + B[k] * r
        return q.astype(np.float64)
    hi = q0.astype(F32)
    lo = (q0 - hi).astype(F32)
    r = np.zeros(q0.shape, F32)
    for _ in range(ns):
        for k in range(5):
            r = A[k] * r + D * rhs_x2(hi, lo, t, geo64=kind == "x2_geo64")
            hi, lo = two_sum_update(hi, lo, B[k] * r)
    return hi.astype(np.float64) + lo.astype(np.float64)


def test_emulated_round_off_of_the_mixed_arrangements():
    m, o, t = setup()
    p = oracle.problem(oracle.MAXWELL_TE)
    q0 = o.exact(p, 0.0).reshape(3, t["K"], t["Np"])
    # the emulation's FP64 operator is the oracle's
    ref = o.rhs(p, 0.0, q0.reshape(-1)).reshape(q0.shape)
    assert np.linalg.norm(rhs_weak(q0, t, np.float64) - ref) < 1e-12 * np.linalg.norm(ref)
    dt0 = 0.5 * meshes.min_edge_length(m) / 25.0
    ns = int(np.ceil(0.5 / dt0))
    dt = 0.5 / ns
    out = {k: run(k, q0, t, ns, dt) for k in ("fp64", "fp32", "x2", "x2_geo64")}
    err = {k: np.linalg.norm(out[k] - out["fp64"]) / np.linalg.norm(out["fp64"]) for k in out}
    assert err["x2"] < err["fp32"] / 5, err
    assert abs(err["x2_geo64"] - err["x2"]) < 0.25 * err["x2"], err
