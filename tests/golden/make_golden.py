"""Regenerate the golden vectors in this folder from the reference's own code.

Builds the reference's USE_CPU_ONLY sources into oracle/_ref/ with the recipe
in oracle/Makefile (needs the reference checkout; run in the development
container, not on the GPU machine), drives them on small meshes and stores what
they compute as compressed .npz files:

  ref_<mesh>_N<order>.npz   reference-element matrices, discretisation arrays,
                            one RHS and 1 / 10 classical-RK4 steps of the
                            advection (a = (1,1)) and TM-Maxwell examples, one
                            laplace_2d apply (homogeneous Dirichlet, tau = 1),
                            grad_2d / div_2d applies, the advection driver's
                            visualisation file, and the MSH text of the mesh
                            (the reference's input file and its exporter's output)
  ref_adv1d_K<K>_N<N>.npz   the 1D advection example: operators, RHS, RK4 states
                            and the driver's error norm
  ref_known_answers.json    mean-square nodal errors of the reference drivers'
                            runs on the reference's coarse mesh (10000 RK4
                            steps of advection, Maxwell to T = 1)
  ref_stokes_jit4_N<N>.npz  two steps of the Stokes example's dual splitting (N = 2, 3, 4)
                            from its exact initial data: everything the
                            reference forms (pressure_bc's hp, right-hand
                            sides, grad p, the projected u~), with the two
                            linear systems (the reference's own assembled
                            matrices) solved densely here in place of its
                            cuSOLVER host LU, which needs a GPU.  The
                            all-Neumann pressure matrix is singular and its
                            right-hand side consistent only to ~1e-4; the
                            reference leaves that to the LU's pivoting, here
                            S = -J M A is solved with -J M rhs projected to zero
                            sum and p taken with zero mean

usage: python tests/golden/make_golden.py [/path/to/reference] [--only stokes]
"""
from __future__ import annotations

import json
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, os.path.join(ROOT, "dg-on-cuda_gb300"))
from dgc_gb300 import meshes  # noqa: E402


def read_dump(path: str) -> dict:
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    i = 0
    while i < len(data):
        (ln,) = struct.unpack_from("<i", data, i); i += 4
        name = data[i:i + ln].decode(); i += ln
        kind, cnt = struct.unpack_from("<iq", data, i); i += 12
        if kind == 0:
            out[name] = np.frombuffer(data, "<f8", cnt, i).copy(); i += 8 * cnt
        else:
            out[name] = np.frombuffer(data, "<i4", cnt, i).copy(); i += 4 * cnt
    return out


def stokes_cases(oracle_dir: str, tmp: str) -> None:
    """Two dual-splitting steps per order on a jittered 4 x 4 mesh (dt = 0.002)."""
    exe = os.path.join(oracle_dir, "_ref", "ref_stokes")
    mesh = meshes.jittered_square(4, seed=7)
    mpath = os.path.join(tmp, "stokes_mesh.bin")
    meshes.write_bin(mesh, mpath)
    a, lam = 2.883356, 1.0 + 2.883356 ** 2   # stokes_2d.h:103-104

    def probe(N, t_prev, t, dt, u, p=None):
        spath, opath = os.path.join(tmp, "state.bin"), os.path.join(tmp, "stokes_out.bin")
        with open(spath, "wb") as f:
            f.write(struct.pack("<dddi", t_prev, t, dt, 0 if p is None else 1))
            for v in list(u) + ([] if p is None else [p]):
                f.write(np.ascontiguousarray(v, dtype="<f8").tobytes())
        subprocess.run([exe, mpath, str(N), spath, opath], check=True)
        return read_dump(opath)

    for N in (2, 3, 4):
        Np = (N + 1) * (N + 2) // 2
        n = mesh.cells.shape[0] * Np
        d0 = probe(N, 0.0, 0.0, 1.0, [np.zeros(n)] * 4)
        x, y = d0["x"], d0["y"]
        ux = np.sin(x) * (a * np.sin(a * y) - np.cos(a) * np.sinh(y))   # exact_solution at t = 0
        uy = np.cos(x) * (np.cos(a * y) + np.cos(a) * np.cosh(y))
        JM = np.kron(np.diag(d0["J"]), d0["M"].reshape(Np, Np))
        u = [ux, uy, ux.copy(), uy.copy()]
        t_prev = t = 0.0
        dt = 0.002
        out = dict(mesh_xy=mesh.xy.reshape(-1), mesh_cells=mesh.cells.reshape(-1), x=x, y=y, bx=d0["bx"],
                   by=d0["by"], dt=np.array([dt]))
        for k in range(2):
            da = probe(N, t_prev, t, dt, u)
            assert np.array_equal(da["hp2"], 2.0 * da["hp"])
            A = da["A_N"].reshape(n, n)
            S = -JM @ A
            b = -JM @ da["p_rhs"]
            b -= b.mean()
            p = np.linalg.lstsq(S, b, rcond=None)[0]
            p -= p.mean()
            db = probe(N, t_prev, t, dt, u, p)
            H = db["H"].reshape(n, n)
            vx = np.linalg.solve(H, db["v_rhs_x"])
            vy = np.linalg.solve(H, db["v_rhs_y"])
            rec = dict(t_prev=np.array([t_prev]), t=np.array([t]), u0x=u[0], u0y=u[1], u1x=u[2], u1y=u[3],
                       ut_x=da["ut_x"], ut_y=da["ut_y"], hp2=da["hp2"], div_ut=da["div_ut"], p_rhs=da["p_rhs"],
                       p=p, grad_p_x=db["grad_p_x"], grad_p_y=db["grad_p_y"], utp_x=db["utp_x"],
                       utp_y=db["utp_y"], v_rhs_x=db["v_rhs_x"], v_rhs_y=db["v_rhs_y"], ux=vx, uy=vy)
            out.update({f"s{k}_{key}": v for key, v in rec.items()})
            u = [u[2], u[3], vx, vy]
            t_prev, t = t, t + dt
        np.savez_compressed(os.path.join(HERE, f"ref_stokes_jit4_N{N}.npz"), **out)


def main() -> None:
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    only = sys.argv[sys.argv.index("--only") + 1] if "--only" in sys.argv else None
    if only:
        args = [a for a in args if a != only]
    ref = args[0] if args else os.environ.get("DGC_REFERENCE_DIR", "")
    if not ref:
        sys.exit("make_golden.py: name the reference checkout (first argument or DGC_REFERENCE_DIR)")
    oracle_dir = os.path.join(ROOT, "oracle")
    subprocess.run(["make", "-s", "-C", oracle_dir, "ref", f"REF={ref}"], check=True)
    if only == "stokes":
        with tempfile.TemporaryDirectory() as tmp:
            stokes_cases(oracle_dir, tmp)
        print(f"wrote the Stokes golden cases to {HERE}")
        return
    dump = os.path.join(oracle_dir, "_ref", "ref_dump")
    timer = os.path.join(oracle_dir, "_ref", "ref_time")
    cases = []
    with tempfile.TemporaryDirectory() as tmp:
        jit = meshes.jittered_square(4, seed=7)
        jpath = os.path.join(tmp, "jit4.bin")
        meshes.write_bin(jit, jpath)
        for N in range(1, 7):
            cases.append(("jit4", ["--bin", jpath], N))
        coarse = os.path.join(ref, "examples", "square_domain_coarse.msh")
        for N in range(1, 7):
            cases.append(("coarse", ["--msh", coarse], N))
        four = os.path.join(ref, "tests", "square_domain_4cells.msh")
        for N in (1, 2, 3):
            cases.append(("cells4", ["--msh", four], N))
        cases.append(("fine", ["--msh", os.path.join(ref, "examples", "square_domain_fine.msh")], 1))
        coarse_bin = None
        for name, src, N in cases:
            out = os.path.join(tmp, f"{name}_{N}.bin")
            exp = os.path.join(tmp, f"{name}_{N}.msh")
            subprocess.run([dump, *src, str(N), out, exp], check=True)
            d = read_dump(out)
            d["adv_datafile"] = d["adv_datafile"].astype(np.uint8)   # text, one byte per character
            # MSH fixtures: the reference's input file (when there is one) and the
            # reference exporter's output for this mesh, as byte arrays
            d["msh_export"] = np.frombuffer(open(exp, "rb").read(), dtype=np.uint8)
            if src[0] == "--msh":
                d["msh_source"] = np.frombuffer(open(src[1], "rb").read(), dtype=np.uint8)
            np.savez_compressed(os.path.join(HERE, f"ref_{name}_N{N}.npz"), **d)
            if name == "coarse" and coarse_bin is None:
                coarse_bin = os.path.join(tmp, "coarse.bin")
                m = meshes.Mesh(xy=d["mesh_xy"].reshape(-1, 2), cells=d["mesh_cells"].reshape(-1, 3))
                meshes.write_bin(m, coarse_bin)
        # 1D advection (examples/advection_1d): operators, states after 1 / 10
        # steps; K = 512, N = 6 also after the driver's 10000 steps
        adv1d = os.path.join(oracle_dir, "_ref", "ref_adv1d")
        for K1, N1, steps in ((8, 1, 10), (16, 2, 10), (48, 3, 10), (32, 4, 10), (24, 5, 10), (64, 6, 10),
                              (512, 6, 10000)):
            out = os.path.join(tmp, f"adv1d_{K1}_{N1}.bin")
            subprocess.run([adv1d, str(K1), str(N1), out, str(steps)], check=True)
            np.savez_compressed(os.path.join(HERE, f"ref_adv1d_K{K1}_N{N1}.npz"), steps=np.array([steps]),
                                **read_dump(out))
        known = {"advection_10000_steps": {}, "maxwell_T1": {}}
        for N in range(1, 5):
            r = subprocess.run([timer, coarse_bin, str(N), "adv", "10000"], check=True,
                               capture_output=True, text=True)
            known["advection_10000_steps"][str(N)] = json.loads(r.stdout)
        for N in range(1, 7):
            r = subprocess.run([timer, coarse_bin, str(N), "mx", "0", "1.0"], check=True,
                               capture_output=True, text=True)
            known["maxwell_T1"][str(N)] = json.loads(r.stdout)
        for v in known.values():
            for rec in v.values():
                rec.pop("seconds", None)
                rec.pop("gdof_per_s", None)
        with open(os.path.join(HERE, "ref_known_answers.json"), "w") as f:
            json.dump(known, f, indent=1, sort_keys=True)
        stokes_cases(oracle_dir, tmp)
    print(f"wrote {len(cases)} golden cases + known answers to {HERE}")


if __name__ == "__main__":
    main()
