"""CPU restatement of the Stokes example's dual-splitting step
(examples/stokes_2d/stokes_2d.h), built on the C oracle's div_2d, grad_2d and
laplace_2d pieces (each pinned against the reference's own outputs).

TEST INFRASTRUCTURE ONLY: the checker of the GPU step in tests/.  The product
never imports this module.

The systems are assembled column by column from apply_homogeneous and solved
densely, as stokes_2d::build_poisson_sys_matrix / build_helmholtz_sys_matrix /
solve_sys do (stokes_2d.h:424-526, which factor with a sparse LU).  The one
departure: the all-Neumann pressure matrix is singular and the right-hand side
only nearly consistent, which the reference leaves to the LU's pivoting; here
(as in the GPU step) the SPD form S = -J M A is solved with -J M rhs projected
to zero sum, and p returned with zero mean.

State vectors: reference CPU layout [cell][node], float64.
"""
from __future__ import annotations

import numpy as np

from oracle import Oracle, face_nodes, operators, STRONG

# the example problem (stokes_2d.h:103-104)
A = 2.883356
LAMBDA = 1.0 + A * A


def gx_fn(x, y):
    """x velocity without the time factor (stokes_2d.h:165-166)."""
    return np.sin(x) * (A * np.sin(A * y) - np.cos(A) * np.sinh(y))


def gy_fn(x, y):
    return np.cos(x) * (np.cos(A * y) + np.cos(A) * np.cosh(y))


def exact(x, y, t):
    """exact_solution (stokes_2d.h:313-340)."""
    e = np.exp(-LAMBDA * t)
    return gx_fn(x, y) * e, gy_fn(x, y) * e


def boundary_data(bx, by, t, t_prev, dt):
    """The example's boundary objects at boundary nodes (bx, by) for the step
    t -> t + dt (stokes_2d.h:108-188, 245-247): u_tilde_bc exterior_val(x, y, 0),
    the dgdt terms of pressure_bc's hp, u_x_bc / u_y_bc exterior_val(x, y, 0)."""
    gx, gy = gx_fn(bx, by), gy_fn(bx, by)
    e_t, e_p, e_n = np.exp(-LAMBDA * t), np.exp(-LAMBDA * t_prev), np.exp(-LAMBDA * (t + dt))
    return dict(ut_x=2.0 * (4.0 * gx * e_t - gx * e_p) / 3.0,
                ut_y=2.0 * (4.0 * gy * e_t - gy * e_p) / 3.0,
                dgdt_x=LAMBDA * gx * e_n, dgdt_y=LAMBDA * gy * e_n,
                g_x=2.0 * gx * e_n, g_y=2.0 * gy * e_n)


class StokesOracle:
    """Dense-matrix dual-splitting step on one mesh and order (tau = 1).

    consistent=False takes the Dirichlet data of the viscous systems as
    apply_inhomogeneous_as_rhs forms them (the reference); True adds the jumps
    of the lifted data it leaves out (Oracle.laplace_bc_rhs)."""

    def __init__(self, xy, cells, N, consistent: bool = False):
        self.o = Oracle(xy, cells, N)
        self.consistent = consistent
        self.N, self.K, self.Np, self.Nfp = N, self.o.K, self.o.Np, self.o.Nfp
        self.arr = self.o.arrays()
        n = self.K * self.Np
        nb = self.arr["bx"].size
        self.nb = nb
        eye = np.eye(n)
        # apply_homogeneous columns (build_*_sys_matrix)
        self.A_D = np.stack([self.o.laplace(eye[i], dirichlet=True) for i in range(n)], axis=1)
        self.A_N = np.stack([self.o.laplace(eye[i], dirichlet=False) for i in range(n)], axis=1)
        self.JM = np.stack([self.o.mass(eye[i]) for i in range(n)], axis=1)
        Dr, Ds, _, _ = operators(N, STRONG)
        self.Dr, self.Ds = Dr, Ds
        self.fn = face_nodes(N)
        self.bxy = np.stack([self.arr["bx"], self.arr["by"]], axis=1)

    def hp(self, ux0, uy0, ux1, uy1, dgdt_x, dgdt_y):
        """pressure_bc's hp per boundary node (stokes_2d.h:191-269); u0 = u^(n-1), u1 = u^n."""
        K, Np = self.K, self.Np
        invJ = self.arr["invJ"].reshape(K, 4)
        nx, ny = self.arr["nx"].reshape(K, 3), self.arr["ny"].reshape(K, 3)
        out = []
        b = 0
        for c in range(K):
            faces = [f for f in range(3) if self._is_boundary(c, f)]
            if not faces:
                continue
            Dx = self.Dr * invJ[c, 0] + self.Ds * invJ[c, 2]
            Dy = self.Dr * invJ[c, 1] + self.Ds * invJ[c, 3]
            s = slice(c * Np, (c + 1) * Np)
            curl_n = Dx @ uy1[s] - Dy @ ux1[s]
            curl_p = Dx @ uy0[s] - Dy @ ux0[s]
            ccx = Dy @ curl_p - 2.0 * (Dy @ curl_n)
            ccy = -(Dx @ curl_p) + 2.0 * (Dx @ curl_n)
            for f in faces:
                for i in range(self.Nfp):
                    j = self.fn[f][i]
                    out.append(dgdt_x[b] * nx[c, f] + dgdt_y[b] * ny[c, f] + ccx[j] * nx[c, f] + ccy[j] * ny[c, f])
                    b += 1
        return np.array(out)

    def _is_boundary(self, c, f):
        return self.arr["nbCell"].reshape(self.K, 3)[c, f] == c

    def step(self, ux0, uy0, ux1, uy1, dt, bc):
        """advance_timestep (stokes_2d.h:393-423): returns (ux, uy, p)."""
        n = self.K * self.Np
        utx = (ux1 * 4.0 - ux0) / 3.0
        uty = (uy1 * 4.0 - uy0) / 3.0
        # pressure step
        hp = self.hp(ux0, uy0, ux1, uy1, bc["dgdt_x"], bc["dgdt_y"])
        w = self.o.div(utx, uty, bc["ut_x"], bc["ut_y"], -1.0) * (1.5 / dt)
        w = self.o.laplace_bc_rhs(np.zeros(self.nb, np.uint8), None, 2.0 * hp, out=w)
        S = -self.JM @ self.A_N
        b = -self.JM @ w
        b = b - b.mean()
        p = np.linalg.lstsq(S, b, rcond=None)[0]
        p = p - p.mean()
        # projection step
        gpx, gpy = self.o.grad(p, None, 1.0)
        utx = utx - 2.0 * dt * gpx / 3.0
        uty = uty - 2.0 * dt * gpy / 3.0
        # viscous step
        H = self.A_D - (1.5 / dt) * np.eye(n)
        out = []
        for ut, g in ((utx, bc["g_x"]), (uty, bc["g_y"])):
            w = -1.5 * ut / dt
            w = self.o.laplace_bc_rhs(np.ones(self.nb, np.uint8), g, None, out=w, consistent=self.consistent)
            out.append(np.linalg.solve(H, w))
        return out[0], out[1], p

    def run(self, T=0.1, dt=0.001):
        """The example driver's loop (examples/stokes_2d/main.cpp:150-190):
        returns (ux, uy, t, error norm)."""
        x, y = self.o.node_xy()
        x, y = x.reshape(-1), y.reshape(-1)
        ux1, uy1 = exact(x, y, 0.0)
        ux0, uy0 = ux1.copy(), uy1.copy()
        t_prev = t = 0.0
        bx, by = self.arr["bx"], self.arr["by"]
        while t < T:
            if t + dt > T:
                dt = T - t
            ux, uy, _ = self.step(ux0, uy0, ux1, uy1, dt, boundary_data(bx, by, t, t_prev, dt))
            ux0, uy0, ux1, uy1 = ux1, uy1, ux, uy
            t_prev = t
            t += dt
        rx, ry = exact(x, y, t)
        return ux1, uy1, t, float(np.sum((rx - ux1) ** 2 + (ry - uy1) ** 2) / x.size)
