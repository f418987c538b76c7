"""The Stokes example's dual-splitting step on the GPU (dgc_stokes_*) and the
example problem of examples/stokes_2d (analytic velocity and boundary data).

Velocity and pressure are FP64 device tensors in the native layout of the
laplace handles (K x NpP); `velocity_space` / `pressure_space` give layout
conversion, node coordinates and boundary nodes.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import (BC_DATA_CONSISTENT, BC_DATA_REFERENCE, LAYOUT_REF_CPU, SOLVE_MIXED_IR, Discretization, SolveOpts,
               SolveStats, _check, _ptr, _stream, _vp, lib)

# the example problem (examples/stokes_2d/stokes_2d.h:103-104)
A = 2.883356
LAMBDA = 1.0 + A * A


def _gx(x, y):
    return np.sin(x) * (A * np.sin(A * y) - np.cos(A) * np.sinh(y))


def _gy(x, y):
    return np.cos(x) * (np.cos(A * y) + np.cos(A) * np.cosh(y))


def exact_velocity(x, y, t):
    """stokes_2d::exact_solution (stokes_2d.h:313-340)."""
    e = np.exp(-LAMBDA * t)
    return _gx(x, y) * e, _gy(x, y) * e


def example_boundary_data(bx, by, t, t_prev, dt):
    """The example's boundary objects at the boundary nodes for the step
    t -> t + dt: u_tilde_bc and u_x_bc / u_y_bc exterior_val(x, y, 0), and the
    dgdt terms of pressure_bc's hp (stokes_2d.h:108-188, 245-248)."""
    gx, gy = _gx(bx, by), _gy(bx, by)
    e_t, e_p, e_n = np.exp(-LAMBDA * t), np.exp(-LAMBDA * t_prev), np.exp(-LAMBDA * (t + dt))
    return dict(ut_x=2.0 * (4.0 * gx * e_t - gx * e_p) / 3.0, ut_y=2.0 * (4.0 * gy * e_t - gy * e_p) / 3.0,
                dgdt_x=LAMBDA * gx * e_n, dgdt_y=LAMBDA * gy * e_n, g_x=2.0 * gx * e_n, g_y=2.0 * gy * e_n)


class StokesBC(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("ut_x", "ut_y", "dgdt_x", "dgdt_y", "g_x", "g_y")]


class Stokes:
    """stokes_2d<Mesh>(mesh, order) on the GPU.  consistent=True takes the
    velocity's Dirichlet data with the jumps apply_inhomogeneous_as_rhs leaves
    out (BC_DATA_CONSISTENT); the default reproduces the reference."""

    def __init__(self, mesh, order: int, consistent: bool = False, rtol: float = 1e-10,
                 mode: int = SOLVE_MIXED_IR, maxit: int = 200000):
        xy = np.ascontiguousarray(mesh.xy, dtype=np.float64).reshape(-1)
        cells = np.ascontiguousarray(mesh.cells, dtype=np.int32).reshape(-1)
        h = _vp()
        _check(lib().dgc_stokes_create(xy.size // 2, xy, cells.size // 3, cells, order, C.byref(h)))
        self._h = h
        hv, hp = _vp(), _vp()
        _check(lib().dgc_stokes_handles(self._h, C.byref(hv), C.byref(hp)))
        self.velocity_space = Discretization._borrow(hv.value, self)
        self.pressure_space = Discretization._borrow(hp.value, self)
        self.velocity_space.set_bc_data_mode(BC_DATA_CONSISTENT if consistent else BC_DATA_REFERENCE)
        self.set_solver(rtol=rtol, mode=mode, maxit=maxit)
        self.state_len = self.velocity_space.state_len
        self._bxy = self.velocity_space.boundary_nodes()

    def close(self):
        if getattr(self, "_h", None):
            lib().dgc_stokes_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_solver(self, rtol: float = 1e-10, mode: int = SOLVE_MIXED_IR, maxit: int = 200000,
                   inner_rtol: float = 1e-4, max_outer: int = 0, graph: bool = True) -> None:
        self._opts = SolveOpts(mode, rtol, maxit, inner_rtol, max_outer, int(graph))
        _check(lib().dgc_stokes_set_solver(self._h, C.byref(self._opts)))

    def empty(self):
        import torch
        return torch.zeros(self.state_len, dtype=torch.float64, device="cuda")

    def boundary_data(self, t: float, t_prev: float, dt: float):
        """The example's boundary data as device tensors (keep them alive over the step)."""
        import torch
        d = example_boundary_data(self._bxy[:, 0], self._bxy[:, 1], t, t_prev, dt)
        return {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in d.items()}

    def step(self, ux_prev, uy_prev, ux, uy, dt: float, bc, out=None, p_out=None, stream=None):
        """advance_timestep: (u^(n-1), u^n) -> u^(n+1); bc = dict of device tensors
        (ut_x, ut_y, dgdt_x, dgdt_y, g_x, g_y).  Returns (ux, uy, stats)."""
        ox, oy = (self.empty(), self.empty()) if out is None else out
        b = StokesBC(*[_ptr(bc[k]) for k in ("ut_x", "ut_y", "dgdt_x", "dgdt_y", "g_x", "g_y")])
        st = SolveStats()
        _check(lib().dgc_stokes_step(self._h, _ptr(ux_prev), _ptr(uy_prev), _ptr(ux), _ptr(uy), dt, C.byref(b),
                                     _ptr(ox), _ptr(oy), None if p_out is None else _ptr(p_out), C.byref(st),
                                     _stream(stream)))
        return ox, oy, st.as_dict()

    def run_example(self, T: float = 0.1, dt: float = 0.001, stream=None):
        """The example driver (examples/stokes_2d/main.cpp:115-190): from the exact
        velocity at t = 0 (u^(-1) = u^0) to T; returns (ux, uy, t, error norm,
        solver iterations)."""
        vs = self.velocity_space
        x, y = vs.node_xy()
        ux0, uy0 = exact_velocity(x.reshape(-1), y.reshape(-1), 0.0)
        up = [vs.upload(ux0, stream), vs.upload(uy0, stream)]
        u = [up[0].clone(), up[1].clone()]
        t_prev = t = 0.0
        iters = 0
        while t < T:
            if t + dt > T:
                dt = T - t
            bc = self.boundary_data(t, t_prev, dt)
            nx, ny, st = self.step(up[0], up[1], u[0], u[1], dt, bc, out=(up[0], up[1]), stream=stream)
            iters += st["iterations"]
            up, u = u, [nx, ny]
            t_prev = t
            t += dt
        rx, ry = exact_velocity(x.reshape(-1), y.reshape(-1), t)
        hx = vs.from_native(u[0], LAYOUT_REF_CPU, stream=stream).cpu().numpy()
        hy = vs.from_native(u[1], LAYOUT_REF_CPU, stream=stream).cpu().numpy()
        err = float(np.sum((rx - hx) ** 2 + (ry - hy) ** 2) / hx.size)
        return u[0], u[1], t, err, iters
