"""ctypes binding of the C oracle (oracle/dgc_oracle.c).

TEST INFRASTRUCTURE ONLY: the CPU restatement of the reference's hot path that
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use as the
checker.  The product never imports this module.

State vectors use the reference CPU layout q[field][cell][node] as float64.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

ADVECTION, MAXWELL_TM, MAXWELL_TE = 0, 1, 2
BC_SINSIN, BC_GAUSS, BC_ZERO = 0, 1, 2
WEAK, STRONG = 0, 1
RK4, LSERK4 = 0, 1

_lock = threading.Lock()
_lib = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


class Problem(C.Structure):
    _fields_ = [("kind", C.c_int), ("ax", C.c_double), ("ay", C.c_double), ("bc", C.c_int),
                ("gx0", C.c_double), ("gy0", C.c_double), ("gw", C.c_double)]


def build() -> str:
    src = [os.path.join(HERE, f) for f in ("dgc_oracle.c", "dgc_oracle.h")]
    if not os.path.exists(LIB_PATH) or any(os.path.getmtime(s) > os.path.getmtime(LIB_PATH) for s in src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            L = C.CDLL(build())
            L.orc_jacobi_p.restype = C.c_double
            L.orc_jacobi_p.argtypes = [C.c_double, C.c_double, C.c_int, C.c_double]
            L.orc_gl_points.argtypes = [C.c_int, _dp]
            L.orc_nodes.argtypes = [C.c_int, _dp, _dp]
            L.orc_face_nodes.argtypes = [C.c_int, C.c_int, _ip]
            L.orc_vandermonde.argtypes = [C.c_int, _dp]
            L.orc_grad_vandermonde.argtypes = [C.c_int, _dp, _dp]
            L.orc_operators.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, C.c_void_p]
            L.orc_create.restype = C.c_void_p
            L.orc_create.argtypes = [C.c_int, C.c_int, _dp, C.c_int, _ip]
            L.orc_destroy.argtypes = [C.c_void_p]
            L.orc_num_boundary_nodes.argtypes = [C.c_void_p]
            L.orc_fill_cell_mappings.argtypes = [C.c_void_p, _dp, _dp, _dp]
            L.orc_fill_cell_interfaces.argtypes = [C.c_void_p, _ip, _ip]
            L.orc_fill_boundary_nodes.argtypes = [C.c_void_p, _dp, _dp]
            L.orc_fill_outward_normals.argtypes = [C.c_void_p, _dp, _dp]
            L.orc_node_xy.argtypes = [C.c_void_p, _dp, _dp]
            L.orc_rhs.argtypes = [C.c_void_p, C.POINTER(Problem), C.c_double, _dp, _dp]
            L.orc_rk4_step.argtypes = [C.c_void_p, C.POINTER(Problem), C.c_double, C.c_double, _dp]
            L.orc_lserk4_step.argtypes = [C.c_void_p, C.POINTER(Problem), C.c_double, C.c_double, _dp, _dp]
            L.orc_run.restype = C.c_double
            L.orc_run.argtypes = [C.c_void_p, C.POINTER(Problem), C.c_int, C.c_double, C.c_double, C.c_int, _dp]
            L.orc_exact.argtypes = [C.c_void_p, C.POINTER(Problem), C.c_double, _dp]
            L.orc_lserk4_coeffs.argtypes = [_dp, _dp, _dp]
            L.orc_laplace_apply.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp]
            L.orc_spd_apply.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
            L.orc_spd_diag_blocks.argtypes = [C.c_void_p, C.c_int, _dp]
            L.orc_mass_apply.argtypes = [C.c_void_p, _dp, _dp]
            L.orc_laplace_apply_bc.argtypes = [C.c_void_p, C.c_void_p, C.c_int, _dp, _dp]
            L.orc_laplace_bc_rhs.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, _dp]
            L.orc_laplace_bc_jump.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, _dp]
            L.orc_grad.argtypes = [C.c_void_p, _dp, C.c_void_p, C.c_double, _dp, _dp]
            L.orc_div.argtypes = [C.c_void_p, _dp, _dp, C.c_void_p, C.c_void_p, C.c_double, _dp]
            L.orc_pcg.restype = C.c_int
            L.orc_pcg.argtypes = [C.c_void_p, C.c_int, _dp, _dp, C.c_double, C.c_int, C.POINTER(C.c_double)]
            L.orc1d_create.restype = C.c_void_p
            L.orc1d_create.argtypes = [C.c_int, C.c_int]
            L.orc1d_destroy.argtypes = [C.c_void_p]
            L.orc1d_operators.argtypes = [C.c_void_p, _dp, _dp]
            L.orc1d_node_x.argtypes = [C.c_void_p, _dp]
            L.orc1d_exact.argtypes = [C.c_void_p, C.c_double, _dp]
            L.orc1d_rhs.argtypes = [C.c_void_p, C.c_double, _dp, _dp]
            L.orc1d_rk4_step.argtypes = [C.c_void_p, C.c_double, C.c_double, _dp]
            _lib = L
    return _lib


def problem(kind: int, ax: float = 1.0, ay: float = 1.0, bc: int = BC_SINSIN,
            gx0: float = -0.3, gy0: float = 0.0, gw: float = 0.02) -> Problem:
    return Problem(kind, ax, ay, bc, gx0, gy0, gw)


def np_(N: int) -> int:
    return (N + 1) * (N + 2) // 2


def nodes(N: int):
    r = np.zeros(np_(N)); s = np.zeros(np_(N))
    if lib().orc_nodes(N, r, s):
        raise ValueError("order out of range")
    return r, s


def face_nodes(N: int):
    out = []
    for f in range(3):
        a = np.zeros(N + 1, np.int32)
        lib().orc_face_nodes(N, f, a)
        out.append(a)
    return out


def gl_points(npts: int):
    x = np.zeros(npts)
    if lib().orc_gl_points(npts, x):
        raise ValueError("npts out of range")
    return x


def vandermonde(N: int):
    n = np_(N)
    V = np.zeros(n * n)
    lib().orc_vandermonde(N, V)
    Vr = np.zeros(n * n); Vs = np.zeros(n * n)
    lib().orc_grad_vandermonde(N, Vr, Vs)
    return V.reshape(n, n), Vr.reshape(n, n), Vs.reshape(n, n)


def operators(N: int, form: int):
    n, nf = np_(N), N + 1
    Dr = np.zeros(n * n); Ds = np.zeros(n * n); L = np.zeros(n * 3 * nf); M = np.zeros(n * n)
    lib().orc_operators(N, form, Dr, Ds, L, M.ctypes.data_as(C.c_void_p))
    return Dr.reshape(n, n), Ds.reshape(n, n), L.reshape(n, 3 * nf), M.reshape(n, n)


class Oracle:
    """Mesh + discretisation + operators of one order (reference CPU layout)."""

    def __init__(self, xy: np.ndarray, cells: np.ndarray, N: int):
        xy = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1)
        cells = np.ascontiguousarray(cells, dtype=np.int32).reshape(-1)
        self.N, self.Np, self.Nfp = N, np_(N), N + 1
        self.K = cells.size // 3
        self._h = lib().orc_create(N, xy.size // 2, xy, self.K, cells)
        if not self._h:
            raise ValueError("oracle: invalid mesh or order")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().orc_destroy(h)
            self._h = None

    def arrays(self):
        K = self.K
        invJ = np.zeros(4 * K); J = np.zeros(K); fJ = np.zeros(3 * K)
        lib().orc_fill_cell_mappings(self._h, invJ, J, fJ)
        nc = np.zeros(3 * K, np.int32); nf = np.zeros(3 * K, np.int32)
        lib().orc_fill_cell_interfaces(self._h, nc, nf)
        nb = lib().orc_num_boundary_nodes(self._h)
        bx = np.zeros(max(nb, 1)); by = np.zeros(max(nb, 1))
        lib().orc_fill_boundary_nodes(self._h, bx, by)
        nx = np.zeros(3 * K); ny = np.zeros(3 * K)
        lib().orc_fill_outward_normals(self._h, nx, ny)
        return dict(invJ=invJ, J=J, faceJ=fJ, nbCell=nc, nbFace=nf, bx=bx[:nb], by=by[:nb], nx=nx, ny=ny)

    def node_xy(self):
        n = self.K * self.Np
        x = np.zeros(n); y = np.zeros(n)
        lib().orc_node_xy(self._h, x, y)
        return x.reshape(self.K, self.Np), y.reshape(self.K, self.Np)

    def nfields(self, p: Problem) -> int:
        return 1 if p.kind == ADVECTION else 3

    def rhs(self, p: Problem, t: float, q: np.ndarray) -> np.ndarray:
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1)
        out = np.zeros_like(q)
        lib().orc_rhs(self._h, C.byref(p), t, q, out)
        return out

    def rk4_step(self, p: Problem, t: float, dt: float, q: np.ndarray) -> np.ndarray:
        q = np.array(q, dtype=np.float64).reshape(-1)
        lib().orc_rk4_step(self._h, C.byref(p), t, dt, q)
        return q

    def lserk4_step(self, p: Problem, t: float, dt: float, q: np.ndarray, res: np.ndarray):
        q = np.array(q, dtype=np.float64).reshape(-1)
        res = np.array(res, dtype=np.float64).reshape(-1)
        lib().orc_lserk4_step(self._h, C.byref(p), t, dt, q, res)
        return q, res

    def run(self, p: Problem, scheme: int, t0: float, dt: float, nsteps: int, q: np.ndarray):
        q = np.array(q, dtype=np.float64).reshape(-1)
        t = lib().orc_run(self._h, C.byref(p), scheme, t0, dt, nsteps, q)
        return q, t

    def exact(self, p: Problem, t: float) -> np.ndarray:
        q = np.zeros(self.nfields(p) * self.K * self.Np)
        lib().orc_exact(self._h, C.byref(p), t, q)
        return q

    def laplace(self, u: np.ndarray, dirichlet: bool = True, tau_mode: int = 0) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        out = np.zeros_like(u)
        lib().orc_laplace_apply(self._h, int(dirichlet), tau_mode, u, out)
        return out

    def laplace_bc(self, u, is_dirichlet, tau_mode: int = 0) -> np.ndarray:
        """apply_homogeneous with a condition type per boundary node (bool array)."""
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        f = np.ascontiguousarray(is_dirichlet, dtype=np.uint8).reshape(-1)
        out = np.zeros_like(u)
        lib().orc_laplace_apply_bc(self._h, f.ctypes.data, tau_mode, u, out)
        return out

    def laplace_bc_rhs(self, is_dirichlet, g=None, h=None, tau_mode: int = 0, out=None,
                       consistent: bool = False) -> np.ndarray:
        """apply_inhomogeneous_as_rhs: adds the boundary-data contribution to out
        (zeros when not given); g, h = exterior_val(x, y, 0), exterior_grad_n(x, y, 0).
        consistent=True adds the jumps of the lifted Dirichlet data as well."""
        out = np.zeros(self.K * self.Np) if out is None else np.array(out, dtype=np.float64).reshape(-1)
        f = np.ascontiguousarray(is_dirichlet, dtype=np.uint8).reshape(-1)
        g, h = self._opt(g), self._opt(h)
        lib().orc_laplace_bc_rhs(self._h, f.ctypes.data, tau_mode, None if g is None else g.ctypes.data,
                                 None if h is None else h.ctypes.data, out)
        if consistent:
            lib().orc_laplace_bc_jump(self._h, f.ctypes.data, None if g is None else g.ctypes.data, out)
        return out

    @staticmethod
    def _opt(a):
        return None if a is None else np.ascontiguousarray(a, dtype=np.float64).reshape(-1)

    def grad(self, u: np.ndarray, g=None, sign: float = 1.0):
        """Weak-form gradient with the central flux (grad_2d); boundary exterior
        value g[b] + sign * interior at boundary node b.  Returns (gx, gy)."""
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        g = self._opt(g)
        gx, gy = np.zeros_like(u), np.zeros_like(u)
        lib().orc_grad(self._h, u, None if g is None else g.ctypes.data, sign, gx, gy)
        return gx, gy

    def div(self, ux: np.ndarray, uy: np.ndarray, gx=None, gy=None, sign: float = 1.0) -> np.ndarray:
        """Weak-form divergence with the central flux (div_2d)."""
        ux = np.ascontiguousarray(ux, dtype=np.float64).reshape(-1)
        uy = np.ascontiguousarray(uy, dtype=np.float64).reshape(-1)
        gx, gy = self._opt(gx), self._opt(gy)
        out = np.zeros_like(ux)
        lib().orc_div(self._h, ux, uy, None if gx is None else gx.ctypes.data,
                      None if gy is None else gy.ctypes.data, sign, out)
        return out

    def spd(self, u: np.ndarray, tau_mode: int = 1) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        out = np.zeros_like(u)
        lib().orc_spd_apply(self._h, tau_mode, u, out)
        return out

    def spd_blocks(self, tau_mode: int = 1) -> np.ndarray:
        b = np.zeros(self.K * self.Np * self.Np)
        lib().orc_spd_diag_blocks(self._h, tau_mode, b)
        return b.reshape(self.K, self.Np, self.Np)

    def mass(self, f: np.ndarray) -> np.ndarray:
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        out = np.zeros_like(f)
        lib().orc_mass_apply(self._h, f, out)
        return out

    def pcg(self, b: np.ndarray, x0=None, rtol: float = 1e-10, maxit: int = 10000, tau_mode: int = 1):
        b = np.ascontiguousarray(b, dtype=np.float64).reshape(-1)
        x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64).reshape(-1)
        rel = C.c_double(0.0)
        it = lib().orc_pcg(self._h, tau_mode, b, x, rtol, maxit, C.byref(rel))
        return x, it, rel.value


class Oracle1D:
    """The 1D advection example (examples/advection_1d/advection_1d.h) on K cells
    of order N; fields in the reference CPU layout [cell][node]."""

    def __init__(self, K: int, N: int):
        self._h = lib().orc1d_create(K, N)
        if not self._h:
            raise ValueError("orc1d_create rejected the arguments")
        self.K, self.N, self.np = K, N, N + 1
        self.h = 2.0 * np.pi / K
        self.c = 2.0 * np.pi

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc1d_destroy(self._h)
            self._h = None

    def operators(self):
        D = np.zeros(self.np * self.np)
        L = np.zeros(self.np * self.np)
        lib().orc1d_operators(self._h, D, L)
        return D.reshape(self.np, self.np), L.reshape(self.np, self.np)

    def node_x(self):
        x = np.zeros(self.K * self.np)
        lib().orc1d_node_x(self._h, x)
        return x

    def exact(self, t: float):
        u = np.zeros(self.K * self.np)
        lib().orc1d_exact(self._h, t, u)
        return u

    def rhs(self, u, t: float):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        out = np.zeros_like(u)
        lib().orc1d_rhs(self._h, t, u, out)
        return out

    def rk4(self, u, t0: float, dt: float, nsteps: int):
        u = np.array(u, dtype=np.float64).reshape(-1)
        t = t0
        for _ in range(nsteps):
            lib().orc1d_rk4_step(self._h, t, dt, u)
            t += dt
        return u


def lserk4_coeffs():
    a = np.zeros(5); b = np.zeros(5); c = np.zeros(5)
    lib().orc_lserk4_coeffs(a, b, c)
    return a, b, c
