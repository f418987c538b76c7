"""Python binding of the GB300 nodal-DG library (lib/libdgc_gb300.so).

A thin ctypes layer over the C ABI in include/dgc_gb300.h.  PyTorch is used
only to own device memory and streams (tensors are passed by data pointer);
all arithmetic runs in the library's CUDA kernels.  There is no CPU fallback:
if the shared library is missing or cannot be loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from . import meshes  # noqa: F401

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "lib", "libdgc_gb300.so")

ADVECTION, MAXWELL_TM, MAXWELL_TE, LAPLACE = 0, 1, 2, 3
F64, F32, F32C = 0, 1, 2  # F32C: FP32 arithmetic, compensated (hi + lo) FP32 state
BC_SINSIN, BC_GAUSS, BC_ZERO = 0, 1, 2
TAU_ONE, TAU_SCALED = 0, 1
LAYOUT_NATIVE, LAYOUT_REF_CPU, LAYOUT_REF_GPU = 0, 1, 2
OP_DR_WEAK, OP_DS_WEAK, OP_LIFT, OP_DR_STRONG, OP_DS_STRONG, OP_MASS, OP_V = range(7)
MPNN_LOSS_L2, MPNN_LOSS_ENERGY = 0, 1
MPNN_ACT_RELU, MPNN_ACT_LINEAR = 0, 1
MPNN_CORR_ADDITIVE, MPNN_CORR_RESIDUAL = 0, 1
PHYSICS = {"advection": ADVECTION, "maxwell_tm": MAXWELL_TM, "maxwell_te": MAXWELL_TE, "laplace": LAPLACE}


class DgcError(RuntimeError):
    pass


class ProblemDesc(C.Structure):
    _fields_ = [("physics", C.c_int), ("order", C.c_int), ("precision", C.c_int),
                ("ax", C.c_double), ("ay", C.c_double), ("bc", C.c_int),
                ("gx0", C.c_double), ("gy0", C.c_double), ("gw", C.c_double),
                ("tau", C.c_int), ("dirichlet", C.c_int)]


class Info(C.Structure):
    _fields_ = [("num_cells", C.c_int64), ("order", C.c_int), ("np", C.c_int), ("np_padded", C.c_int),
                ("nfp", C.c_int), ("num_fields", C.c_int), ("precision", C.c_int),
                ("state_len", C.c_int64), ("scalar_bytes", C.c_int64), ("num_boundary_faces", C.c_int),
                ("min_edge", C.c_double), ("min_altitude", C.c_double),
                ("rhs_tile", C.c_int), ("rhs_threads", C.c_int), ("rhs_smem", C.c_int),
                ("rhs_blocks_per_sm", C.c_int), ("sm_count", C.c_int)]


class SolveOpts(C.Structure):
    _fields_ = [("mode", C.c_int), ("rtol", C.c_double), ("maxit", C.c_int), ("inner_rtol", C.c_double),
                ("max_outer", C.c_int), ("use_graph", C.c_int)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("outer_iterations", C.c_int), ("inner_iterations", C.c_int),
                ("converged", C.c_int), ("final_relres", C.c_double), ("seconds", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


SOLVE_FP64_PCG, SOLVE_MIXED_IR, SOLVE_TWO_LEVEL, SOLVE_TWO_LEVEL_MIXED = 0, 1, 2, 3
BC_DATA_REFERENCE, BC_DATA_CONSISTENT = 0, 1
ERR_NOT_CONVERGED = -6

_lock = threading.Lock()
_lib = None
_vp = C.c_void_p
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def lib():
    """Load the CUDA library (raises if it was not built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise DgcError(f"{LIB_PATH} not built: run __graft_entry__.build() "
                               "or python dg-on-cuda_gb300/dgc_gb300/build.py")
            L = C.CDLL(LIB_PATH)
            L.dgc_last_error.restype = C.c_char_p
            L.dgc_create.argtypes = [C.c_int, _dp, C.c_int, _ip, C.POINTER(ProblemDesc), C.POINTER(_vp)]
            L.dgc_create_from_arrays.argtypes = [C.c_int, _dp, _dp, _dp, _ip, _ip, C.c_int, C.c_void_p,
                                                 C.c_void_p, _dp, _dp, C.POINTER(ProblemDesc), C.POINTER(_vp)]
            L.dgc_destroy.argtypes = [_vp]
            L.dgc_get_info.argtypes = [_vp, C.POINTER(Info)]
            L.dgc_node_coordinates.argtypes = [_vp, _dp, _dp]
            L.dgc_get_operator.argtypes = [_vp, C.c_int, _dp]
            L.dgc_set_operators.argtypes = [_vp, C.c_int, _dp, _dp, _dp]
            L.dgc_to_native.argtypes = [_vp, C.c_int, _vp, _vp, _vp]
            L.dgc_from_native.argtypes = [_vp, C.c_int, _vp, _vp, _vp]
            L.dgc_rhs.argtypes = [_vp, _vp, C.c_double, _vp, _vp]
            L.dgc_axpy.argtypes = [_vp, C.c_double, _vp, _vp, _vp, _vp]
            L.dgc_rk4_step.argtypes = [_vp, _vp, C.c_double, C.c_double, C.POINTER(_vp), _vp]
            L.dgc_lserk4_step.argtypes = [_vp, _vp, _vp, _vp, C.c_double, C.c_double, _vp]
            L.dgc_lserk4_stage.argtypes = [_vp, C.c_int, _vp, _vp, _vp, C.c_double, C.c_double, _vp]
            L.dgc_lserk4_run.argtypes = [_vp, _vp, _vp, _vp, C.c_double, C.c_double, C.c_int, C.c_int,
                                         C.POINTER(_vp), _vp]
            L.dgc_check_device_status.argtypes = [_vp, C.POINTER(C.c_int)]
            L.dgc_launch_count.restype = C.c_int64
            L.dgc_launch_count.argtypes = [_vp]
            L.dgc_laplace_apply.argtypes = [_vp, _vp, _vp, _vp]
            L.dgc_laplace_spd_apply.argtypes = [_vp, _vp, _vp, _vp]
            L.dgc_mass_apply.argtypes = [_vp, _vp, _vp, _vp]
            L.dgc_boundary_nodes.argtypes = [_vp, _dp]
            L.dgc_laplace_set_bc_types.argtypes = [_vp, C.c_void_p]
            L.dgc_laplace_set_shift.argtypes = [_vp, C.c_double]
            L.dgc_laplace_bc_rhs.argtypes = [_vp, _vp, _vp, _vp, _vp]
            L.dgc_laplace_set_bc_data_mode.argtypes = [_vp, C.c_int]
            L.dgc_stokes_create.argtypes = [C.c_int, _dp, C.c_int, _ip, C.c_int, C.POINTER(_vp)]
            L.dgc_stokes_destroy.argtypes = [_vp]
            L.dgc_stokes_handles.argtypes = [_vp, C.POINTER(_vp), C.POINTER(_vp)]
            L.dgc_stokes_set_solver.argtypes = [_vp, C.POINTER(SolveOpts)]
            L.dgc_stokes_step.argtypes = [_vp, _vp, _vp, _vp, _vp, C.c_double, C.c_void_p, _vp, _vp, _vp,
                                          C.POINTER(SolveStats), _vp]
            L.dgc_adv1d_create.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(_vp)]
            L.dgc_adv1d_destroy.argtypes = [_vp]
            L.dgc_adv1d_info.argtypes = [_vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
            L.dgc_adv1d_node_x.argtypes = [_vp, _dp]
            L.dgc_adv1d_get_operator.argtypes = [_vp, C.c_int, _dp]
            L.dgc_adv1d_rhs.argtypes = [_vp, _vp, C.c_double, _vp, _vp]
            L.dgc_adv1d_rk4_step.argtypes = [_vp, _vp, C.c_double, C.c_double, C.POINTER(_vp), _vp]
            L.dgc_adv1d_launch_count.restype = C.c_int64
            L.dgc_adv1d_launch_count.argtypes = [_vp]
            L.dgc_msh_read.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.c_void_p, C.POINTER(C.c_int), C.c_void_p]
            L.dgc_msh_write.argtypes = [C.c_char_p, C.c_int, _dp, C.c_int, _ip, C.c_int]
            L.dgc_write_data_file.argtypes = [C.c_char_p, C.c_int64, _dp, _dp, _dp, C.c_void_p]
            L.dgc_save_state.argtypes = [_vp, C.c_char_p, _vp, C.c_double, _vp]
            L.dgc_load_state.argtypes = [_vp, C.c_char_p, _vp, C.POINTER(C.c_double), _vp]
            L.dgc_grad_apply.argtypes = [_vp, _vp, _vp, _vp, _vp, C.c_double, _vp]
            L.dgc_div_apply.argtypes = [_vp, _vp, _vp, _vp, _vp, _vp, C.c_double, _vp]
            L.dgc_pcg_solve.argtypes = [_vp, _vp, _vp, C.POINTER(SolveOpts), C.POINTER(SolveStats), _vp]
            L.dgc_block_jacobi.argtypes = [_vp, _vp, _vp]
            L.dgc_num_variants.argtypes = [_vp]
            L.dgc_set_variant.argtypes = [_vp, C.c_int]
            L.dgc_autotune.argtypes = [_vp, C.c_int, C.c_void_p, C.POINTER(C.c_int), _vp]
            L.dgc_ref_nodes.argtypes = [C.c_int, _dp, _dp]
            L.dgc_ref_operator.argtypes = [C.c_int, C.c_int, _dp]
            L.dgc_host_mesh.argtypes = [C.c_int, _dp, C.c_int, _ip, C.c_int, _dp, _ip, C.POINTER(C.c_int)]
            L.dgc_mesh_neighbors.argtypes = [_vp, _ip, C.POINTER(C.c_int)]
            L.dgc_batch_create.argtypes = [C.POINTER(_vp), C.c_int, C.POINTER(_vp)]
            L.dgc_batch_destroy.argtypes = [_vp]
            L.dgc_batch_lserk4_step.argtypes = [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), _dp, _dp, _vp]
            L.dgc_batch_lserk4_run.argtypes = [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), _dp, _dp,
                                               C.c_int, C.c_int, C.POINTER(C.c_int), _vp]
            L.dgc_batch_launch_count.restype = C.c_int64
            L.dgc_batch_launch_count.argtypes = [_vp]
            L.dgc_mpnn_create.argtypes = [_vp, C.c_int, C.c_uint64, C.POINTER(_vp)]
            L.dgc_mpnn_destroy.argtypes = [_vp]
            L.dgc_mpnn_num_params.restype = C.c_int64
            L.dgc_mpnn_num_params.argtypes = [_vp]
            L.dgc_mpnn_get_weights.argtypes = [_vp, C.c_void_p]
            L.dgc_mpnn_set_weights.argtypes = [_vp, C.c_void_p]
            L.dgc_mpnn_train_step.argtypes = [_vp, _vp, _vp, C.c_int, C.c_float, C.POINTER(C.c_float), _vp, _vp]
            L.dgc_mpnn_forward.argtypes = [_vp, _vp, _vp, _vp]
            L.dgc_mpnn_set_loss.argtypes = [_vp, C.c_int]
            L.dgc_mpnn_set_activation.argtypes = [_vp, C.c_int]
            L.dgc_mpnn_set_correction.argtypes = [_vp, C.c_int]
            L.dgc_mpnn_set_coarse.argtypes = [_vp, C.c_int, _vp]
            L.dgc_coarse_build.argtypes = [_vp, C.c_int, _vp]
            L.dgc_coarse_apply.argtypes = [_vp, _vp, _vp, C.c_int, _vp]
            L.dgc_coarse_info.argtypes = [_vp, C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                          C.POINTER(C.c_double)]
            L.dgc_mpnn_precondition.argtypes = [_vp, _vp, _vp, _vp]
            L.dgc_fpcg_solve.argtypes = [_vp, _vp, _vp, _vp, C.POINTER(SolveOpts), C.POINTER(SolveStats), _vp]
            L.dgc_learned_solve.argtypes = [_vp, _vp, _vp, _vp, C.POINTER(SolveOpts), C.c_int,
                                            C.POINTER(SolveStats), C.POINTER(C.c_int), _vp]
            _lib = L
    return _lib


def _check(rc: int) -> None:
    if rc != 0:
        raise DgcError(f"dgc error {rc}: {lib().dgc_last_error().decode()}")


def _stream(stream=None) -> int:
    if stream is not None:
        return int(stream)
    import torch
    return int(torch.cuda.current_stream().cuda_stream)


def _ptr(t) -> int:
    return int(t.data_ptr())


def ref_nodes(order: int):
    n = (order + 1) * (order + 2) // 2
    r = np.zeros(n)
    s = np.zeros(n)
    _check(lib().dgc_ref_nodes(order, r, s))
    return r, s


def ref_operator(order: int, which: int) -> np.ndarray:
    n, nfp = (order + 1) * (order + 2) // 2, order + 1
    shape = (n, 3 * nfp) if which == OP_LIFT else (n, n)
    out = np.zeros(shape[0] * shape[1])
    _check(lib().dgc_ref_operator(order, which, out))
    return out.reshape(shape)


def host_mesh(mesh, order: int):
    """Validated topology and geometry computed on the host (no GPU)."""
    xy = np.ascontiguousarray(mesh.xy, dtype=np.float64).reshape(-1)
    cells = np.ascontiguousarray(mesh.cells, dtype=np.int32).reshape(-1)
    K = cells.size // 3
    geom = np.zeros(K * 16)
    nbr = np.zeros(K * 4, np.int32)
    nb = C.c_int(0)
    _check(lib().dgc_host_mesh(xy.size // 2, xy, K, cells, order, geom, nbr, C.byref(nb)))
    return geom.reshape(K, 16), nbr.reshape(K, 4), nb.value


def read_msh(path: str):
    """Triangle mesh of a Gmsh MSH 4 file (dgc_msh_read) as a meshes.Mesh."""
    nv, K = C.c_int(0), C.c_int(0)
    _check(lib().dgc_msh_read(os.fsencode(path), C.byref(nv), None, C.byref(K), None))
    xy = np.zeros(2 * max(nv.value, 1))
    cells = np.zeros(3 * max(K.value, 1), np.int32)
    _check(lib().dgc_msh_read(os.fsencode(path), C.byref(nv), xy.ctypes.data, C.byref(K), cells.ctypes.data))
    return meshes.Mesh(xy=xy[:2 * nv.value].reshape(-1, 2), cells=cells[:3 * K.value].reshape(-1, 3))


def write_msh(path: str, mesh, digits: int = 0) -> None:
    """MSH 4.1 file of a triangle mesh (dgc_msh_write); digits 0 = the reference's 6."""
    xy = np.ascontiguousarray(mesh.xy, dtype=np.float64).reshape(-1)
    cells = np.ascontiguousarray(mesh.cells, dtype=np.int32).reshape(-1)
    _check(lib().dgc_msh_write(os.fsencode(path), xy.size // 2, xy, cells.size // 3, cells, digits))


def write_data_file(path: str, x, y, u, ref=None) -> None:
    """The reference drivers' visualisation text file (dgc_write_data_file); host arrays."""
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64).reshape(-1)  # noqa: E731
    x, y, u = f(x), f(y), f(u)
    r = None if ref is None else f(ref)
    _check(lib().dgc_write_data_file(os.fsencode(path), x.size, x, y, u, None if r is None else r.ctypes.data))


class Discretization:
    """Mesh + order + physics on the current CUDA device (the handle of the C ABI)."""

    def __init__(self, mesh, physics, order: int, precision: int = F64, ax: float = 1.0, ay: float = 1.0,
                 bc: int = BC_SINSIN, gx0: float = -0.3, gy0: float = 0.0, gw: float = 0.02,
                 tau: int = TAU_SCALED, dirichlet: bool = True):
        if isinstance(physics, str):
            physics = PHYSICS[physics]
        xy = np.ascontiguousarray(mesh.xy, dtype=np.float64).reshape(-1)
        cells = np.ascontiguousarray(mesh.cells, dtype=np.int32).reshape(-1)
        self.desc = ProblemDesc(physics, order, precision, ax, ay, bc, gx0, gy0, gw, tau, int(dirichlet))
        h = _vp()
        _check(lib().dgc_create(xy.size // 2, xy, cells.size // 3, cells, C.byref(self.desc), C.byref(h)))
        self._adopt(h, precision)

    @classmethod
    def from_arrays(cls, arrays, physics, order: int, precision: int = F64, ax: float = 1.0, ay: float = 1.0,
                    bc: int = BC_SINSIN, gx0: float = -0.3, gy0: float = 0.0, gw: float = 0.02,
                    tau: int = TAU_SCALED, dirichlet: bool = True):
        """Handle from the reference's flattened discretisation arrays (a mapping with
        invJ, J, faceJ, nbCell, nbFace, bx, by, nx, ny as simple_discretization_2d's
        fill_* functions produce them), through dgc_create_from_arrays."""
        if isinstance(physics, str):
            physics = PHYSICS[physics]
        self = cls.__new__(cls)
        f = lambda k: np.ascontiguousarray(arrays[k], dtype=np.float64).reshape(-1)  # noqa: E731
        i = lambda k: np.ascontiguousarray(arrays[k], dtype=np.int32).reshape(-1)   # noqa: E731
        J = f("J")
        bx, by = f("bx"), f("by")
        self.desc = ProblemDesc(physics, order, precision, ax, ay, bc, gx0, gy0, gw, tau, int(dirichlet))
        h = _vp()
        _check(lib().dgc_create_from_arrays(J.size, f("invJ"), J, f("faceJ"), i("nbCell"), i("nbFace"), bx.size,
                                            bx.ctypes.data, by.ctypes.data, f("nx"), f("ny"),
                                            C.byref(self.desc), C.byref(h)))
        self._adopt(h, precision)
        return self

    def _adopt(self, h, precision: int) -> None:
        self._h = h
        info = Info()
        _check(lib().dgc_get_info(self._h, C.byref(info)))
        self.info = info
        self.K, self.N, self.Np, self.NpP = info.num_cells, info.order, info.np, info.np_padded
        self.Nfp, self.Nf = info.nfp, info.num_fields
        self.state_len = info.state_len
        self.precision = precision

    @classmethod
    def _borrow(cls, h, owner):
        """View of a handle owned by another object (kept alive through owner)."""
        self = cls.__new__(cls)
        self._h = _vp(h)
        self._owner = owner
        info = Info()
        _check(lib().dgc_get_info(self._h, C.byref(info)))
        self.info = info
        self.K, self.N, self.Np, self.NpP = info.num_cells, info.order, info.np, info.np_padded
        self.Nfp, self.Nf = info.nfp, info.num_fields
        self.state_len = info.state_len
        self.precision = info.precision
        return self

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and getattr(self, "_owner", None) is None:
            try:
                lib().dgc_destroy(h)
            except Exception:
                pass
        self._h = None

    # ---------------------------------------------------------------- host-side info
    @property
    def torch_dtype(self):
        import torch
        return torch.float64 if self.precision == F64 else torch.float32

    @property
    def state_elems(self) -> int:
        """Elements of torch_dtype in one native state buffer (F32C: hi and lo vectors)."""
        return 2 * self.state_len if self.precision == F32C else self.state_len

    @property
    def ref_dtype(self):
        """dtype of the reference-layout arrays dgc_to_native / dgc_from_native exchange."""
        import torch
        return torch.float32 if self.precision == F32 else torch.float64

    def node_xy(self):
        x = np.zeros(self.K * self.Np)
        y = np.zeros(self.K * self.Np)
        _check(lib().dgc_node_coordinates(self._h, x, y))
        return x.reshape(self.K, self.Np), y.reshape(self.K, self.Np)

    def neighbors(self):
        """The twin map [K][4] ((k << 2 | f) of the twin face, -(1 + b) for boundary face b)
        and the number of boundary faces."""
        out = np.zeros(4 * self.K, np.int32)
        nb = C.c_int()
        _check(lib().dgc_mesh_neighbors(self._h, out, C.byref(nb)))
        return out.reshape(self.K, 4), nb.value

    def operator(self, which: int) -> np.ndarray:
        shape = {OP_LIFT: (self.Np, 3 * self.Nfp)}.get(which, (self.Np, self.Np))
        out = np.zeros(shape[0] * shape[1])
        _check(lib().dgc_get_operator(self._h, which, out))
        return out.reshape(shape)

    def set_operators(self, form: int, Dr, Ds, L) -> None:
        f = lambda a: np.ascontiguousarray(a, dtype=np.float64).reshape(-1)  # noqa: E731
        _check(lib().dgc_set_operators(self._h, form, f(Dr), f(Ds), f(L)))

    def launch_count(self) -> int:
        return int(lib().dgc_launch_count(self._h))

    def num_variants(self) -> int:
        n = lib().dgc_num_variants(self._h)
        if n < 0:
            _check(n)
        return n

    def set_variant(self, v: int) -> None:
        _check(lib().dgc_set_variant(self._h, v))
        info = Info()
        _check(lib().dgc_get_info(self._h, C.byref(info)))
        self.info = info

    def autotune(self, reps: int = 10, measure: bool = True, stream=None):
        """Time the tile-shape variants and keep the fastest; returns (chosen, times_ms or None)."""
        n = self.num_variants()
        times = (C.c_double * n)() if measure else None
        chosen = C.c_int(-1)
        _check(lib().dgc_autotune(self._h, reps, C.cast(times, C.c_void_p) if measure else None,
                                  C.byref(chosen), _stream(stream)))
        info = Info()
        _check(lib().dgc_get_info(self._h, C.byref(info)))
        self.info = info
        return chosen.value, (list(times) if measure else None)

    def check(self) -> None:
        code = C.c_int(0)
        _check(lib().dgc_check_device_status(self._h, C.byref(code)))

    # ---------------------------------------------------------------- device state
    def empty_state(self, zero: bool = True):
        import torch
        f = torch.zeros if zero else torch.empty
        return f(self.state_elems, dtype=self.torch_dtype, device="cuda")

    def to_native(self, src, layout: int = LAYOUT_REF_CPU, out=None, stream=None):
        out = self.empty_state() if out is None else out
        _check(lib().dgc_to_native(self._h, layout, _ptr(src), _ptr(out), _stream(stream)))
        return out

    def from_native(self, q, layout: int = LAYOUT_REF_CPU, out=None, stream=None):
        import torch
        if out is None:
            out = torch.empty(self.Nf * self.K * self.Np, dtype=self.ref_dtype, device="cuda")
        _check(lib().dgc_from_native(self._h, layout, _ptr(q), _ptr(out), _stream(stream)))
        return out

    def upload(self, q_ref_cpu: np.ndarray, stream=None):
        """Host array in the reference CPU layout [field][cell][node] -> native device state."""
        import torch
        src = torch.from_numpy(np.ascontiguousarray(q_ref_cpu).reshape(-1)).to(self.ref_dtype).cuda()
        return self.to_native(src, LAYOUT_REF_CPU, stream=stream)

    def download(self, q, stream=None) -> np.ndarray:
        """Native device state -> host float64 array in the reference CPU layout."""
        return self.from_native(q, LAYOUT_REF_CPU, stream=stream).double().cpu().numpy()

    # ---------------------------------------------------------------- operators
    def rhs(self, q, t: float, out=None, stream=None):
        out = self.empty_state() if out is None else out
        _check(lib().dgc_rhs(self._h, _ptr(q), t, _ptr(out), _stream(stream)))
        return out

    def axpy(self, a: float, x, y, out, stream=None):
        _check(lib().dgc_axpy(self._h, a, _ptr(x), _ptr(y), _ptr(out), _stream(stream)))
        return out

    def rk4_step(self, q, t: float, dt: float, work, stream=None):
        arr = (_vp * 3)(*[_ptr(w) for w in work])
        _check(lib().dgc_rk4_step(self._h, _ptr(q), t, dt, arr, _stream(stream)))
        return q

    def lserk4_step(self, q_in, q_out, res, t: float, dt: float, stream=None):
        _check(lib().dgc_lserk4_step(self._h, _ptr(q_in), _ptr(q_out), _ptr(res), t, dt, _stream(stream)))
        return q_out

    def lserk4_stage(self, stage: int, q_in, q_out, res, t: float, dt: float, stream=None):
        _check(lib().dgc_lserk4_stage(self._h, stage, _ptr(q_in), _ptr(q_out), _ptr(res), t, dt,
                                      _stream(stream)))
        return q_out

    def lserk4_run(self, qa, qb, res, t0: float, dt: float, nsteps: int, graph: bool = True, stream=None):
        fin = _vp()
        _check(lib().dgc_lserk4_run(self._h, _ptr(qa), _ptr(qb), _ptr(res), t0, dt, nsteps, int(graph),
                                    C.byref(fin), _stream(stream)))
        return qa if fin.value == _ptr(qa) else qb

    # ---------------------------------------------------------------- checkpoints
    def save_state(self, path: str, q, t: float, stream=None) -> None:
        _check(lib().dgc_save_state(self._h, os.fsencode(path), _ptr(q), t, _stream(stream)))

    def load_state(self, path: str, q=None, stream=None):
        """Returns (q, t)."""
        q = self.empty_state(zero=False) if q is None else q
        t = C.c_double(0.0)
        _check(lib().dgc_load_state(self._h, os.fsencode(path), _ptr(q), C.byref(t), _stream(stream)))
        return q, t.value

    # ---------------------------------------------------------------- grad_2d / div_2d
    def boundary_nodes(self) -> np.ndarray:
        """Boundary face node coordinates, (num_boundary_faces * Nfp, 2)."""
        xy = np.zeros(max(self.info.num_boundary_faces * self.Nfp, 1) * 2)
        _check(lib().dgc_boundary_nodes(self._h, xy))
        return xy[:2 * self.info.num_boundary_faces * self.Nfp].reshape(-1, 2)

    @staticmethod
    def _bdata(g):
        import torch
        if g is None:
            return None, None
        t = g if isinstance(g, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(g, dtype=np.float64))
        t = t.to(device="cuda", dtype=torch.float64).contiguous()
        return t, _ptr(t)

    def grad(self, u, g=None, sign: float = 1.0, out=None, stream=None):
        """(gx, gy) = weak-form gradient of the scalar field u (central flux); boundary
        exterior value g[b] + sign * u- at boundary node b."""
        gx, gy = (self.empty_state(), self.empty_state()) if out is None else out
        keep, gp = self._bdata(g)
        _check(lib().dgc_grad_apply(self._h, _ptr(u), _ptr(gx), _ptr(gy), gp, sign, _stream(stream)))
        return gx, gy

    def div(self, ux, uy, gx=None, gy=None, sign: float = 1.0, out=None, stream=None):
        """Weak-form divergence of (ux, uy) (central flux)."""
        out = self.empty_state() if out is None else out
        kx, px = self._bdata(gx)
        ky, py = self._bdata(gy)
        _check(lib().dgc_div_apply(self._h, _ptr(ux), _ptr(uy), _ptr(out), px, py, sign, _stream(stream)))
        return out

    # ---------------------------------------------------------------- laplace_2d
    def laplace(self, u, out=None, stream=None):
        out = self.empty_state() if out is None else out
        _check(lib().dgc_laplace_apply(self._h, _ptr(u), _ptr(out), _stream(stream)))
        return out

    def set_shift(self, shift: float) -> None:
        """SPD form S = -J M (A - shift I) for spd(), pcg() and the block-Jacobi blocks."""
        _check(lib().dgc_laplace_set_shift(self._h, shift))

    def set_bc_data_mode(self, mode: int) -> None:
        """BC_DATA_REFERENCE (apply_inhomogeneous_as_rhs as the reference forms it)
        or BC_DATA_CONSISTENT (plus the jumps of the lifted Dirichlet data)."""
        _check(lib().dgc_laplace_set_bc_data_mode(self._h, mode))

    def set_bc_types(self, is_dirichlet=None) -> None:
        """Per-boundary-node condition types (bool array in boundary_nodes() order); None = uniform."""
        if is_dirichlet is None:
            _check(lib().dgc_laplace_set_bc_types(self._h, None))
            return
        f = np.ascontiguousarray(is_dirichlet, dtype=np.uint8).reshape(-1)
        _check(lib().dgc_laplace_set_bc_types(self._h, f.ctypes.data))

    def laplace_bc_rhs(self, g=None, h=None, out=None, stream=None):
        """out += the boundary-data contribution (apply_inhomogeneous_as_rhs); g, h per boundary node."""
        out = self.empty_state() if out is None else out
        kg, pg = self._bdata(g)
        kh, ph = self._bdata(h)
        _check(lib().dgc_laplace_bc_rhs(self._h, pg, ph, _ptr(out), _stream(stream)))
        return out

    def spd(self, u, out=None, stream=None):
        out = self.empty_state() if out is None else out
        _check(lib().dgc_laplace_spd_apply(self._h, _ptr(u), _ptr(out), _stream(stream)))
        return out

    def mass(self, f, out=None, stream=None):
        import torch
        out = torch.zeros(self.state_len, dtype=torch.float64, device="cuda") if out is None else out
        _check(lib().dgc_mass_apply(self._h, _ptr(f), _ptr(out), _stream(stream)))
        return out

    def block_jacobi(self, stream=None):
        import torch
        out = torch.zeros(self.K * self.Np * self.Np, dtype=torch.float64, device="cuda")
        _check(lib().dgc_block_jacobi(self._h, _ptr(out), _stream(stream)))
        return out.view(self.K, self.Np, self.Np)

    def coarse_build(self, cells_per_aggregate: int, stream=None) -> None:
        _check(lib().dgc_coarse_build(self._h, cells_per_aggregate, _stream(stream)))

    def coarse_apply(self, r, out=None, precision: int = F64, stream=None):
        """out = P A_c^-1 P^T r (FP64 device vectors; precision of the smoothing applies)."""
        import torch
        out = torch.zeros(self.state_len, dtype=torch.float64, device="cuda") if out is None else out
        _check(lib().dgc_coarse_apply(self._h, _ptr(r), _ptr(out), precision, _stream(stream)))
        return out

    def coarse_info(self):
        """(aggregate of each cell, number of aggregates, number of colours, omega)."""
        agg = np.zeros(self.K, np.int32)
        na, nc, om = C.c_int(), C.c_int(), C.c_double()
        _check(lib().dgc_coarse_info(self._h, agg.ctypes.data, C.byref(na), C.byref(nc), C.byref(om)))
        return agg, na.value, nc.value, om.value

    def pcg(self, b, x=None, mode: int = SOLVE_FP64_PCG, rtol: float = 1e-10, maxit: int = 20000,
            inner_rtol: float = 1e-4, max_outer: int = 20, graph: bool = True, stream=None, check: bool = True):
        """Solve S x = b (FP64 device vectors, native layout).  Returns (x, stats dict)."""
        import torch
        x = torch.zeros(self.state_len, dtype=torch.float64, device="cuda") if x is None else x
        opts = SolveOpts(mode, rtol, maxit, inner_rtol, max_outer, int(graph))
        st = SolveStats()
        rc = lib().dgc_pcg_solve(self._h, _ptr(b), _ptr(x), C.byref(opts), C.byref(st), _stream(stream))
        if rc != 0 and not (rc == ERR_NOT_CONVERGED and not check):
            _check(rc)
        return x, st.as_dict()


class Advection1D:
    """The 1D advection example (dgc_adv1d_*): K cells of order N on [0, 2 pi];
    device state [cell][node] in the given precision."""

    def __init__(self, num_cells: int, order: int, precision: int = F64):
        h = _vp()
        _check(lib().dgc_adv1d_create(num_cells, order, precision, C.byref(h)))
        self._h = h
        self.K, self.N, self.np, self.precision = num_cells, order, order + 1, precision
        hh, c = C.c_double(), C.c_double()
        _check(lib().dgc_adv1d_info(self._h, C.byref(hh), C.byref(c)))
        self.min_elem_size, self.wave_speed = hh.value, c.value

    def close(self):
        if getattr(self, "_h", None):
            lib().dgc_adv1d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def torch_dtype(self):
        import torch
        return torch.float64 if self.precision == F64 else torch.float32

    def node_x(self) -> np.ndarray:
        x = np.zeros(self.K * self.np)
        _check(lib().dgc_adv1d_node_x(self._h, x))
        return x

    def operator(self, which: int) -> np.ndarray:
        out = np.zeros(self.np * self.np)
        _check(lib().dgc_adv1d_get_operator(self._h, which, out))
        return out.reshape(self.np, self.np)

    def upload(self, u):
        import torch
        return torch.from_numpy(np.ascontiguousarray(u, dtype=np.float64).reshape(-1)).to(self.torch_dtype).cuda()

    def empty_state(self):
        import torch
        return torch.zeros(self.K * self.np, dtype=self.torch_dtype, device="cuda")

    def rhs(self, q, t: float, out=None, stream=None):
        out = self.empty_state() if out is None else out
        _check(lib().dgc_adv1d_rhs(self._h, _ptr(q), t, _ptr(out), _stream(stream)))
        return out

    def rk4_step(self, q, t: float, dt: float, work, stream=None):
        arr = (_vp * 3)(*[_ptr(w) for w in work])
        _check(lib().dgc_adv1d_rk4_step(self._h, _ptr(q), t, dt, arr, _stream(stream)))
        return q

    def launch_count(self) -> int:
        return int(lib().dgc_adv1d_launch_count(self._h))


class Batch:
    """Many independent FP32 advection / Maxwell discretizations advanced together:
    every LSERK4 stage of every instance is one persistent launch (dgc_batch_*)."""

    def __init__(self, discretizations):
        self.items = list(discretizations)
        n = len(self.items)
        arr = (_vp * n)(*[d._h for d in self.items])
        h = _vp()
        _check(lib().dgc_batch_create(arr, n, C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().dgc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _ptrs(ts):
        return (_vp * len(ts))(*[_ptr(t) for t in ts])

    def lserk4_step(self, q_in, q_out, res, t, dt, stream=None):
        """One step of every instance: q_in[i] -> q_out[i] at times t[i], steps dt[i]."""
        tt = np.ascontiguousarray(t, dtype=np.float64)
        dd = np.ascontiguousarray(dt, dtype=np.float64)
        _check(lib().dgc_batch_lserk4_step(self._h, self._ptrs(q_in), self._ptrs(q_out), self._ptrs(res), tt, dd,
                                           _stream(stream)))
        return q_out

    def lserk4_run(self, qa, qb, res, t0, dt, nsteps: int, graph: bool = True, stream=None):
        """nsteps steps from qa; returns the list of tensors holding the results."""
        tt = np.ascontiguousarray(t0, dtype=np.float64)
        dd = np.ascontiguousarray(dt, dtype=np.float64)
        fin = C.c_int()
        _check(lib().dgc_batch_lserk4_run(self._h, self._ptrs(qa), self._ptrs(qb), self._ptrs(res), tt, dd,
                                          int(nsteps), int(graph), C.byref(fin), _stream(stream)))
        return list(qb) if fin.value else list(qa)

    def launch_count(self) -> int:
        return int(lib().dgc_batch_launch_count(self._h))


class MPNN:
    """Learned preconditioner of a Dirichlet laplace Discretization: a message-passing
    network over element adjacency (width 64), BF16 weights, FP32 accumulation,
    used as M(r) = Binv r + (|r|/c) net(c r/|r|), c = sqrt(K Np), inside truncated
    flexible CG (dgc_mpnn_*, dgc_fpcg_solve)."""

    WIDTH = 64

    def __init__(self, disc, layers: int = 4, seed: int = 0):
        self.disc = disc
        self.layers = layers
        h = _vp()
        _check(lib().dgc_mpnn_create(disc._h, layers, seed, C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().dgc_mpnn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_params(self) -> int:
        return int(lib().dgc_mpnn_num_params(self._h))

    def set_coarse(self, cells_per_aggregate: int, stream=None):
        """Two-level form: M(r) = Binv r + P A_c^-1 P^T r + network (0 = off)."""
        _check(lib().dgc_mpnn_set_coarse(self._h, cells_per_aggregate, _stream(stream)))

    def set_loss(self, kind: int):
        """MPNN_LOSS_ENERGY (default: |d|_S^2 / |t|_S^2) or MPNN_LOSS_L2 (|d|^2 / |t|^2)."""
        _check(lib().dgc_mpnn_set_loss(self._h, kind))


    def set_activation(self, kind: int):
        """MPNN_ACT_RELU (default) or MPNN_ACT_LINEAR (no ReLU, biases zero and held there)."""
        _check(lib().dgc_mpnn_set_activation(self._h, kind))

    def set_correction(self, kind: int):
        """MPNN_CORR_ADDITIVE (default) or MPNN_CORR_RESIDUAL (the network acts on r - S z0)."""
        _check(lib().dgc_mpnn_set_correction(self._h, kind))
    def get_weights(self) -> np.ndarray:
        w = np.zeros(self.num_params, dtype=np.float32)
        _check(lib().dgc_mpnn_get_weights(self._h, w.ctypes.data))
        return w

    def set_weights(self, w: np.ndarray):
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert w.size == self.num_params
        _check(lib().dgc_mpnn_set_weights(self._h, w.ctypes.data))

    def train_step(self, x, t, lr: float = 0.0, want_grad: bool = False, stream=None):
        """x, t: device FP32 tensors of S fields (S * K * NpP); returns (loss, grad or None)."""
        import torch
        S = x.numel() // (self.disc.K * self.disc.NpP)
        grad = torch.empty(self.num_params, dtype=torch.float32, device="cuda") if want_grad else None
        loss = C.c_float()
        _check(lib().dgc_mpnn_train_step(self._h, _ptr(x), _ptr(t), S, float(lr), C.byref(loss),
                                         _ptr(grad) if grad is not None else None, _stream(stream)))
        return float(loss.value), grad

    def forward(self, x, stream=None):
        import torch
        y = torch.empty_like(x)
        _check(lib().dgc_mpnn_forward(self._h, _ptr(x), _ptr(y), _stream(stream)))
        return y

    def precondition(self, r, stream=None):
        import torch
        z = torch.empty_like(r)
        _check(lib().dgc_mpnn_precondition(self._h, _ptr(r), _ptr(z), _stream(stream)))
        return z

    def fpcg(self, b, x=None, rtol: float = 1e-10, maxit: int = 20000, window: int = 4, stream=None,
             check: bool = True):
        """Truncated flexible CG (window previous directions) on S x = b with this network as
        preconditioner; returns (x, stats dict)."""
        import torch
        x = torch.zeros(self.disc.state_len, dtype=torch.float64, device="cuda") if x is None else x
        opts = SolveOpts(0, rtol, maxit, 0.0, window, 0)
        st = SolveStats()
        rc = lib().dgc_fpcg_solve(self.disc._h, self._h, _ptr(b), _ptr(x), C.byref(opts), C.byref(st),
                                  _stream(stream))
        if rc != 0 and not (rc == ERR_NOT_CONVERGED and not check):
            _check(rc)
        return x, st.as_dict()

    def solve(self, b, x=None, rtol: float = 1e-10, maxit: int = 100000, fcg_maxit: int = 1000,
              mode: int = SOLVE_FP64_PCG, window: int = 4, stream=None, check: bool = True):
        """Learned solve with block-Jacobi PCG (mode) as fallback and final check: flexible CG with
        this network for at most fcg_maxit iterations, then PCG from the current iterate.
        Returns (x, stats dict with "fell_back")."""
        import torch
        x = torch.zeros(self.disc.state_len, dtype=torch.float64, device="cuda") if x is None else x
        opts = SolveOpts(mode, rtol, maxit, 1e-4, window, 1)
        st = SolveStats()
        fb = C.c_int(0)
        rc = lib().dgc_learned_solve(self.disc._h, self._h, _ptr(b), _ptr(x), C.byref(opts), fcg_maxit,
                                     C.byref(st), C.byref(fb), _stream(stream))
        if rc != 0 and not (rc == ERR_NOT_CONVERGED and not check):
            _check(rc)
        d = st.as_dict()
        d["fell_back"] = bool(fb.value)
        return x, d
