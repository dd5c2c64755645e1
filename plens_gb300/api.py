"""Python host mirror of the reference's solver interface, over the two C ABIs.

``Case`` is the setup chain (PLENS::PLENS ... read_time_settings, dgsem/plens.cc:13-1499): it
parses input.prm text and owns the mesh description, parameters and initial state.
``GpuSolver`` is the hot path on the GPU (PLENS::calc_rhs / calc_time_step / update,
dgsem/plens.cc:3688-4518) through include/plens_gpu.h. Errors raise ``PlensError`` with the
library's message; a positivity failure raises ``PositivityError`` carrying the first bad dof
(the reference prints the dof location and calls std::exit, dgsem/plens.cc:2531-2546).
"""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_DIR = _PKG / "lib"

PLENS_GPU_OK = 0
PLENS_GPU_E_INVALID = 1
PLENS_GPU_E_CUDA = 2
PLENS_GPU_E_POSITIVITY = 3
PLENS_GPU_E_TIMEOUT = 4

PRECISION_FP64 = 0
PRECISION_MIXED = 1
PRECISION_MIXED_R32 = 2
PRECISIONS = {"fp64": PRECISION_FP64, "mixed": PRECISION_MIXED, "mixed_r32": PRECISION_MIXED_R32}
SENSOR_MODAL = 0
SENSOR_LEARNED = 1
MLP_N_PARAMS = 64 * 64 + 64 + 64 * 64 + 64 + 64 + 1


class PlensError(RuntimeError):
    pass


class PositivityError(PlensError):
    def __init__(self, msg: str, dof: int):
        super().__init__(msg)
        self.dof = dof


class BCDesc(C.Structure):
    _fields_ = [
        ("type", C.c_int32), ("expr_p", C.c_int32), ("expr_T", C.c_int32),
        ("expr_vel", C.c_int32 * 3), ("p", C.c_double), ("T", C.c_double),
        ("vel", C.c_double * 3), ("cons", C.c_double * 5),
    ]


class Params(C.Structure):
    _fields_ = [
        ("degree", C.c_int32),
        ("gamma", C.c_double), ("R", C.c_double), ("Pr", C.c_double), ("mu0", C.c_double),
        ("T0", C.c_double), ("S", C.c_double),
        ("const_viscosity", C.c_int32), ("inv_surf_flux", C.c_int32), ("inv_vol_flux", C.c_int32),
        ("plens_2d", C.c_int32), ("blender_variable", C.c_int32), ("blender_function", C.c_int32),
        ("threshold_factor", C.c_double), ("threshold_exp_factor", C.c_double),
        ("sharpness_factor", C.c_double), ("alpha_min", C.c_double), ("alpha_max", C.c_double),
        ("expr_wall_blender_limit", C.c_int32), ("expr_vis_blending_region", C.c_int32),
        ("expr_courant", C.c_int32), ("do_filtering", C.c_int32), ("rk_order", C.c_int32),
        ("local_stepping", C.c_int32), ("limit_local_step", C.c_int32), ("local_start_time", C.c_double),
        ("local_nbr_factor", C.c_double), ("local_global_factor", C.c_double),
        ("calc_ss_error", C.c_int32), ("calc_conv_error", C.c_int32), ("expr_conv_exact", C.c_int32),
        ("precision", C.c_int32), ("sensor", C.c_int32), ("judge_every", C.c_int32),
        ("judge_alpha_tol", C.c_double),
        ("n_bc", C.c_int32), ("bcs", C.POINTER(BCDesc)),
        ("n_expr", C.c_int32), ("expr_offset", C.POINTER(C.c_int32)),
        ("expr_length", C.POINTER(C.c_int32)),
        ("n_expr_insn", C.c_int32), ("expr_code", C.c_void_p),
    ]


class MeshDesc(C.Structure):
    _fields_ = [
        ("degree", C.c_int32), ("n_cells", C.c_int64),
        ("detJ", C.POINTER(C.c_double)), ("Ja", C.POINTER(C.c_double)), ("Jinv", C.POINTER(C.c_double)),
        ("h_min", C.POINTER(C.c_double)), ("cell_center", C.POINTER(C.c_double)),
        ("cell_nbr", C.POINTER(C.c_int32)), ("cell_face_bc", C.POINTER(C.c_int32)),
        ("n_face_tasks", C.c_int64),
        ("ft_cell", C.POINTER(C.c_int32)), ("ft_face", C.POINTER(C.c_int32)),
        ("ft_nbr_cell", C.POINTER(C.c_int32)), ("ft_nbr_face", C.POINTER(C.c_int32)),
        ("ft_bc", C.POINTER(C.c_int32)), ("ft_nbr_fdof", C.POINTER(C.c_int32)),
        ("ft_normal", C.POINTER(C.c_double)), ("ft_xyz", C.POINTER(C.c_double)),
        ("gauss_interp", C.POINTER(C.c_double)), ("q_wJ", C.POINTER(C.c_double)),
        ("q_xyz", C.POINTER(C.c_double)),
    ]


_host = None
_gpu = None
_GEOMETRY_GPU = re.compile(r"^\s*set\s+geometry\s+setup\s*=\s*gpu\s*(#.*)?$", re.MULTILINE | re.IGNORECASE)


def _load(name: str) -> C.CDLL:
    path = LIB_DIR / name
    if not path.exists():
        raise PlensError(f"{path} is missing: build it with __graft_entry__.build() or "
                         "python -m plens_gb300.build")
    return C.CDLL(str(path))


def host_lib() -> C.CDLL:
    global _host
    if _host is None:
        L = _load("libplens_host.so")
        vp, i64, dbl, i32 = C.c_void_p, C.c_int64, C.c_double, C.c_int32
        L.plens_case_create.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.POINTER(vp)]
        L.plens_case_create_ex.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, vp, C.POINTER(vp)]
        L.plens_case_last_error.restype = C.c_char_p
        L.plens_case_destroy.argtypes = [vp]
        L.plens_case_mesh.argtypes = [vp]
        L.plens_case_mesh.restype = vp
        L.plens_case_params.argtypes = [vp]
        L.plens_case_params.restype = vp
        L.plens_case_params_mut.argtypes = [vp]
        L.plens_case_params_mut.restype = C.POINTER(Params)
        L.plens_case_n_cells.argtypes = [vp]
        L.plens_case_n_cells.restype = i64
        L.plens_case_n_dofs.argtypes = [vp]
        L.plens_case_n_dofs.restype = i64
        L.plens_case_initial_state.argtypes = [vp, vp]
        L.plens_case_setup_times.argtypes = [vp, vp]
        L.plens_case_dof_xyz.argtypes = [vp, vp]
        L.plens_case_start_time.argtypes = [vp]
        L.plens_case_start_time.restype = dbl
        L.plens_case_end_time.argtypes = [vp]
        L.plens_case_end_time.restype = dbl
        L.plens_case_eval_expr.argtypes = [vp, i32, dbl, dbl, dbl, dbl]
        L.plens_case_eval_expr.restype = dbl
        L.plens_case_prm_echo.argtypes = [vp]
        L.plens_case_prm_echo.restype = C.c_char_p
        L.plens_expr_eval_string.argtypes = [C.c_char_p, dbl, dbl, dbl, dbl, C.POINTER(dbl)]
        L.plens_gll_1d.argtypes = [C.c_int, vp, vp]
        L.plens_write_vtu.argtypes = [vp, C.c_char_p, vp, vp, vp, vp, dbl]
        L.plens_write_pvd.argtypes = [C.c_char_p, i64, vp, C.POINTER(C.c_char_p)]
        L.plens_write_archive.argtypes = [vp, C.c_char_p, vp, dbl, i64, i64]
        L.plens_read_archive.argtypes = [vp, C.c_char_p, vp, C.POINTER(dbl), C.POINTER(i64), C.POINTER(i64)]
        _host = L
    return _host


def gpu_lib() -> C.CDLL:
    """The CUDA library. Raises if it was not built: there is no CPU fallback for the hot path."""
    global _gpu
    if _gpu is None:
        L = _load("libplens_gpu.so")
        vp, i64, dbl, i32 = C.c_void_p, C.c_int64, C.c_double, C.c_int32
        L.plens_gpu_create.argtypes = [vp, vp, C.POINTER(vp)]
        L.plens_gpu_destroy.argtypes = [vp]
        L.plens_gpu_last_error.argtypes = [vp]
        L.plens_gpu_last_error.restype = C.c_char_p
        L.plens_gpu_kernel_launches.argtypes = [vp]
        L.plens_gpu_kernel_launches.restype = i64
        L.plens_gpu_stream.argtypes = [vp]
        L.plens_gpu_stream.restype = vp
        L.plens_gpu_set_state.argtypes = [vp, vp]
        L.plens_gpu_get_state.argtypes = [vp, vp]
        L.plens_gpu_set_time.argtypes = [vp, dbl, i64]
        L.plens_gpu_get_time.argtypes = [vp, C.POINTER(dbl), C.POINTER(i64), C.POINTER(dbl)]
        L.plens_gpu_rhs.argtypes = [vp, vp]
        L.plens_gpu_time_step.argtypes = [vp, C.POINTER(dbl)]
        L.plens_gpu_advance.argtypes = [vp, i64, dbl]
        L.plens_gpu_advance_async.argtypes = [vp, i64, dbl]
        L.plens_gpu_synchronize.argtypes = [vp]
        L.plens_gpu_advance_states.argtypes = [vp, i64, vp, vp, dbl, i64, dbl, vp]
        L.plens_gpu_get_cell_scalars.argtypes = [vp, vp, vp, vp]
        L.plens_gpu_error_norms.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.plens_gpu_get_avars.argtypes = [vp, vp]
        L.plens_gpu_troubled_cells.argtypes = [vp, vp, C.POINTER(i64)]
        L.plens_gpu_first_bad_dof.argtypes = [vp, C.POINTER(i64)]
        L.plens_gpu_set_sensor_weights.argtypes = [vp, vp]
        L.plens_gpu_sensor_stats.argtypes = [vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(dbl), C.POINTER(i64)]
        L.plens_gpu_sensor_pairs.argtypes = [vp, vp, vp]
        L.plens_gpu_mlp_train.argtypes = [vp, vp, i64, vp, i32, i32, C.c_float, C.c_float, C.c_uint64, vp]
        L.plens_gpu_mlp_loss_grad.argtypes = [vp, vp, i64, vp, C.c_float, C.POINTER(C.c_float), vp]
        L.plens_gpu_mlp_infer.argtypes = [vp, i64, vp, C.c_float, vp]
        L.plens_gpu_selftest_conversions.argtypes = [i64, C.c_uint64, C.POINTER(i64)]
        L.plens_gpu_snapshot_begin.argtypes = [vp]
        L.plens_gpu_set_sensor_tensor_cores.argtypes = [vp, C.c_int]
        L.plens_gpu_set_indicator_tensor_cores.argtypes = [vp, C.c_int]
        L.plens_gpu_set_list_decoding.argtypes = [vp, C.c_int]
        L.plens_gpu_snapshot_end.argtypes = [vp, vp, vp, vp, vp, C.POINTER(dbl), C.POINTER(i64), C.POINTER(dbl)]
        L.plens_gpu_set_kernel_timing.argtypes = [vp, C.c_int]
        L.plens_gpu_setup_geometry.argtypes = [vp]
        L.plens_gpu_kernel_timing.argtypes = [vp, C.POINTER(dbl), C.POINTER(i64)]
        _gpu = L
    return _gpu


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class Case:
    """input.prm text -> mesh description, parameters and initial state.

    The setup runs on the host; with ``set geometry setup = gpu`` in the prm's ``GB300``
    subsection the metric terms and face dofs are computed by the CUDA library's
    ``plens_gpu_setup_geometry`` (same bits), which must then be built."""

    def __init__(self, prm_text: str, fe_degree: int, mapping_degree: int = 2, base_dir: str = "."):
        L = host_lib()
        h = C.c_void_p()
        geometry = None
        # the CUDA library is loaded only when the prm asks for the GPU geometry job, so that a
        # host-only setup (and a CPU-only process) never maps it
        if _GEOMETRY_GPU.search(prm_text):
            geometry = C.cast(gpu_lib().plens_gpu_setup_geometry, C.c_void_p)
        rc = L.plens_case_create_ex(prm_text.encode(), str(base_dir).encode(), mapping_degree,
                                    fe_degree, geometry, C.byref(h))
        if rc != 0:
            raise PlensError(L.plens_case_last_error().decode())
        self._h = h
        self._L = L
        self.degree = fe_degree
        self.n_cells = L.plens_case_n_cells(h)
        self.n_dofs = L.plens_case_n_dofs(h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.plens_case_destroy(h)
            self._h = None

    @property
    def mesh_ptr(self) -> int:
        return self._L.plens_case_mesh(self._h)

    @property
    def params_ptr(self) -> int:
        return self._L.plens_case_params(self._h)

    @property
    def params(self) -> Params:
        return self._L.plens_case_params_mut(self._h).contents

    def mesh_arrays(self) -> dict:
        """Copies of the mesh-description arrays (metric terms, neighbour and face tables)."""
        m = C.cast(C.c_void_p(self.mesh_ptr), C.POINTER(MeshDesc)).contents
        P = m.degree + 1
        nd, nc, nt = self.n_dofs, m.n_cells, m.n_face_tasks
        arr = lambda p, n: np.ctypeslib.as_array(p, shape=(n,)).copy()  # noqa: E731
        return {
            "degree": m.degree, "n_cells": nc, "n_face_tasks": nt,
            "detJ": arr(m.detJ, nd), "Ja": arr(m.Ja, 9 * nd).reshape(3, 3, nd),
            "Jinv": arr(m.Jinv, 9 * nd).reshape(3, 3, nd), "h_min": arr(m.h_min, nc),
            "cell_center": arr(m.cell_center, 3 * nc).reshape(nc, 3),
            "cell_nbr": arr(m.cell_nbr, 6 * nc).reshape(nc, 6),
            "cell_face_bc": arr(m.cell_face_bc, 6 * nc).reshape(nc, 6),
            "ft_cell": arr(m.ft_cell, nt), "ft_face": arr(m.ft_face, nt),
            "ft_nbr_cell": arr(m.ft_nbr_cell, nt), "ft_nbr_face": arr(m.ft_nbr_face, nt),
            "ft_bc": arr(m.ft_bc, nt), "ft_nbr_fdof": arr(m.ft_nbr_fdof, nt * P * P).reshape(nt, P * P),
            "ft_normal": arr(m.ft_normal, nt * P * P * 3).reshape(nt, P * P, 3),
            "ft_xyz": arr(m.ft_xyz, nt * P * P * 3).reshape(nt, P * P, 3),
            "gauss_interp": arr(m.gauss_interp, P * P).reshape(P, P) if m.gauss_interp else None,
            "q_wJ": arr(m.q_wJ, nd) if m.q_wJ else None,
            "q_xyz": arr(m.q_xyz, 3 * nd).reshape(3, nd) if m.q_xyz else None,
        }

    def setup_times(self) -> dict:
        """Wall seconds of the setup phases (mesh, geometry, topology, initial condition)."""
        t = np.zeros(4)
        self._L.plens_case_setup_times(self._h, _ptr(t))
        return dict(zip(("mesh", "geometry", "topology", "initial_condition"), t.tolist()))

    def initial_state(self) -> np.ndarray:
        U = np.empty((5, self.n_dofs), dtype=np.float64)
        self._L.plens_case_initial_state(self._h, _ptr(U))
        return U

    def dof_xyz(self) -> np.ndarray:
        X = np.empty((3, self.n_dofs), dtype=np.float64)
        self._L.plens_case_dof_xyz(self._h, _ptr(X))
        return X

    @property
    def start_time(self) -> float:
        return self._L.plens_case_start_time(self._h)

    @property
    def end_time(self) -> float:
        return self._L.plens_case_end_time(self._h)

    def eval_expr(self, idx: int, x=0.0, y=0.0, z=0.0, t=0.0) -> float:
        return self._L.plens_case_eval_expr(self._h, idx, x, y, z, t)

    def prm_echo(self) -> str:
        return self._L.plens_case_prm_echo(self._h).decode()

    def _hcheck(self, rc: int):
        if rc != 0:
            raise PlensError(self._L.plens_case_last_error().decode())

    def write_vtu(self, path, U, avars=None, alpha=None, alpha_d=None, loc_dt=0.0):
        """PLENS::write of one snapshot: a .vtu of the GLL nodes with rho, p, T, u, v, w (and the
        auxiliary variables), alpha, alpha_d and loc_dt as cell data."""
        arrs = [np.ascontiguousarray(a, dtype=np.float64) if a is not None else None for a in (U, avars, alpha, alpha_d)]
        ptrs = [_ptr(a) if a is not None else None for a in arrs]
        self._hcheck(self._L.plens_write_vtu(self._h, str(path).encode(), ptrs[0], ptrs[1], ptrs[2], ptrs[3], loc_dt))

    def write_archive(self, path, U, time: float, n_steps: int = 0, output_counter: int = 0):
        U = np.ascontiguousarray(U, dtype=np.float64)
        self._hcheck(self._L.plens_write_archive(self._h, str(path).encode(), _ptr(U), time, n_steps, output_counter))

    def read_archive(self, path):
        U = np.empty((5, self.n_dofs), dtype=np.float64)
        t, n, k = C.c_double(), C.c_int64(), C.c_int64()
        self._hcheck(self._L.plens_read_archive(self._h, str(path).encode(), _ptr(U), C.byref(t), C.byref(n), C.byref(k)))
        return U, t.value, n.value, k.value


def write_pvd(path, entries):
    """ParaView collection record of (time, file name) pairs."""
    L = host_lib()
    times = np.array([e[0] for e in entries], dtype=np.float64)
    names = (C.c_char_p * max(len(entries), 1))(*[str(e[1]).encode() for e in entries])
    if L.plens_write_pvd(str(path).encode(), len(entries), _ptr(times), names) != 0:
        raise PlensError(L.plens_case_last_error().decode())


def eval_expression(src: str, x=0.0, y=0.0, z=0.0, t=0.0) -> float:
    L = host_lib()
    out = C.c_double()
    if L.plens_expr_eval_string(src.encode(), x, y, z, t, C.byref(out)) != 0:
        raise PlensError(L.plens_case_last_error().decode())
    return out.value


def gll_1d(n: int):
    x = np.empty(n)
    w = np.empty(n)
    if host_lib().plens_gll_1d(n, _ptr(x), _ptr(w)) != 0:
        raise PlensError(host_lib().plens_case_last_error().decode())
    return x, w


class GpuSolver:
    """The GPU hot path for one Case (plens_gpu_create ... plens_gpu_destroy)."""

    def __init__(self, case: Case):
        self.L = gpu_lib()
        self.case = case
        h = C.c_void_p()
        rc = self.L.plens_gpu_create(case.mesh_ptr, case.params_ptr, C.byref(h))
        if rc != 0:
            msg = self.L.plens_gpu_last_error(h).decode() if h else "plens_gpu_create failed"
            raise PlensError(f"plens_gpu_create: {msg} (status {rc})")
        self.h = h
        self.n_dofs = case.n_dofs
        self.n_cells = case.n_cells

    def close(self):
        if getattr(self, "h", None):
            self.L.plens_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, rc: int, what: str):
        if rc == PLENS_GPU_OK:
            return
        msg = self.L.plens_gpu_last_error(self.h).decode()
        if rc == PLENS_GPU_E_POSITIVITY:
            d = C.c_int64(-1)
            self.L.plens_gpu_first_bad_dof(self.h, C.byref(d))
            raise PositivityError(f"{what}: {msg}", d.value)
        raise PlensError(f"{what}: {msg} (status {rc})")

    @property
    def kernel_launches(self) -> int:
        return self.L.plens_gpu_kernel_launches(self.h)

    @property
    def stream(self) -> int:
        return self.L.plens_gpu_stream(self.h) or 0

    def set_state(self, U: np.ndarray, t: float | None = None, n_steps: int = 0):
        U = np.ascontiguousarray(U, dtype=np.float64)
        assert U.shape == (5, self.n_dofs)
        self._check(self.L.plens_gpu_set_state(self.h, _ptr(U)), "set_state")
        if t is not None:
            self._check(self.L.plens_gpu_set_time(self.h, t, n_steps), "set_time")

    def get_state(self, out: np.ndarray | None = None) -> np.ndarray:
        U = out if out is not None else np.empty((5, self.n_dofs))
        self._check(self.L.plens_gpu_get_state(self.h, _ptr(U)), "get_state")
        return U

    def get_time(self):
        t, n, dt = C.c_double(), C.c_int64(), C.c_double()
        self._check(self.L.plens_gpu_get_time(self.h, C.byref(t), C.byref(n), C.byref(dt)), "get_time")
        return t.value, n.value, dt.value

    def rhs(self) -> np.ndarray:
        R = np.empty((5, self.n_dofs))
        self._check(self.L.plens_gpu_rhs(self.h, _ptr(R)), "rhs")
        return R

    def time_step(self) -> float:
        dt = C.c_double()
        self._check(self.L.plens_gpu_time_step(self.h, C.byref(dt)), "time_step")
        return dt.value

    def advance(self, n_steps: int, end_time: float = 1e300):
        self._check(self.L.plens_gpu_advance(self.h, n_steps, end_time), "advance")

    def advance_async(self, n_steps: int, end_time: float = 1e300):
        self._check(self.L.plens_gpu_advance_async(self.h, n_steps, end_time), "advance_async")

    def synchronize(self):
        self._check(self.L.plens_gpu_synchronize(self.h), "synchronize")

    def advance_states(self, U_in, U_out, t0: float, n_steps: int, end_time: float = 1e300) -> np.ndarray:
        """Advance each state of the sequence U_in ([5][ndof] FP64 host arrays) from time t0 by
        n_steps steps into the matching array of U_out, with the host transfers overlapping the
        steps (plens_gpu_advance_states; page-locked arrays give the overlap). Returns each
        member's clock."""
        n = len(U_in)
        assert len(U_out) == n
        for U in list(U_in) + list(U_out):
            assert U.dtype == np.float64 and U.shape == (5, self.n_dofs) and U.flags.c_contiguous
        pin = (C.c_void_p * max(n, 1))(*[_ptr(U) for U in U_in])
        pout = (C.c_void_p * max(n, 1))(*[_ptr(U) for U in U_out])
        t = np.empty(max(n, 1))
        self._check(self.L.plens_gpu_advance_states(self.h, n, pin, pout, t0, n_steps, end_time, _ptr(t)),
                    "advance_states")
        return t[:n]

    def error_norms(self):
        """(steady-state error, convergence error) of the current state, as PLENS::write logs
        them; a norm not requested at setup is returned as None."""
        ss, cv = C.c_double(), C.c_double()
        p = self.case.params
        self._check(self.L.plens_gpu_error_norms(self.h, C.byref(ss) if p.calc_ss_error else None,
                                                  C.byref(cv) if p.calc_conv_error else None), "error_norms")
        return (ss.value if p.calc_ss_error else None), (cv.value if p.calc_conv_error else None)

    def cell_scalars(self):
        a = np.empty(self.n_cells)
        ad = np.empty(self.n_cells)
        dt = np.empty(self.n_cells)
        self._check(self.L.plens_gpu_get_cell_scalars(self.h, _ptr(a), _ptr(ad), _ptr(dt)), "cell_scalars")
        return a, ad, dt

    def troubled_cells(self) -> np.ndarray:
        """The compacted troubled-cell list of the last RHS (cells with alpha > 0, ascending)."""
        cells = np.empty(self.n_cells, dtype=np.int32)
        n = C.c_int64()
        self._check(self.L.plens_gpu_troubled_cells(self.h, _ptr(cells), C.byref(n)), "troubled_cells")
        return cells[:n.value].copy()

    def avars(self) -> np.ndarray:
        A = np.empty((9, self.n_dofs))
        self._check(self.L.plens_gpu_get_avars(self.h, _ptr(A)), "avars")
        return A

    def set_kernel_timing(self, enable: bool):
        self._check(self.L.plens_gpu_set_kernel_timing(self.h, 1 if enable else 0), "set_kernel_timing")

    def kernel_timing(self):
        ms, n = C.c_double(), C.c_int64()
        self._check(self.L.plens_gpu_kernel_timing(self.h, C.byref(ms), C.byref(n)), "kernel_timing")
        return ms.value, n.value

    def set_sensor_weights(self, params: np.ndarray):
        p = np.ascontiguousarray(params, dtype=np.float32)
        assert p.size == MLP_N_PARAMS
        self._check(self.L.plens_gpu_set_sensor_weights(self.h, _ptr(p)), "set_sensor_weights")

    def sensor_stats(self):
        j, f, lo = C.c_int64(), C.c_int64(), C.c_int64()
        e = C.c_double()
        self._check(self.L.plens_gpu_sensor_stats(self.h, C.byref(j), C.byref(f), C.byref(e), C.byref(lo)), "sensor_stats")
        return {"judged": j.value, "fallbacks": f.value, "max_alpha_err": e.value, "lo_cells_last": lo.value}

    def set_sensor_tensor_cores(self, enable: bool):
        """Learned sensor: hidden layers on the tensor cores or the CUDA cores (the default)."""
        self._check(self.L.plens_gpu_set_sensor_tensor_cores(self.h, 1 if enable else 0), "set_sensor_tensor_cores")

    def set_indicator_tensor_cores(self, enable: bool):
        """Mixed form, degree 3, modal indicator: the change of basis on the tensor cores."""
        self._check(self.L.plens_gpu_set_indicator_tensor_cores(self.h, 1 if enable else 0), "set_indicator_tensor_cores")

    def set_list_decoding(self, enable: bool):
        """Mixed forms, troubled-cell list: positions decoded in the subcell kernel (the default
        where it fits) or the list written first by a list kernel."""
        self._check(self.L.plens_gpu_set_list_decoding(self.h, 1 if enable else 0), "set_list_decoding")

    def snapshot_begin(self):
        """Start an asynchronous snapshot (state, alpha, alpha_d, auxiliary variables, clock)."""
        self._check(self.L.plens_gpu_snapshot_begin(self.h), "snapshot_begin")

    def snapshot_end(self) -> dict:
        U = np.empty((5, self.n_dofs))
        a = np.empty(self.n_cells)
        ad = np.empty(self.n_cells)
        av = np.empty((9, self.n_dofs))
        t, n, dt = C.c_double(), C.c_int64(), C.c_double()
        self._check(self.L.plens_gpu_snapshot_end(self.h, _ptr(U), _ptr(a), _ptr(ad), _ptr(av), C.byref(t),
                                                  C.byref(n), C.byref(dt)), "snapshot_end")
        return {"U": U, "alpha": a, "alpha_d": ad, "avars": av, "time": t.value, "n_steps": n.value, "dt": dt.value}

    def sensor_pairs(self):
        x = np.empty((self.n_cells, 64), dtype=np.float32)
        y = np.empty(self.n_cells, dtype=np.float32)
        self._check(self.L.plens_gpu_sensor_pairs(self.h, _ptr(x), _ptr(y)), "sensor_pairs")
        return x, y


def mlp_train(x: np.ndarray, y: np.ndarray, params: np.ndarray, epochs=20, batch=4096, lr=1e-3,
              alpha_max=0.5, seed=0):
    L = gpu_lib()
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    p = np.ascontiguousarray(params, dtype=np.float32).copy()
    loss = np.zeros(epochs, dtype=np.float32)
    rc = L.plens_gpu_mlp_train(_ptr(x), _ptr(y), len(y), _ptr(p), epochs, batch, lr, alpha_max, seed, _ptr(loss))
    if rc != 0:
        raise PlensError(f"plens_gpu_mlp_train failed with status {rc}")
    return p, loss


def mlp_loss_grad(x: np.ndarray, y: np.ndarray, params: np.ndarray, alpha_max=0.5):
    L = gpu_lib()
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    p = np.ascontiguousarray(params, dtype=np.float32)
    g = np.zeros(MLP_N_PARAMS, dtype=np.float32)
    loss = C.c_float()
    rc = L.plens_gpu_mlp_loss_grad(_ptr(x), _ptr(y), len(y), _ptr(p), alpha_max, C.byref(loss), _ptr(g))
    if rc != 0:
        raise PlensError(f"plens_gpu_mlp_loss_grad failed with status {rc}")
    return loss.value, g


def mlp_infer(x: np.ndarray, params: np.ndarray, alpha_max=0.5) -> np.ndarray:
    L = gpu_lib()
    x = np.ascontiguousarray(x, dtype=np.float32)
    p = np.ascontiguousarray(params, dtype=np.float32)
    out = np.empty(x.shape[0], dtype=np.float32)
    rc = L.plens_gpu_mlp_infer(_ptr(x), x.shape[0], _ptr(p), alpha_max, _ptr(out))
    if rc != 0:
        raise PlensError(f"plens_gpu_mlp_infer failed with status {rc}")
    return out


def selftest_conversions(n: int = 1 << 24, seed: int = 1) -> int:
    """Mismatches between the mixed form's integer-pipe FP64 <-> FP32 conversions and the
    hardware conversions over n seeded samples (0 when they agree)."""
    L = gpu_lib()
    bad = C.c_int64(0)
    rc = L.plens_gpu_selftest_conversions(n, seed, C.byref(bad))
    if rc != 0:
        raise PlensError(f"plens_gpu_selftest_conversions failed with status {rc}")
    return bad.value
