"""ctypes wrapper of the CPU oracle (test infrastructure; see oracle.cpp's header).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs import this.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        vp, i64, dbl = C.c_void_p, C.c_int64, C.c_double
        L.oracle_create.argtypes = [vp, vp]
        L.oracle_create.restype = vp
        L.oracle_destroy.argtypes = [vp]
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_max_threads.restype = C.c_int
        L.oracle_set_state.argtypes = [vp, vp, dbl, i64]
        L.oracle_get_state.argtypes = [vp, vp, C.POINTER(dbl), C.POINTER(i64), C.POINTER(dbl)]
        L.oracle_rhs.argtypes = [vp, vp, vp, vp, vp]
        L.oracle_time_step.argtypes = [vp, C.POINTER(dbl)]
        L.oracle_loc_time_steps.argtypes = [vp, vp]
        L.oracle_error_norms.argtypes = [vp, C.POINTER(dbl), C.POINTER(dbl)]
        L.oracle_advance.argtypes = [vp, i64, dbl]
        L.oracle_first_bad_dof.argtypes = [vp]
        L.oracle_first_bad_dof.restype = i64
        L.oracle_operators.argtypes = [vp, vp, vp, vp]
        L.oracle_flux.argtypes = [vp, C.c_int, vp, vp, vp, dbl, vp]
        L.oracle_cell_blender.argtypes = [vp, vp]
        L.oracle_cell_blender.restype = dbl
        _lib = L
    return _lib


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


class OracleError(RuntimeError):
    def __init__(self, msg, status, dof=-1):
        super().__init__(msg)
        self.status = status
        self.dof = dof


class Oracle:
    """FP64 CPU restatement of PLENS::calc_rhs / calc_time_step / update for one Case."""

    def __init__(self, case, threads: int | None = None):
        self.L = lib()
        if threads:
            self.L.oracle_set_threads(threads)
        self.h = self.L.oracle_create(case.mesh_ptr, case.params_ptr)
        if not self.h:
            raise OracleError("oracle_create failed", 1)
        self.case = case
        self.n_dofs = case.n_dofs
        self.n_cells = case.n_cells
        self.P = case.degree + 1

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.L.oracle_destroy(h)
            self.h = None

    def set_state(self, U, t=0.0, n_steps=0):
        U = np.ascontiguousarray(U, dtype=np.float64)
        self.L.oracle_set_state(self.h, _p(U), t, n_steps)

    def get_state(self):
        U = np.empty((5, self.n_dofs))
        t, dt = C.c_double(), C.c_double()
        n = C.c_int64()
        self.L.oracle_get_state(self.h, _p(U), C.byref(t), C.byref(n), C.byref(dt))
        return U, t.value, n.value, dt.value

    def _status(self, rc, what):
        if rc:
            raise OracleError(f"{what} failed with status {rc}", rc, self.L.oracle_first_bad_dof(self.h))

    def rhs(self, with_avars=False):
        R = np.empty((5, self.n_dofs))
        a = np.empty(self.n_cells)
        ad = np.empty(self.n_cells)
        av = np.empty((9, self.n_dofs)) if with_avars else None
        self._status(self.L.oracle_rhs(self.h, _p(R), _p(a), _p(ad), _p(av) if av is not None else None), "rhs")
        return (R, a, ad, av) if with_avars else (R, a, ad)

    def time_step(self):
        dt = C.c_double()
        self.L.oracle_time_step(self.h, C.byref(dt))
        return dt.value

    def loc_time_steps(self):
        """Per-cell factor of the RHS from the last time-step calculation (loc_time_steps)."""
        out = np.empty(self.n_cells)
        self._status(self.L.oracle_loc_time_steps(self.h, _p(out)), "loc_time_steps")
        return out

    def error_norms(self):
        """(steady-state error, convergence error) of the current state, as write() logs them."""
        ss, cv = C.c_double(), C.c_double()
        self._status(self.L.oracle_error_norms(self.h, C.byref(ss), C.byref(cv)), "error_norms")
        return ss.value, cv.value

    def advance(self, n_steps, end_time=1e300):
        self._status(self.L.oracle_advance(self.h, n_steps, end_time), "advance")

    def operators(self):
        P = self.P
        w = np.empty(P)
        D = np.empty((P, P))
        cbm = np.empty((P ** 3, P ** 3))
        self.L.oracle_operators(self.h, _p(w), _p(D), _p(cbm))
        return w, D, cbm

    def cell_blender(self, var):
        var = np.ascontiguousarray(var, dtype=np.float64)
        return self.L.oracle_cell_blender(self.h, _p(var))


def flux(params_ptr, which, left, right, normal, blender=1.0):
    """NavierStokes flux functions in isolation: which = 0 get_inv_surf_flux, 1 get_inv_vol_flux,
    2 hllc_xflux, 3 rusanov_xflux, 4 ausm_plus_up_xflux."""
    L = lib()
    l = np.ascontiguousarray(left, dtype=np.float64)
    r = np.ascontiguousarray(right, dtype=np.float64)
    n = np.ascontiguousarray(normal, dtype=np.float64)
    f = np.empty(5)
    if L.oracle_flux(params_ptr, which, _p(l), _p(r), _p(n), blender, _p(f)):
        raise OracleError("bad flux selector", 1)
    return f


def max_threads() -> int:
    return lib().oracle_max_threads()
