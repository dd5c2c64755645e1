"""The allocation-free time-step entry point (plens_gpu_time_step_noalloc) against the context
entry point plens_gpu_time_step, through the C ABI.

It exists for callers that may not allocate device memory (a framework that owns all GPU memory
through its own pool, or a loop that must not allocate while it runs): they pass device arrays
they already own and a device output, and the library uses its own file-scope device scratch.
The cases cover the inviscid step (degrees 1, 3 and 5, which change how many cells a block
holds), Sutherland viscosity on the curved cylinder mesh and constant viscosity on the periodic
shock-vortex box. This file is collected last so that a failure here stops a -x run only after
everything else.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import make
from plens_gb300 import configs
from plens_gb300.api import PLENS_GPU_E_CUDA, PLENS_GPU_E_INVALID, GpuSolver, gpu_lib

pytestmark = pytest.mark.gpu

MAX_CELLS = 1 << 18


def _fn():
    L = gpu_lib()
    f = L.plens_gpu_time_step_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_double,
                  C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


CASES = {
    "dmr_N3_inviscid": lambda: configs.dmr(nx=24, ny=6),
    "dmr_N1_inviscid": lambda: configs.dmr(nx=24, ny=6, degree=1),
    "dmr_N5_inviscid": lambda: configs.dmr(nx=12, ny=3, degree=5),
    "cylinder_sutherland": lambda: configs.cylinder(n_radial=8, n_azimuthal=16),
    "shock_vortex_const_mu": lambda: configs.shock_vortex(n=4, modes=2),
}


@pytest.mark.parametrize("name", list(CASES))
def test_time_step_noalloc_matches_context_entry_point(name):
    import torch

    f = _fn()
    case = make(CASES[name]())
    m = case.mesh_arrays()
    g = GpuSolver(case)
    g.set_state(case.initial_state(), 0.0)
    dev = torch.device("cuda", 0)
    d_jinv = torch.from_numpy(np.ascontiguousarray(m["Jinv"].reshape(9, -1))).to(dev)
    d_h = torch.from_numpy(m["h_min"]).to(dev)
    d_out = torch.full((1,), -1.0, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    courant = case.eval_expr(case.params.expr_courant)
    for call in range(2):
        if call == 1:
            g.advance(2)  # a different state for the second call
        U = g.get_state()
        dt_ref = g.time_step()
        d_u = torch.from_numpy(U).to(dev)
        torch.cuda.synchronize()
        rc = f(d_u.data_ptr(), d_jinv.data_ptr(), d_h.data_ptr(), case.n_cells, case.degree, case.params_ptr,
               courant, d_out.data_ptr(), stream.cuda_stream)
        assert rc == 0, gpu_lib().plens_gpu_last_error(None).decode()
        torch.cuda.synchronize()
        assert d_out.item() == pytest.approx(dt_ref, rel=1e-13, abs=0)


def test_time_step_noalloc_rejects_meshes_beyond_its_scratch():
    import torch

    f = _fn()
    case = make(configs.sod(n=4))
    dev = torch.device("cuda", 0)
    d = torch.zeros(16, dtype=torch.float64, device=dev)
    rc = f(d.data_ptr(), d.data_ptr(), d.data_ptr(), MAX_CELLS + 1, case.degree, case.params_ptr, 0.5,
           d.data_ptr(), None)
    assert rc == PLENS_GPU_E_INVALID
    assert b"scratch" in gpu_lib().plens_gpu_last_error(None)
    assert rc != PLENS_GPU_E_CUDA
