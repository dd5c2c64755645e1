"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Tolerances (plain FP64 form):
- one RHS evaluation: max over equations of max|R_gpu - R_oracle| / max|R_oracle| <= 1e-12;
- after 100 time steps: relative L1 of rho, momentum and rho E <= 1e-10.
Mixed form (FP32 flux differencing, FP64 state and registers): relative L1 of rho <= 1e-4.
"""
import numpy as np
import pytest

from helpers import make, max_rel_err, rel_l1
from oracle.pyoracle import Oracle
from plens_gb300 import configs
from plens_gb300.api import GpuSolver, PositivityError

RHS_TOL = 1e-12
STEPS_TOL = 1e-10

pytestmark = pytest.mark.gpu


def _rhs_pair(case, U, t=0.0):
    o = Oracle(case)
    o.set_state(U, t)
    Ro, ao, ado = o.rhs()
    g = GpuSolver(case)
    g.set_state(U, t)
    Rg = g.rhs()
    ag, adg, _ = g.cell_scalars()
    return Ro, Rg, ao, ag, ado, adg, g


def _evolved_state(case, steps):
    o = Oracle(case)
    o.set_state(case.initial_state(), case.start_time)
    o.advance(steps)
    U, t, _, _ = o.get_state()
    return U, t


def test_sod_rhs_parity():
    case = make(configs.sod(n=40))
    for steps in (0, 15):
        U, t = _evolved_state(case, steps)
        Ro, Rg, ao, ag, _, _, g = _rhs_pair(case, U, t)
        assert g.kernel_launches > 0
        np.testing.assert_allclose(ag, ao, rtol=0, atol=1e-12)
        if steps:
            assert (ao > 0).any(), "evolved Sod state should have troubled cells"
        assert max_rel_err(Rg, Ro) <= RHS_TOL


def test_sod_time_step_parity():
    case = make(configs.sod(n=40))
    U, t = _evolved_state(case, 5)
    o = Oracle(case)
    o.set_state(U, t)
    g = GpuSolver(case)
    g.set_state(U, t)
    assert abs(g.time_step() - o.time_step()) <= 1e-14 * o.time_step()


def test_sod_100_steps_parity():
    """Config 1 at full size: 200x1x1 cells, N=2, 100 steps."""
    case = make(configs.sod(n=200))
    U0 = case.initial_state()
    o = Oracle(case)
    o.set_state(U0, 0.0)
    o.advance(100)
    Uo, to, no, _ = o.get_state()
    g = GpuSolver(case)
    g.set_state(U0, 0.0)
    g.advance(100)
    Ug = g.get_state()
    tg, ng, _ = g.get_time()
    assert ng == no == 100
    assert abs(tg - to) <= 1e-12 * to
    assert rel_l1(Ug, Uo).max() <= STEPS_TOL


def test_dmr_rhs_and_steps_parity():
    case = make(configs.dmr(nx=24, ny=6))
    U, t = _evolved_state(case, 3)
    Ro, Rg, ao, ag, _, _, _ = _rhs_pair(case, U, t)
    assert (ao > 0).any()
    np.testing.assert_allclose(ag, ao, rtol=0, atol=1e-12)
    assert max_rel_err(Rg, Ro) <= RHS_TOL
    # 10 steps from the initial condition
    o = Oracle(case)
    o.set_state(case.initial_state(), 0.0)
    o.advance(10)
    Uo = o.get_state()[0]
    g = GpuSolver(case)
    g.set_state(case.initial_state(), 0.0)
    g.advance(10)
    assert rel_l1(g.get_state(), Uo).max() <= STEPS_TOL


def test_end_time_clip_matches():
    """The last step's dt is clipped for the clock only (update_rk4, dgsem/plens.cc:4341)."""
    case = make(configs.sod(n=20, end_time=0.003))
    o = Oracle(case)
    o.set_state(case.initial_state(), 0.0)
    o.advance(1000, 0.003)
    Uo, to, no, _ = o.get_state()
    g = GpuSolver(case)
    g.set_state(case.initial_state(), 0.0)
    g.advance(1000, 0.003)
    tg, ng, _ = g.get_time()
    assert ng == no and abs(tg - 0.003) < 1e-15 and abs(to - 0.003) < 1e-15
    assert rel_l1(g.get_state(), Uo).max() <= STEPS_TOL


@pytest.mark.parametrize("scheme", ["Rusanov", "AUSM+-up", "Rusanov-HLLC", "Chandrashekhar", "Modified SW"])
def test_surface_schemes_rhs_parity(scheme):
    prm, files, deg = configs.sod(n=20)
    prm = prm.replace("set inviscid surface flux scheme = HLLC", f"set inviscid surface flux scheme = {scheme}")
    case = make((prm, files, deg))
    U, t = _evolved_state(case, 10)
    Ro, Rg, *_ = _rhs_pair(case, U, t)
    assert max_rel_err(Rg, Ro) <= RHS_TOL


@pytest.mark.parametrize("scheme", ["KG", "IR"])
def test_volume_schemes_rhs_parity(scheme):
    prm, files, deg = configs.dmr(nx=8, ny=4)
    prm = prm.replace("set inviscid volume flux scheme = Chandrashekhar", f"set inviscid volume flux scheme = {scheme}")
    case = make((prm, files, deg))
    U, t = _evolved_state(case, 2)
    Ro, Rg, *_ = _rhs_pair(case, U, t)
    assert max_rel_err(Rg, Ro) <= RHS_TOL


def test_rk3_steps_parity():
    prm, files, deg = configs.sod(n=40)
    prm = prm.replace("set RK order = 4", "set RK order = 3")
    case = make((prm, files, deg))
    o = Oracle(case)
    o.set_state(case.initial_state(), 0.0)
    o.advance(20)
    g = GpuSolver(case)
    g.set_state(case.initial_state(), 0.0)
    g.advance(20)
    assert rel_l1(g.get_state(), o.get_state()[0]).max() <= STEPS_TOL


def test_viscous_cylinder_rhs_parity():
    """Curved O-mesh (cylinder manifold), BR1 viscous terms, Sutherland, isothermal wall."""
    case = make(configs.cylinder(n_radial=6, n_azimuthal=12))
    U, t = _evolved_state(case, 2)
    o = Oracle(case)
    o.set_state(U, t)
    Ro, ao, _, Ao = o.rhs(with_avars=True)
    g = GpuSolver(case)
    g.set_state(U, t)
    Rg = g.rhs()
    Ag = g.avars()
    # stress components measured against the largest stress, heat-flux components against the
    # largest heat flux (z components are round-off noise in this 2D flow)
    d = np.abs(Ag - Ao)
    assert d[:6].max() / np.abs(Ao[:6]).max() <= RHS_TOL
    assert d[6:].max() / np.abs(Ao[6:]).max() <= RHS_TOL
    assert max_rel_err(Rg, Ro) <= RHS_TOL


def test_viscous_shock_vortex_rhs_and_steps_parity():
    case = make(configs.shock_vortex(n=3, modes=2))
    U = case.initial_state()
    Ro, Rg, *_ = _rhs_pair(case, U, 0.0)
    assert max_rel_err(Rg, Ro) <= RHS_TOL
    o = Oracle(case)
    o.set_state(U, 0.0)
    o.advance(3)
    g = GpuSolver(case)
    g.set_state(U, 0.0)
    g.advance(3)
    assert rel_l1(g.get_state(), o.get_state()[0]).max() <= STEPS_TOL


def test_positivity_failure_reports_first_bad_dof():
    """A state with rho < 0 at two dofs: the GPU path returns PLENS_GPU_E_POSITIVITY with the
    first offending dof (the reference prints it and exits, dgsem/plens.cc:2531-2546)."""
    case = make(configs.sod(n=10))
    U = case.initial_state()
    U[0, 37] = -1.0
    U[0, 101] = -2.0
    g = GpuSolver(case)
    g.set_state(U)
    with pytest.raises(PositivityError) as ei:
        g.rhs()
    assert ei.value.dof == 37
    # the context stays usable after the error
    g.set_state(case.initial_state(), 0.0)
    g.rhs()


@pytest.mark.parametrize("prec", ["mixed", "mixed_r32"])
def test_mixed_precision_dmr_error_bound(prec):
    """FP32 flux differencing (with FP64 registers and metric terms in "mixed", FP32 registers and
    metric images in "mixed_r32"): rho relative L1 vs the FP64 oracle <= 1e-4."""
    spec_fp64 = configs.dmr(nx=24, ny=6)
    spec_mixed = configs.dmr(nx=24, ny=6, precision=prec)
    c64 = make(spec_fp64)
    cmx = make(spec_mixed)
    o = Oracle(c64)
    o.set_state(c64.initial_state(), 0.0)
    o.advance(20)
    Uo = o.get_state()[0]
    g = GpuSolver(cmx)
    g.set_state(cmx.initial_state(), 0.0)
    g.advance(20)
    err = rel_l1(g.get_state(), Uo)
    assert err[0] <= 1e-4, err
