"""Local time stepping on the GPU (calc_time_step, dgsem/plens.cc:3876-3911, and the per-cell
multiply_time_step_to_rhs, 3925-3940) against the oracle, on the wall-clustered cylinder O-mesh
(viscous, Mach 8), where the cell steps span orders of magnitude.

Tolerances: the per-cell steps of the plain FP64 form match the oracle's to 1e-13 relative (they
are minima of the same per-dof bounds); the state after the steps to the parity bar of the global
stepping, relative L1 <= 1e-10; the mixed form's rho to 1e-4 relative L1 of the FP64 form."""
import numpy as np
import pytest

from helpers import make, rel_l1
from oracle.pyoracle import Oracle
from plens_gb300 import configs
from plens_gb300.api import GpuSolver

pytestmark = pytest.mark.gpu

LOCAL = dict(start=0.0, limit=True, neighbor=1.05, global_=50.0)


def _spec(precision="fp64", local=LOCAL):
    return configs.cylinder(n_radial=8, n_azimuthal=16, precision=precision, local=local)


def test_cell_steps_and_state_match_oracle():
    case = make(_spec())
    o = Oracle(case)
    o.set_state(case.initial_state(), 0.0)
    g = GpuSolver(case)
    g.set_state(case.initial_state(), 0.0)
    for steps in (1, 4, 15):  # the first step (t = 0) is global, the rest local
        o.advance(steps)
        g.advance(steps)
        loc_o = o.loc_time_steps()
        _, _, loc_g = g.cell_scalars()
        np.testing.assert_allclose(loc_g, loc_o, rtol=1e-13, atol=0)
    assert loc_o.max() > 2 * loc_o.min()
    Uo, to, _, _ = o.get_state()
    assert rel_l1(g.get_state(), Uo).max() <= 1e-10
    assert g.get_time()[0] == pytest.approx(to, rel=1e-13)


def test_unlimited_local_steps_match_oracle():
    case = make(_spec(local=dict(start=0.0, limit=False)))
    o = Oracle(case)
    o.set_state(case.initial_state(), 0.0)
    o.advance(6)
    g = GpuSolver(case)
    g.set_state(case.initial_state(), 0.0)
    g.advance(6)
    np.testing.assert_allclose(g.cell_scalars()[2], o.loc_time_steps(), rtol=1e-13, atol=0)
    assert rel_l1(g.get_state(), o.get_state()[0]).max() <= 1e-10


def test_mixed_form_local_steps():
    c64, cmx = make(_spec()), make(_spec("mixed"))
    o = Oracle(c64)
    o.set_state(c64.initial_state(), 0.0)
    o.advance(30)
    g = GpuSolver(cmx)
    g.set_state(cmx.initial_state(), 0.0)
    g.advance(30)
    assert rel_l1(g.get_state(), o.get_state()[0])[0] <= 1e-4
    # FP32 per-dof bounds: the cell steps agree to FP32 rounding
    np.testing.assert_allclose(g.cell_scalars()[2], o.loc_time_steps(), rtol=1e-5, atol=0)
