"""Parity of the GPU boundary-condition ghosts with the oracle for the BC types the configurations
do not use: symmetry (inviscid and viscous), empty, insulated wall and ZPG inflow
(IBCs/symmetry.cc:17-98, IBCs/empty.cc:15-91, IBCs/insulated_wall.cc:17-102,
IBCs/zpg_inflow.cc:9-55), through one RHS (auxiliary variables included on the viscous cases)
and a few steps. Tolerances as in test_gpu_parity: one RHS <= 1e-12 of each equation's largest
residual, steps <= 1e-10 relative L1.
"""
import numpy as np
import pytest

from helpers import make, max_rel_err, rel_l1
from oracle.pyoracle import Oracle
from plens_gb300 import configs
from plens_gb300.api import GpuSolver

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12
STEPS_TOL = 1e-10


def _evolved(case, steps):
    o = Oracle(case)
    o.set_state(case.initial_state(), case.start_time)
    o.advance(steps)
    U, t, _, _ = o.get_state()
    return U, t


def _check(case, pre_steps=2, steps=5, viscous=True):
    U, t = _evolved(case, pre_steps)
    o = Oracle(case)
    o.set_state(U, t)
    if viscous:
        Ro, ao, _, Ao = o.rhs(with_avars=True)
    else:
        Ro, ao, _ = o.rhs()
    g = GpuSolver(case)
    g.set_state(U, t)
    Rg = g.rhs()
    ag, _, _ = g.cell_scalars()
    assert max_rel_err(Rg, Ro) <= RHS_TOL
    np.testing.assert_allclose(ag, ao, rtol=0, atol=1e-12)
    if viscous:
        Ag = g.avars()
        d = np.abs(Ag - Ao)
        assert d[:6].max() / np.abs(Ao[:6]).max() <= RHS_TOL
        assert d[6:].max() / np.abs(Ao[6:]).max() <= RHS_TOL
    o.set_state(U, t)
    o.advance(steps)
    g.set_state(U, t)
    g.advance(steps)
    assert rel_l1(g.get_state(), o.get_state()[0]).max() <= STEPS_TOL


def test_symmetry_inviscid_dmr():
    """The reference's own DMR z boundaries (study1/dmr/scripts/base_input.prm:43-48)."""
    _check(make(configs.dmr(nx=24, ny=6, z_bc="symmetry")), pre_steps=3, steps=10, viscous=False)


@pytest.mark.parametrize("z_bc", ["symmetry", "empty"])
def test_symmetry_and_empty_viscous(z_bc):
    _check(make(configs.cylinder(n_radial=6, n_azimuthal=12, z_bc=z_bc)))


def test_insulated_wall_viscous():
    _check(make(configs.cylinder(n_radial=6, n_azimuthal=12, wall_bc="insulated wall")))


def test_zpg_inflow_viscous():
    _check(make(configs.cylinder(n_radial=6, n_azimuthal=12, inflow_bc="ZPG inflow")))
