"""Parity with the oracle at the configurations' full sizes (the FP64 form), and the mixed form's
accuracy bound at full size.

- double Mach reflection, 240x60x1 cells, N=3 (921,600 DoFs): one RHS <= 1e-12 and 100 steps
  <= 1e-10 relative L1 (rho, momentum, rho E); the mixed form with the learned sensor keeps rho
  within 1e-4 relative L1 of the FP64 form after the same 100 steps (momentum and rho E printed);
- Mach-8 cylinder, 160x128x1 cells, N=3 (1,310,720 DoFs, viscous, curved): one RHS <= 1e-12 with
  the auxiliary variables, 10 steps <= 1e-10;
- shock-vortex box, 64^3 cells, N=3 (16.8 M DoFs, viscous, constant mu): one RHS <= 1e-12 and
  one step <= 1e-10.
The oracle runs on all host cores (OpenMP).
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


def _weights():
    from pathlib import Path
    p = Path(__file__).resolve().parent.parent / "plens_gb300" / "sensor_weights.bin"
    return np.fromfile(p, dtype=np.float32)


def _rhs_check(case, U, t, with_avars=False):
    o = Oracle(case)
    o.set_state(U, t)
    out = o.rhs(with_avars=with_avars)
    g = GpuSolver(case)
    g.set_state(U, t)
    Rg = g.rhs()
    assert max_rel_err(Rg, out[0]) <= RHS_TOL
    ag, _, _ = g.cell_scalars()
    np.testing.assert_allclose(ag, out[1], rtol=0, atol=1e-12)
    if with_avars:
        Ao, Ag = out[3], g.avars()
        d = np.abs(Ag - Ao)
        assert d[:6].max() / np.abs(Ao[:6]).max() <= RHS_TOL
        assert d[6:].max() / np.abs(Ao[6:]).max() <= RHS_TOL
    return o, g


def test_dmr_full_size_fp64_and_mixed_learned():
    case = make(configs.dmr())
    assert case.n_dofs == 921600
    U0 = case.initial_state()
    o, g = _rhs_check(case, U0, 0.0)
    o.set_state(U0, 0.0)
    o.advance(100)
    Uo = o.get_state()[0]
    g.set_state(U0, 0.0)
    g.advance(100)
    Ug = g.get_state()
    e = rel_l1(Ug, Uo)
    print(f"DMR full size, 100 steps, FP64 GPU vs oracle rel L1 (rho, momentum, rhoE): {e}")
    assert e.max() <= STEPS_TOL
    g.close()
    cmx = make(configs.dmr(precision="mixed", sensor="learned"))
    gm = GpuSolver(cmx)
    gm.set_sensor_weights(_weights())
    gm.set_state(U0, 0.0)
    gm.advance(100)
    em = rel_l1(gm.get_state(), Ug)
    print(f"DMR full size, 100 steps, mixed + learned sensor vs FP64 rel L1 (rho, momentum, rhoE): {em}")
    assert em[0] <= 1e-4


def test_cylinder_full_size():
    case = make(configs.cylinder())
    assert case.n_dofs == 1310720
    U0 = case.initial_state()
    o, g = _rhs_check(case, U0, 0.0, with_avars=True)
    o.set_state(U0, 0.0)
    o.advance(10)
    g.set_state(U0, 0.0)
    g.advance(10)
    e = rel_l1(g.get_state(), o.get_state()[0])
    print(f"cylinder full size, 10 steps rel L1: {e}")
    assert e.max() <= STEPS_TOL


def test_shock_vortex_full_size():
    case = make(configs.shock_vortex())
    assert case.n_dofs == 64 ** 3 * 64
    U0 = case.initial_state()
    o, g = _rhs_check(case, U0, 0.0)
    o.set_state(U0, 0.0)
    o.advance(1)
    g.set_state(U0, 0.0)
    g.advance(1)
    e = rel_l1(g.get_state(), o.get_state()[0])
    print(f"shock-vortex 64^3, 1 step rel L1: {e}")
    assert e.max() <= STEPS_TOL
