"""Error norms of the output steps (PLENS::write, dgsem/plens.cc:4234-4243) in the oracle:
calc_ss_error (3985-4035) and calc_convergence_error (4044-4098), L2 norms by QGauss(N+1).

Pins: the quadrature reproduces integrals of known polynomials on the straight box exactly and
the volume of the curved O-mesh annulus to the accuracy of its cubic mapping; the steady-state
error is recomputed from its definition with numpy (sum factorisation written independently
with einsum) from the two states and the per-cell steps."""
import math

import numpy as np
import pytest

from helpers import make
from oracle.pyoracle import Oracle
from plens_gb300 import configs


def _state_from_rho(case, rho, p=1.0):
    gamma = case.params.gamma
    U = np.zeros((5, case.n_dofs))
    U[0] = rho
    U[4] = p / (gamma - 1)
    return U


def test_conv_error_box_polynomial_exact():
    """rho = 1 + 2x against exact 0 on [0,1]x[0,0.005]^2: ||rho||^2 = A (1 + 2 + 4/3)."""
    case = make(configs.with_error_norms(configs.sod(n=8, noise=0.0), conv_exact="0"))
    x = case.dof_xyz()[0]
    o = Oracle(case)
    o.set_state(_state_from_rho(case, 1 + 2 * x), 0.0)
    _, conv = o.error_norms()
    A = 0.005 * 0.005
    assert conv == pytest.approx(math.sqrt(A * 13.0 / 3.0), rel=1e-13)


def test_conv_error_uses_time_and_location():
    """rho = 1 + x - exact(1 + x + t) at t = 0.25: ||0.25|| = 0.25 sqrt(A)."""
    case = make(configs.with_error_norms(configs.sod(n=6, noise=0.0), conv_exact="1 + x + t"))
    x = case.dof_xyz()[0]
    o = Oracle(case)
    o.set_state(_state_from_rho(case, 1 + x), 0.25)
    _, conv = o.error_norms()
    assert conv == pytest.approx(0.25 * 0.005, rel=1e-12)


def test_conv_error_annulus_volume():
    """Uniform rho = 1 against exact 0 on the cylinder O-mesh: sqrt of the annulus volume
    pi (10^2 - 1^2) 0.05, to the accuracy of the cubic cylinder mapping."""
    spec = configs.with_error_norms(configs.cylinder(n_radial=6, n_azimuthal=32), conv_exact="0")
    case = make(spec)
    o = Oracle(case)
    o.set_state(_state_from_rho(case, np.ones(case.n_dofs), p=1e4), 0.0)
    _, conv = o.error_norms()
    vol = math.pi * (100.0 - 1.0) * 0.05
    assert conv ** 2 == pytest.approx(vol, rel=1e-5)


def test_ss_error_matches_definition():
    case = make(configs.with_error_norms(configs.cylinder(n_radial=6, n_azimuthal=16,
                                                          local=dict(start=0.0, limit=True))))
    o = Oracle(case)
    o.set_state(case.initial_state(), 0.0)
    o.advance(2)
    U_prev_start = o.get_state()[0].copy()
    o.advance(1)
    U = o.get_state()[0]
    ss, conv = o.error_norms()
    assert conv == 0.0
    dt = o.loc_time_steps()  # recomputed at the current state by error_norms
    m = case.mesh_arrays()
    P = case.degree + 1
    G, wJ = m["gauss_interp"], m["q_wJ"].reshape(case.n_cells, P, P, P)
    nc = case.n_cells

    def norm2(f):  # f: [ndof] nodal -> sum over cells and Gauss points of w|J| f^2
        F = f.reshape(nc, P, P, P)  # (cell, k, j, i)
        Fq = np.einsum("ai,bj,ck,nkji->ncba", G, G, G, F)
        return float((wJ * Fq ** 2).sum())

    diff = (U[4] - U_prev_start[4]) / np.repeat(dt, P ** 3)
    expect = math.sqrt(norm2(diff)) / math.sqrt(norm2(U[4]))
    assert ss == pytest.approx(expect, rel=1e-12)
    assert 0 < ss < 1e3


def test_ss_error_before_the_first_step_uses_zero():
    """rhoE_old starts at zero: the first output's error is ||rho E / dt|| / ||rho E||."""
    case = make(configs.with_error_norms(configs.sod(n=8, noise=0.0)))
    o = Oracle(case)
    U = case.initial_state()
    o.set_state(U, 0.0)
    ss, _ = o.error_norms()
    dt = o.time_step()
    assert ss == pytest.approx(1.0 / dt, rel=1e-12)


def test_norms_off_by_default_for_convergence():
    case = make(configs.sod(n=4))
    assert case.params.calc_ss_error == 1 and case.params.calc_conv_error == 0
    m = case.mesh_arrays()
    assert m["q_wJ"] is not None and m["q_xyz"] is None
