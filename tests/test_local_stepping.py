"""Local time stepping (calc_time_step, dgsem/plens.cc:3876-3911; multiply_time_step_to_rhs,
3925-3940) in the oracle: the per-cell factor of the RHS is the global step until t passes the
start time, then each cell's own stable step, limited by its interior-face neighbours and by the
global step when asked. The GPU forms are checked against these in test_gpu_local_stepping.py."""
import numpy as np

from helpers import make
from oracle.pyoracle import Oracle
from plens_gb300 import configs


def _case(limit, start=0.0, nbr=1.05, glob=1000.0):
    return make(configs.cylinder(n_radial=8, n_azimuthal=16,
                                 local=dict(start=start, limit=limit, neighbor=nbr, global_=glob)))


def _stepped(case, steps=1):
    o = Oracle(case)
    o.set_state(case.initial_state(), 0.0)
    o.advance(steps)
    return o


def test_global_until_start_time():
    case = _case(limit=False, start=0.0)
    o = Oracle(case)
    o.set_state(case.initial_state(), 0.0)
    o.advance(1)  # t = 0 is not past the start time: global stepping
    dt0 = o.loc_time_steps()
    assert np.all(dt0 == dt0[0])
    o.advance(1)  # now t > 0
    dt1 = o.loc_time_steps()
    assert dt1.max() > 1.5 * dt1.min()


def test_unlimited_steps_are_the_cell_bounds():
    o = _stepped(_case(limit=False), 2)
    g = o.time_step()
    # the global step is their minimum
    assert o.loc_time_steps().min() == g


def test_limited_steps():
    nbr_f, glob_f = 1.05, 3.0
    case_u, case_l = _case(limit=False), _case(limit=True, nbr=nbr_f, glob=glob_f)
    ou = _stepped(case_u, 1)
    ol = _stepped(case_l, 1)
    U, t, _, _ = ou.get_state()
    ol.set_state(U, t)
    ou.time_step()
    ol.time_step()
    free, lim = ou.loc_time_steps(), ol.loc_time_steps()
    nbr = case_l.mesh_arrays()["cell_nbr"]
    g = free.min()
    expect = free.copy()
    for c in range(case_l.n_cells):
        for nb in nbr[c]:
            if nb >= 0:
                expect[c] = min(expect[c], nbr_f * free[nb])
        expect[c] = min(expect[c], glob_f * g)
    np.testing.assert_array_equal(lim, expect)
    assert (lim < free).any()
    # the z faces of the cylinder mesh are periodic: boundary faces, never limiting
    assert (nbr < 0).sum() >= 2 * case_l.n_cells


def test_local_run_differs_and_stays_positive():
    case_g = make(configs.cylinder(n_radial=8, n_azimuthal=16))
    og = _stepped(case_g, 3)
    ol = _stepped(_case(limit=True), 3)
    Ug, Ul = og.get_state()[0], ol.get_state()[0]
    assert np.all(Ul[0] > 0)
    assert np.abs(Ug - Ul).max() > 0
