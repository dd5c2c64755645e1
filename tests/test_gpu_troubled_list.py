"""The compacted troubled-cell list of the mixed forms, and the subcell residual that runs over it.

The list holds exactly the cells with alpha > 0 (the cells calc_cell_lo_inv_residual runs on,
dgsem/plens.cc:3469-3583), in increasing index order, and is the same on every run (it is built
from per-block counts and warp ballots, without atomics). The residual of the troubled cells,
which the volume kernel takes from the list kernel's output, matches the oracle within the mixed
form's RHS tolerance.
"""
import numpy as np
import pytest

from helpers import make, max_rel_err
from oracle.pyoracle import Oracle
from plens_gb300 import configs
from plens_gb300.api import GpuSolver, PlensError

pytestmark = pytest.mark.gpu


def _weights():
    from pathlib import Path
    return np.fromfile(Path(__file__).resolve().parent.parent / "plens_gb300" / "sensor_weights.bin", dtype=np.float32)


@pytest.mark.parametrize("prec,sensor", [("mixed", "modal"), ("mixed_r32", "modal"), ("mixed", "learned")])
def test_list_is_the_ordered_set_of_troubled_cells(prec, sensor):
    case64 = make(configs.dmr(nx=48, ny=12))
    o = Oracle(case64)
    o.set_state(case64.initial_state(), 0.0)
    o.advance(10)
    U, t, _, _ = o.get_state()
    case = make(configs.dmr(nx=48, ny=12, precision=prec, sensor=sensor))
    g = GpuSolver(case)
    if sensor == "learned":
        g.set_sensor_weights(_weights())
    g.set_state(U, t)
    R1 = g.rhs()
    alpha, _, _ = g.cell_scalars()
    lst = g.troubled_cells()
    expect = np.flatnonzero(alpha > 0).astype(np.int32)
    assert len(expect) > 0
    np.testing.assert_array_equal(lst, expect)
    assert g.sensor_stats()["lo_cells_last"] == len(expect)
    # the same list and the same residual bits on a second evaluation
    R2 = g.rhs()
    np.testing.assert_array_equal(g.troubled_cells(), lst)
    assert np.array_equal(R1, R2)
    if sensor == "modal":
        # the subcell residual of the troubled cells, through the list, against the oracle
        o.set_state(U, t)
        Ro = o.rhs()[0]
        assert max_rel_err(R1, Ro) <= 2e-4
        P3 = (case.degree + 1) ** 3
        dofs = (lst[:, None] * P3 + np.arange(P3)[None, :]).ravel()
        assert max_rel_err(R1[:, dofs], Ro[:, dofs]) <= 2e-4


def test_fp64_context_has_no_list():
    case = make(configs.dmr(nx=12, ny=4))
    g = GpuSolver(case)
    g.set_state(case.initial_state(), 0.0)
    g.rhs()
    with pytest.raises(PlensError):
        g.troubled_cells()
