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


def _long_list(spec):
    """The DMR with the blender threshold factor at 1e-6 and pre-shock noise at 1e-3: about 90%
    of the cells troubled, so every block of the subcell kernel's grid takes several groups."""
    prm, files, deg = spec
    key = "    set wall blender limit = 0\n"
    assert key in prm
    return prm.replace(key, key + "    set threshold factor = 1e-6\n"), files, deg


@pytest.mark.parametrize("prec,sensor,long", [("mixed", "modal", False), ("mixed", "modal", True),
                                              ("mixed", "learned", True), ("mixed_r32", "modal", True)])
def test_list_decoding_and_list_kernel_agree(prec, sensor, long):
    """The two forms of the list: the subcell kernel decoding each position's cell from the
    smoothing kernel's block counts and ballots (the default), and the list kernel writing the
    list first (the form of meshes above 1,048,448 cells). The same list and the same RHS, bit
    for bit, and the same state after five steps."""
    spec = configs.dmr(nx=120, ny=30, noise=1e-3, precision=prec, sensor=sensor)
    case = make(_long_list(spec) if long else spec)
    out = []
    for decode in (True, False):
        g = GpuSolver(case)
        if sensor == "learned":
            g.set_sensor_weights(_weights())
        g.set_list_decoding(decode)
        g.set_state(case.initial_state(), case.start_time)
        g.advance(2)
        R = g.rhs()
        lst = g.troubled_cells()
        g.advance(5)
        out.append((R, lst, g.get_state()))
        g.close()
    (Ra, la, Ua), (Rb, lb, Ub) = out
    print(f"{len(la)} listed cells")
    assert len(la) > 0
    if long:
        assert len(la) > 2 * 4 * 152 * 2
    assert np.array_equal(la, lb)
    assert np.array_equal(Ra, Rb)
    assert np.array_equal(Ua, Ub)
