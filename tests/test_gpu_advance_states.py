"""plens_gpu_advance_states: a sequence of independent states advanced with the host transfers
overlapping the steps gives, member for member, the bits of the serial loop set_state -> advance ->
get_state (PLENS::run advances one state per run, dgsem/plens.cc:1509-1550), with page-locked and
with pageable host buffers, and reports a failing member by its index."""
from pathlib import Path

import numpy as np
import pytest

from helpers import make
from plens_gb300 import configs
from plens_gb300.api import GpuSolver, PositivityError

pytestmark = pytest.mark.gpu

T0 = 0.0


def _weights():
    return np.fromfile(Path(__file__).resolve().parent.parent / "plens_gb300" / "sensor_weights.bin", dtype=np.float32)


def _members(case, n):
    """n different states: the initial condition with its density scaled by seeded factors."""
    rng = np.random.default_rng(11)
    U0 = case.initial_state()
    out = []
    for k in range(n):
        U = U0.copy()
        f = 1.0 + 1e-3 * k * rng.uniform(-1, 1, U.shape[1])
        U[0] *= f
        U[1:] *= f  # same velocities and specific energy
        out.append(U)
    return out


def _pinned(n_dofs, count):
    torch = pytest.importorskip("torch")
    keep = [torch.empty((5, n_dofs), dtype=torch.float64).pin_memory() for _ in range(count)]
    return keep, [t.numpy() for t in keep]


def _serial(case, members, n_steps, weights=None):
    g = GpuSolver(case)
    if weights is not None:
        g.set_sensor_weights(weights)
    outs, times = [], []
    for U in members:
        g.set_state(U, T0)
        g.advance(n_steps)
        outs.append(g.get_state())
        times.append(g.get_time()[0])
    g.close()
    return outs, times


@pytest.mark.parametrize("prec,sensor,pinned", [("fp64", "modal", True), ("fp64", "modal", False),
                                                ("mixed", "modal", True), ("mixed", "learned", True)])
def test_sequence_matches_the_serial_loop(prec, sensor, pinned):
    case = make(configs.dmr(nx=24, ny=6, precision=prec, sensor=sensor))
    weights = _weights() if sensor == "learned" else None
    members = _members(case, 4)
    n_steps = 3
    ref, ref_t = _serial(case, members, n_steps, weights)
    if pinned:
        keep_in, U_in = _pinned(case.n_dofs, len(members))
        keep_out, U_out = _pinned(case.n_dofs, len(members))
        for a, b in zip(U_in, members):
            a[:] = b
    else:
        U_in = [m.copy() for m in members]
        U_out = [np.empty_like(m) for m in members]
    g = GpuSolver(case)
    if weights is not None:
        g.set_sensor_weights(weights)
    t = g.advance_states(U_in, U_out, T0, n_steps)
    for k in range(len(members)):
        assert np.array_equal(U_out[k], ref[k]), f"member {k}"
        assert t[k] == ref_t[k]
    # the context holds the last member
    assert np.array_equal(g.get_state(), ref[-1])
    if sensor == "learned":
        return  # the judge schedule runs on across calls: a second call judges other steps
    # a second call on the same context (buffers made on the first call are reused)
    t2 = g.advance_states(U_in[:2], U_out[:2], T0, n_steps)
    assert np.array_equal(U_out[0], ref[0]) and np.array_equal(U_out[1], ref[1])
    assert list(t2) == ref_t[:2]


@pytest.mark.parametrize("sensor", ["modal", "learned"])
def test_failing_member_is_named_and_earlier_outputs_are_complete(sensor):
    """Member 1 has a negative density: the call reports member 1 and its dof (the first stage's
    positivity assertion; no later stage moves the state on). Member 0 is complete; without the
    learned sensor every member is advanced, so member 2 is complete too, while the learned
    sensor's sequence stops at the failure."""
    case = make(configs.dmr(nx=24, ny=6, precision="mixed", sensor=sensor))
    weights = _weights() if sensor == "learned" else None
    members = _members(case, 3)
    bad = members[1].copy()
    bad[0, 77] = -1.0
    members[1] = bad
    ref, _ = _serial(case, [members[0], members[2]], 2, weights)
    U_out = [np.full_like(m, np.nan) for m in members]
    g = GpuSolver(case)
    if weights is not None:
        g.set_sensor_weights(weights)
    with pytest.raises(PositivityError) as ei:
        g.advance_states(members, U_out, T0, 2)
    assert "member 1" in str(ei.value)
    assert ei.value.dof == 77
    assert np.array_equal(U_out[0], ref[0])
    if sensor == "learned":
        assert np.isnan(U_out[2]).all()
    else:
        assert np.array_equal(U_out[2], ref[1])
