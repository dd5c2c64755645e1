"""The learned troubled-cell sensor against the method without it (the FP32 modal indicator of the
mixed form), on the same double Mach reflection window, both against the FP64 plain form.

For each sensor the test reports and bounds: the relative L1 distance of rho, momentum and rho E
from the FP64 form after the window; the per-cell agreement of the learned form's alpha with the
modal form's on the same state (mean absolute difference, and the share of cells where one is
troubled and the other is not); the judge's outcome (judged steps, cells handed back to the
plain indicator and their rate, the largest alpha error it saw). The workload is the double Mach
reflection configuration itself (240 x 60 x 1 cells, N = 3) over its first 100 steps; the
learned sensor has to stay within the configuration's rho bound (1e-4); the modal form, which
evaluates the indicator it imitates, is the accuracy reference.
"""
from pathlib import Path

import numpy as np
import pytest

from helpers import make, rel_l1
from plens_gb300 import configs
from plens_gb300.api import GpuSolver

pytestmark = pytest.mark.gpu

STEPS = 100


def _weights():
    return np.fromfile(Path(__file__).resolve().parent.parent / "plens_gb300" / "sensor_weights.bin", dtype=np.float32)


def _run(prec, sensor, nx=240, ny=60):
    case = make(configs.dmr(nx=nx, ny=ny, precision=prec, sensor=sensor))
    g = GpuSolver(case)
    if sensor == "learned":
        g.set_sensor_weights(_weights())
    g.set_state(case.initial_state(), 0.0)
    g.advance(STEPS)
    return case, g


def test_learned_sensor_against_the_modal_indicator():
    _, g64 = _run("fp64", "modal")
    U64 = g64.get_state()
    case, gm = _run("mixed", "modal")
    _, gl = _run("mixed", "learned")
    Um, Ul = gm.get_state(), gl.get_state()
    err_m, err_l = rel_l1(Um, U64), rel_l1(Ul, U64)
    # alpha of both sensors on the same state (the modal form's state at the end of the window)
    gl.set_state(Um, gm.get_time()[0])
    gl.rhs()
    a_l = gl.cell_scalars()[0]
    gm.rhs()
    a_m = gm.cell_scalars()[0]
    mad = float(np.abs(a_l - a_m).mean())
    disagree = float(((a_l > 0) != (a_m > 0)).mean())
    st = gl.sensor_stats()
    rate = st["fallbacks"] / max(st["judged"] * case.n_cells, 1)
    print(f"\nDMR 240x60, {STEPS} steps; rel L1 (rho, momentum, rho E) vs FP64: modal {err_m}, learned {err_l}; "
          f"alpha vs modal: mean |diff| {mad:.2e}, troubled-set disagreement {disagree:.3%}; judge: {st['judged']} "
          f"judged steps, {st['fallbacks']} cells handed back ({rate:.3%}), max alpha error {st['max_alpha_err']:.3f}")
    assert err_m[0] <= 1e-6  # the modal form: FP32 round-off only
    assert err_l[0] <= 1e-4  # the configuration's bound for the learned form
    assert mad <= 0.02
    assert disagree <= 0.05
    assert st["judged"] >= 2
    assert rate <= 0.05
