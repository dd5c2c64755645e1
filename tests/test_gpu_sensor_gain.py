"""What the trained network gains over the same learned-sensor path without training.

The shipped weights (plens_gb300/sensor_weights.bin, trained by our CUDA kernels on pairs from
plain runs) and a random-initialised network run the same double Mach reflection window in the
mixed form with the judge every 5th step. The judge hands every cell whose alpha is off by more
than 0.05 back to the plain indicator, so both runs stay accurate; what training buys is that the
network's alpha is the one used: the trained network is handed back a small fraction of the
cells the untrained one is, and the run stays within the accuracy bound against the FP64 form
without leaning on the fallback.
"""
from pathlib import Path

import numpy as np
import pytest

from helpers import make, rel_l1
from oracle import mlp_oracle
from plens_gb300 import configs
from plens_gb300.api import MLP_N_PARAMS, GpuSolver

pytestmark = pytest.mark.gpu

WEIGHTS = Path(__file__).resolve().parents[1] / "plens_gb300" / "sensor_weights.bin"
STEPS = 60


def _run(weights, precision="mixed", sensor="learned"):
    prm, files, deg = configs.dmr(nx=120, ny=30, precision=precision, sensor=sensor)
    prm = prm.replace("set judge every = 25", "set judge every = 5")
    case = make((prm, files, deg))
    g = GpuSolver(case)
    if weights is not None:
        g.set_sensor_weights(weights)
    g.set_state(case.initial_state(), 0.0)
    g.advance(STEPS)
    st = g.sensor_stats() if sensor == "learned" else None
    return g.get_state(), st, case.n_cells


def test_trained_network_gains_over_untrained():
    w = np.fromfile(WEIGHTS, dtype=np.float32)
    assert w.size == MLP_N_PARAMS
    U64, _, nc = _run(None, precision="fp64", sensor="modal")
    Ut, st_t, _ = _run(w)
    Uu, st_u, _ = _run(mlp_oracle.init_params(0))
    judged_cells = st_t["judged"] * nc
    rate_t = st_t["fallbacks"] / judged_cells
    rate_u = st_u["fallbacks"] / max(st_u["judged"] * nc, 1)
    err_t = rel_l1(Ut, U64)
    err_u = rel_l1(Uu, U64)
    print(f"trained: handed back {rate_t:.4%} of judged cells, max alpha err {st_t['max_alpha_err']:.3g}, "
          f"rel L1 {err_t}; untrained: {rate_u:.4%}, max alpha err {st_u['max_alpha_err']:.3g}, rel L1 {err_u}")
    assert st_t["judged"] >= 10
    assert rate_t < 0.02
    assert rate_t < 0.1 * rate_u
    assert err_t[0] <= 1e-4
