"""Data output on the GPU path: the asynchronous snapshot hands out the state of the step at which
it was started while later steps run, and the command-line driver (the reference's main + PLENS::run)
writes .vtu/.pvd/.times/.ar every `write frequency` steps; restarting from an archive with the
"from archive restart" initial condition continues the run bit for bit."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from helpers import make
from plens_gb300 import configs
from plens_gb300.api import GpuSolver

pytestmark = pytest.mark.gpu

DRIVER = Path(__file__).resolve().parents[1] / "plens_gb300" / "lib" / "plens_gpu.out"


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_async_snapshot_is_the_state_at_begin(precision):
    case = make(configs.dmr(nx=24, ny=6, precision=precision))
    a = GpuSolver(case)
    a.set_state(case.initial_state(), 0.0)
    a.advance(5)
    a.snapshot_begin()
    a.advance_async(4)  # runs while the snapshot is copied out
    snap = a.snapshot_end()
    a.synchronize()
    b = GpuSolver(case)
    b.set_state(case.initial_state(), 0.0)
    b.advance(5)
    np.testing.assert_array_equal(snap["U"], b.get_state())
    t, n, _ = b.get_time()
    assert snap["time"] == t and snap["n_steps"] == n == 5
    alpha, alpha_d, _ = b.cell_scalars()
    np.testing.assert_array_equal(snap["alpha"], alpha)
    assert a.get_time()[1] == 9


def _write_case(d: Path, spec, end_time, extra=""):
    prm, files, deg = spec
    for name, text in files.items():
        (d / name).write_text(text)
    prm = prm.replace("set end time = 1.0", f"set end time = {end_time!r}")
    prm = prm.replace("subsection data output\n    set write frequency = 1000000", "subsection data output\n    set write frequency = 10")
    (d / "input.prm").write_text(prm + extra)
    return deg


def test_driver_output_and_restart(tmp_path):
    spec = configs.sod(n=20)
    prm = spec[0]
    assert "set end time = 1.0" in prm
    full = tmp_path / "full"
    full.mkdir()
    deg = _write_case(full, spec, 0.02)
    subprocess.run([str(DRIVER), "2", str(deg)], cwd=full, check=True, capture_output=True, timeout=300)
    res = full / "result"
    vtus = sorted(res.glob("output_*.vtu"))
    ars = sorted(res.glob("output_*.ar"))
    times = (res / "output.times").read_text().split("\n")
    assert len(vtus) >= 3 and len(vtus) == len(ars) == len([t for t in times if t.strip()])
    assert (res / "output.pvd").exists()
    U_full = np.fromfile(res / "output.state", dtype=np.float64)
    # restart from the second archive and run to the same end time
    case = make(spec)
    U_ar, t_ar, n_ar, k_ar = case.read_archive(ars[1])
    assert n_ar == 10 and k_ar == 1
    rs = tmp_path / "restart"
    rs.mkdir()
    prm_r = (prm.replace("set type = piecewise function", "set type = from archive restart", 1)
             .replace("set file name = ic.dat", f"set file name = {ars[1]}", 1)
             .replace("set variable = rho", "set variable = none", 1))
    prm_r = prm_r.replace("subsection time integration", f"subsection time integration\n    set start time = {t_ar!r}", 1)
    _write_case(rs, (prm_r, spec[1], deg), 0.02)
    subprocess.run([str(DRIVER), "2", str(deg)], cwd=rs, check=True, capture_output=True, timeout=300)
    U_rs = np.fromfile(rs / "result" / "output.state", dtype=np.float64)
    np.testing.assert_array_equal(U_rs, U_full)
