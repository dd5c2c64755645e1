"""Error norms of the output steps on the GPU (plens_gpu_error_norms: calc_ss_error and
calc_convergence_error as PLENS::write logs them, dgsem/plens.cc:3985-4098, 4234-4319) against
the oracle, and the driver's .ss_error / .conv_error logs.

Tolerances: plain FP64 form, relative 1e-12 (the same quadrature sums in another order); the
driver's logs are printed with six significant digits."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from helpers import make
from oracle.pyoracle import Oracle
from plens_gb300 import configs
from plens_gb300.api import GpuSolver

pytestmark = pytest.mark.gpu

DRIVER = Path(__file__).resolve().parents[1] / "plens_gb300" / "lib" / "plens_gpu.out"
EXACT = "1 + 0.001*x*y + 0.5*t"


@pytest.mark.parametrize("local", [None, dict(start=0.0, limit=True, neighbor=1.05, global_=50.0)])
def test_error_norms_match_oracle(local):
    spec = configs.with_error_norms(configs.cylinder(n_radial=6, n_azimuthal=16, local=local), conv_exact=EXACT)
    case = make(spec)
    o = Oracle(case)
    o.set_state(case.initial_state(), 0.0)
    g = GpuSolver(case)
    g.set_state(case.initial_state(), 0.0)
    for steps in (0, 1, 3):
        o.advance(steps)
        g.advance(steps)
        ss_o, cv_o = o.error_norms()
        ss_g, cv_g = g.error_norms()
        assert ss_g == pytest.approx(ss_o, rel=1e-12)
        assert cv_g == pytest.approx(cv_o, rel=1e-12)
    # the norms leave the run unchanged: the next steps match the oracle's
    o.advance(2)
    g.advance(2)
    np.testing.assert_allclose(g.get_state(), o.get_state()[0], rtol=0, atol=1e-9 * np.abs(o.get_state()[0]).max())


def test_mixed_form_error_norms():
    spec64 = configs.with_error_norms(configs.dmr(nx=24, ny=6), conv_exact="8")
    specmx = configs.with_error_norms(configs.dmr(nx=24, ny=6, precision="mixed"), conv_exact="8")
    c64, cmx = make(spec64), make(specmx)
    o = Oracle(c64)
    o.set_state(c64.initial_state(), 0.0)
    o.advance(10)
    g = GpuSolver(cmx)
    g.set_state(cmx.initial_state(), 0.0)
    g.advance(10)
    ss_o, cv_o = o.error_norms()
    ss_g, cv_g = g.error_norms()
    assert ss_g == pytest.approx(ss_o, rel=1e-2)
    assert cv_g == pytest.approx(cv_o, rel=1e-4)


def test_driver_error_logs(tmp_path):
    prm, files, deg = configs.with_error_norms(configs.sod(n=20), conv_exact=EXACT)
    for name, text in files.items():
        (tmp_path / name).write_text(text)
    prm = prm.replace("set end time = 1.0", "set end time = 0.02")
    prm = prm.replace("    set write frequency = 1000000", "    set write frequency = 10")
    (tmp_path / "input.prm").write_text(prm)
    subprocess.run([str(DRIVER), "2", str(deg)], cwd=tmp_path, check=True, capture_output=True, timeout=300)
    res = tmp_path / "result"
    rows = lambda f: [r.split() for r in (res / f).read_text().splitlines() if r.strip()]  # noqa: E731
    times, ss, cv = rows("output.times"), rows("output.ss_error"), rows("output.conv_error")
    assert len(times) >= 3 and len(ss) == len(cv) == len(times)
    assert [r[0] for r in ss] == [r[0] for r in times]
    # the same outputs through the library: the norms at steps 0, 10, 20, ...
    case = make(configs.with_error_norms(configs.sod(n=20), conv_exact=EXACT))
    g = GpuSolver(case)
    g.set_state(case.initial_state(), 0.0)
    for k in range(len(times)):
        if k:
            g.advance(10, 0.02)
        s, c = g.error_norms()
        assert float(ss[k][2]) == pytest.approx(s, rel=1e-5)
        assert float(cv[k][2]) == pytest.approx(c, rel=1e-5)
        assert float(ss[k][1]) == pytest.approx(g.get_time()[0], rel=1e-5, abs=1e-12)
