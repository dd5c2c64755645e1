"""The mixed forms against the FP64 oracle, over the kernels they dispatch to: the TMA-staged
volume kernel (even P: N = 1, 3, 5; inviscid and viscous), the generic one (odd P), every surface
and volume flux scheme, RK3 and the positivity check. "mixed": FP32 flux differencing with the
state, the metric terms, the 1/det J scaling, the RK registers and their accumulation in FP64;
"mixed_r32": the same flux arithmetic with FP32 registers and FP32 metric images.

Tolerances: one RHS, max over equations of max|R_mixed - R_oracle| / max|R_oracle| <= 2e-4 (2e-3
on the 1e-3-clustered curved O-mesh, where the wall-cell residual is a small difference of large
fluxes); after 20 steps, relative L1 of rho, momentum and rho E <= 1e-4.
"""
import numpy as np
import pytest

from helpers import make, max_rel_err, rel_l1
from oracle.pyoracle import Oracle
from plens_gb300 import configs
from plens_gb300.api import GpuSolver, PositivityError

pytestmark = pytest.mark.gpu

RHS_TOL = 2e-4
STEPS_TOL = 1e-4
PRECS = ["mixed", "mixed_r32"]


def _state(case64, steps):
    o = Oracle(case64)
    o.set_state(case64.initial_state(), case64.start_time)
    o.advance(steps)
    U, t, _, _ = o.get_state()
    return U, t


def _rhs_err(spec64, specmx, steps=2):
    c64, cmx = make(spec64), make(specmx)
    U, t = _state(c64, steps)
    o = Oracle(c64)
    o.set_state(U, t)
    Ro = o.rhs()[0]
    g = GpuSolver(cmx)
    g.set_state(U, t)
    Rg = g.rhs()
    return max_rel_err(Rg, Ro)


def _steps_err(spec64, specmx, steps=20):
    c64, cmx = make(spec64), make(specmx)
    o = Oracle(c64)
    o.set_state(c64.initial_state(), c64.start_time)
    o.advance(steps)
    g = GpuSolver(cmx)
    g.set_state(cmx.initial_state(), cmx.start_time)
    g.advance(steps)
    return rel_l1(g.get_state(), o.get_state()[0])


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5])
def test_mixed_dmr_degrees(degree, prec):
    e = _rhs_err(configs.dmr(nx=12, ny=4, degree=degree), configs.dmr(nx=12, ny=4, degree=degree, precision=prec))
    print(f"N={degree} rhs err {e:.3e}")
    assert e <= RHS_TOL
    s = _steps_err(configs.dmr(nx=12, ny=4, degree=degree), configs.dmr(nx=12, ny=4, degree=degree, precision=prec))
    print(f"N={degree} 20-step rel L1 {s}")
    assert s.max() <= STEPS_TOL


@pytest.mark.parametrize("prec", PRECS)
def test_mixed_sod(prec):
    e = _rhs_err(configs.sod(n=40), configs.sod(n=40, precision=prec), steps=10)
    assert e <= RHS_TOL
    assert _steps_err(configs.sod(n=40), configs.sod(n=40, precision=prec), 100).max() <= STEPS_TOL


@pytest.mark.parametrize("scheme", ["Rusanov", "AUSM+-up", "Rusanov-HLLC", "Chandrashekhar", "Modified SW"])
def test_mixed_surface_schemes(scheme):
    def spec(prec):
        prm, files, deg = configs.dmr(nx=12, ny=4, precision=prec)
        return prm.replace("set inviscid surface flux scheme = HLLC", f"set inviscid surface flux scheme = {scheme}"), files, deg
    e = _rhs_err(spec("fp64"), spec("mixed"))
    print(f"{scheme} rhs err {e:.3e}")
    assert e <= RHS_TOL


@pytest.mark.parametrize("scheme", ["KG", "IR"])
def test_mixed_volume_schemes(scheme):
    def spec(prec):
        prm, files, deg = configs.dmr(nx=8, ny=4, precision=prec)
        return prm.replace("set inviscid volume flux scheme = Chandrashekhar", f"set inviscid volume flux scheme = {scheme}"), files, deg
    e = _rhs_err(spec("fp64"), spec("mixed"))
    print(f"{scheme} rhs err {e:.3e}")
    assert e <= RHS_TOL


@pytest.mark.parametrize("prec", PRECS)
def test_mixed_viscous_cylinder(prec):
    c64 = make(configs.cylinder(n_radial=6, n_azimuthal=12))
    cmx = make(configs.cylinder(n_radial=6, n_azimuthal=12, precision=prec))
    U, t = _state(c64, 2)
    o = Oracle(c64)
    o.set_state(U, t)
    Ro = o.rhs()[0]
    g = GpuSolver(cmx)
    g.set_state(U, t)
    Rg = g.rhs()
    e = max_rel_err(Rg, Ro)
    d = np.abs(Rg - Ro)
    worst = np.unravel_index(np.argmax(d / np.abs(Ro).max(axis=1, keepdims=True)), d.shape)
    print(f"cylinder rhs err {e:.3e} (worst var {worst[0]} cell {worst[1] // 64}); per-var rel L1 "
          f"{d.sum(axis=1) / np.abs(Ro).sum(axis=1)}")
    assert e <= 2e-3
    s = _steps_err(configs.cylinder(n_radial=6, n_azimuthal=12), configs.cylinder(n_radial=6, n_azimuthal=12, precision=prec))
    print(f"cylinder 20-step rel L1 {s}")
    assert s.max() <= STEPS_TOL


@pytest.mark.parametrize("prec", PRECS)
def test_mixed_viscous_shock_vortex(prec):
    e = _rhs_err(configs.shock_vortex(n=3, modes=2), configs.shock_vortex(n=3, modes=2, precision=prec), steps=1)
    print(f"shock-vortex rhs err {e:.3e}")
    assert e <= RHS_TOL
    s = _steps_err(configs.shock_vortex(n=3, modes=2), configs.shock_vortex(n=3, modes=2, precision=prec), 5)
    assert s.max() <= STEPS_TOL


def _all_troubled(spec):
    """The same workload with the blender's threshold factor at 1e-6 (threshold 2.9e-9 at N = 3):
    with the DMR's pre-shock density noise at 1e-3 the cells' high-mode energies (~1e-6) clear
    it by orders of magnitude in both precisions, and 90% of the cells are troubled after two
    steps. (Noise near the FP32 rounding level would leave the FP32 and FP64 indicators deciding
    different cells.)"""
    prm, files, deg = spec
    key = "    set wall blender limit = 0\n"
    assert key in prm
    return prm.replace(key, key + "    set threshold factor = 1e-6\n"), files, deg


@pytest.mark.parametrize("prec", PRECS)
def test_mixed_long_troubled_list(prec):
    """A troubled-cell list long enough that every block of the subcell kernel's persistent grid
    (at most four blocks per SM, two cells per group) takes several groups, so its pipelined loads
    of the next group and of the list entries after it all run: one RHS against the oracle, the
    list against the oracle's alpha > 0, and 20 steps."""
    spec64 = _all_troubled(configs.dmr(nx=120, ny=30, noise=1e-3))
    specmx = _all_troubled(configs.dmr(nx=120, ny=30, noise=1e-3, precision=prec))
    c64, cmx = make(spec64), make(specmx)
    U, t = _state(c64, 2)
    o = Oracle(c64)
    o.set_state(U, t)
    Ro, alpha_o, _ = o.rhs()
    g = GpuSolver(cmx)
    g.set_state(U, t)
    Rg = g.rhs()
    cells = g.troubled_cells()
    g.close()
    ref = np.flatnonzero(alpha_o > 0)
    print(f"{len(cells)} listed cells, oracle {len(ref)}")
    assert len(cells) > 2 * (4 * 152) * 2  # two groups of two cells for each of 4 x 152 blocks
    assert np.all(np.diff(cells) > 0)
    assert len(np.setxor1d(cells, ref)) <= 0.01 * len(ref)
    e = max_rel_err(Rg, Ro)
    print(f"rhs err {e:.3e}")
    assert e <= RHS_TOL
    s = _steps_err(spec64, specmx)
    print(f"20-step rel L1 {s}")
    assert s.max() <= STEPS_TOL


@pytest.mark.parametrize("prec", PRECS)
def test_mixed_rk3(prec):
    def spec(p):
        prm, files, deg = configs.dmr(nx=12, ny=4, precision=p)
        return prm.replace("set RK order = 4", "set RK order = 3"), files, deg
    assert _steps_err(spec("fp64"), spec(prec)).max() <= STEPS_TOL


def test_mixed_positivity_failure_reports_first_bad_dof():
    """The mixed form's screened check decides rho > 0, e > 0 in FP64: a state with e < 0 by a
    tiny margin at one dof (invisible to an FP32 test) and rho < 0 at a later one."""
    case = make(configs.dmr(nx=12, ny=4, precision="mixed"))
    U = case.initial_state()
    k = 301
    ke = 0.5 * (U[1, k] ** 2 + U[2, k] ** 2 + U[3, k] ** 2) / U[0, k]
    U[4, k] = ke * (1 - 1e-12)
    U[0, 777] = -1.0
    g = GpuSolver(case)
    g.set_state(U)
    with pytest.raises(PositivityError) as ei:
        g.rhs()
    assert ei.value.dof == k
    g.set_state(case.initial_state(), 0.0)
    g.rhs()
