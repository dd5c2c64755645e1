"""The CPU oracle against the reference's own known-answer and property checks, against the
reference's exact Riemann solver (golden fixture), and against its committed regression vector."""
from pathlib import Path

import numpy as np
import pytest

from helpers import make, max_rel_err
from oracle import pyoracle
from oracle.pyoracle import Oracle
from plens_gb300 import configs

GOLDEN = Path(__file__).parent / "golden"


@pytest.fixture(scope="module")
def air_params():
    case = make(configs.sod(n=4))
    return case


def _rot(f, perm_sign):
    """Apply a velocity-component permutation/sign map to a 5-vector."""
    out = np.array(f, dtype=float)
    out[1:4] = [perm_sign[k][1] * f[1 + perm_sign[k][0]] for k in range(3)]
    return out


def test_surface_flux_rotational_invariance(air_params):
    """navier_stokes.cc:1726-1774: the HLLC interface flux with x, -x, y and z normals and
    correspondingly rotated states is the rotated x flux."""
    pp = air_params.params_ptr
    ocs, ncs = [1.5, 3, 1.5, 4.5, 23], [2, 2, 4, 4, 34]
    fx = pyoracle.flux(pp, 0, ocs, ncs, [1, 0, 0])
    np.testing.assert_allclose(fx, pyoracle.flux(pp, 2, ocs, ncs, [1, 0, 0]), rtol=1e-14)
    # -x normal, velocities reversed: flux along -x
    f = pyoracle.flux(pp, 0, [1.5, -3, -1.5, -4.5, 23], [2, -2, -4, -4, 34], [-1, 0, 0])
    np.testing.assert_allclose(f, [fx[0], -fx[1], -fx[2], -fx[3], fx[4]], rtol=1e-13)
    # y normal, velocities rotated 90 degrees ccw in xy
    f = pyoracle.flux(pp, 0, [1.5, -1.5, 3, 4.5, 23], [2, -4, 2, 4, 34], [0, 1, 0])
    np.testing.assert_allclose(f, [fx[0], -fx[2], fx[1], fx[3], fx[4]], rtol=1e-13, atol=1e-13)
    # z normal, x and z rotated
    f = pyoracle.flux(pp, 0, [1.5, -4.5, 1.5, 3, 23], [2, -4, 4, 2, 34], [0, 0, 1])
    np.testing.assert_allclose(f, [fx[0], -fx[3], fx[2], fx[1], fx[4]], rtol=1e-13, atol=1e-13)
    # an oblique normal: invariance under a rotation of both states and the normal
    th = 0.7
    R = np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1]])
    n = R @ np.array([1.0, 0, 0])
    o2 = np.r_[ocs[0], R @ np.array(ocs[1:4]), ocs[4]]
    n2 = np.r_[ncs[0], R @ np.array(ncs[1:4]), ncs[4]]
    f = pyoracle.flux(pp, 0, o2, n2, n)
    np.testing.assert_allclose(f, np.r_[fx[0], R @ fx[1:4], fx[4]], rtol=1e-12, atol=1e-12)


def test_consistency_of_two_point_fluxes(air_params):
    """Every surface flux equals the physical flux for identical states; the volume flux too."""
    pp = air_params.params_ptr
    s = [1.3, 0.4, -0.2, 0.1, 3.1]
    n = np.array([0.3, -0.5, 0.8])
    n /= np.linalg.norm(n)
    rho, m, E = s[0], np.array(s[1:4]), s[4]
    p = 0.4 * (E - 0.5 * m @ m / rho)
    vn = m @ n / rho
    phys = np.r_[rho * vn, vn * m + p * n, (E + p) * vn]
    for which in (0, 1):
        np.testing.assert_allclose(pyoracle.flux(pp, which, s, s, n), phys, rtol=1e-13, atol=1e-14)


def test_blender_linear_field_gives_zero_and_step_gives_alpha():
    """BlenderCalculator::test (blender_calculator.cc:386-407): one N=3 cell; a linear field has
    no high modes (alpha = 0), a step in x is troubled (alpha > 0)."""
    case = make(configs.dmr(nx=1, ny=1))
    o = Oracle(case)
    X = case.dof_xyz()[:, :64]
    x, y, z = [(X[d] - X[d].min()) / (X[d].max() - X[d].min() + 1e-300) for d in range(3)]
    assert o.cell_blender(x + 2 * y + 5 * z + 3) == 0.0
    step = np.where(x >= 0.5, 2.0, 1.0)
    assert o.cell_blender(step) > 0


def test_change_of_basis_is_orthonormal_projection():
    """C maps nodal values of Legendre mode j to the unit vector e_j
    (change_of_basis_matrix.h:74-98 with the orthonormal Legendre basis on [0,1])."""
    case = make(configs.dmr(nx=1, ny=1))
    o = Oracle(case)
    w, D, C = o.operators()
    X = case.dof_xyz()[:, :64]
    x = (X[0] - X[0].min()) / (X[0].max() - X[0].min())
    for k in range(4):
        leg = np.polynomial.legendre.Legendre.basis(k)(2 * x - 1) * np.sqrt(2 * k + 1)
        modes = C @ leg
        e = np.zeros(64)
        e[k] = 1
        np.testing.assert_allclose(modes, e, atol=1e-13)
    # D differentiates polynomials of degree N exactly; rows sum to zero
    np.testing.assert_allclose(D.sum(axis=1), 0, atol=1e-12)


def test_free_stream_preservation():
    """A uniform state on a fully periodic straight mesh has a zero residual."""
    case = make(configs.shock_vortex(n=2, modes=1))
    U = case.initial_state()
    rho, u, p = 1.2, np.array([0.3, -0.2, 0.5]), 0.9
    U[0], U[1:4], U[4] = rho, (rho * u)[:, None], p / 0.4 + 0.5 * rho * u @ u
    o = Oracle(case)
    o.set_state(U)
    R, a, _ = o.rhs()
    assert np.abs(R).max() < 1e-12 and (a == 0).all()


def test_conservation_on_periodic_domain():
    """sum over dofs of w_i w_j w_k detJ R = 0 for mass, momentum and energy on a periodic box
    (interior fluxes cancel pairwise). The viscous blending factor (1 - alpha_d) differs between
    neighbours and breaks momentum/energy conservation by design (dgsem/plens.cc:3759-3765), so
    the blending region is switched off here."""
    prm, files, deg = configs.shock_vortex(n=3, modes=2)
    prm = prm.replace("subsection blender parameters\n", "subsection blender parameters\n    set viscous blending region = -1\n")
    case = make((prm, files, deg))
    o = Oracle(case)
    o.set_state(case.initial_state())
    R, a, _ = o.rhs()
    w, _, _ = o.operators()
    W = np.einsum("i,j,k->kji", w, w, w).ravel()
    detJ = case.mesh_arrays()["detJ"]
    wt = np.tile(W, case.n_cells) * detJ
    tot = (R * wt).sum(axis=1)
    scale = (np.abs(R) * wt).sum(axis=1)
    assert (np.abs(tot) <= 1e-12 * scale).all(), tot / scale


def test_sod_against_reference_exact_solver():
    """Config-1 physics against the exact solution of the reference's own Riemann solver
    (utilities/shockTubeSoln.py, via tests/golden/sod_exact_t0.2.npz): L1 density error at t=0.2."""
    g = np.load(GOLDEN / "sod_exact_t0.2.npz")
    case = make(configs.sod(n=200, end_time=0.2, noise=0.0))
    o = Oracle(case)
    o.set_state(case.initial_state(), 0.0)
    o.advance(10000, 0.2)
    U, t, n, _ = o.get_state()
    assert t == pytest.approx(0.2, abs=1e-14)
    X = case.dof_xyz()
    exact = np.interp(X[0], g["x"], g["rho"])
    l1 = np.mean(np.abs(U[0] - exact))
    assert l1 < 5e-3, l1


def test_oracle_regression_vector():
    """The committed oracle vector (tests/golden/make_golden.py) is reproduced on this host."""
    g = np.load(GOLDEN / "oracle_sod_rhs.npz")
    case = make(configs.sod(n=40))
    o = Oracle(case)
    o.set_state(g["U"], float(g["t"]))
    R, a, _ = o.rhs()
    np.testing.assert_allclose(a, g["alpha"], atol=1e-13)
    assert max_rel_err(R, g["R"]) <= 1e-13


def test_time_step_formula():
    """calc_time_step (dgsem/plens.cc:3839-3864) on a uniform state: Co/(N^1.5 (u/h... ))."""
    case = make(configs.sod(n=10))
    U = case.initial_state()
    rho, u, p = 1.0, 0.7, 1.0
    U[0], U[1], U[2], U[3], U[4] = rho, rho * u, 0, 0, p / 0.4 + 0.5 * rho * u * u
    o = Oracle(case)
    o.set_state(U)
    h = 0.005  # min vertex distance of the 0.1 x 0.005 x 0.005 cells
    a = np.sqrt(1.4 * p / rho)
    dt = 0.5 / (2 ** 1.5 * (u / 0.1 + a / h))
    assert o.time_step() == pytest.approx(dt, rel=1e-13)


def test_positivity_failure_is_reported():
    case = make(configs.sod(n=4))
    U = case.initial_state()
    U[4, 7] = 0.0  # e <= 0
    o = Oracle(case)
    o.set_state(U)
    with pytest.raises(pyoracle.OracleError) as e:
        o.rhs()
    assert e.value.status == 3 and e.value.dof == 7


def test_modified_steger_warming_flux(air_params):
    """The modified Steger-Warming flux (navier_stokes.cc:1172-1234): identical states give the
    physical flux (the pressure weight is 1/2, A+ + A- = A and A u = F(u)), and the flux is
    invariant under rotations of the states and the normal (the rotation to the normal frame of
    navier_stokes.cc:482-569)."""
    prm = air_params.params
    old = prm.inv_surf_flux
    prm.inv_surf_flux = 5  # PLENS_ISF_MODIFIED_SW
    try:
        pp = air_params.params_ptr
        s = [1.3, 0.4, -0.2, 0.1, 3.1]
        n = np.array([0.3, -0.5, 0.8])
        n /= np.linalg.norm(n)
        rho, m, E = s[0], np.array(s[1:4]), s[4]
        p = 0.4 * (E - 0.5 * m @ m / rho)
        vn = m @ n / rho
        phys = np.r_[rho * vn, vn * m + p * n, (E + p) * vn]
        np.testing.assert_allclose(pyoracle.flux(pp, 0, s, s, n), phys, rtol=1e-12, atol=1e-13)
        ocs, ncs = [1.5, 3, 1.5, 4.5, 23], [2, 2, 4, 4, 34]
        fx = pyoracle.flux(pp, 0, ocs, ncs, [1, 0, 0])
        f = pyoracle.flux(pp, 0, [1.5, -3, -1.5, -4.5, 23], [2, -2, -4, -4, 34], [-1, 0, 0])
        np.testing.assert_allclose(f, [fx[0], -fx[1], -fx[2], -fx[3], fx[4]], rtol=1e-12, atol=1e-12)
        th = 0.7
        R = np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1]])
        o2 = np.r_[ocs[0], R @ np.array(ocs[1:4]), ocs[4]]
        n2 = np.r_[ncs[0], R @ np.array(ncs[1:4]), ncs[4]]
        f = pyoracle.flux(pp, 0, o2, n2, R @ np.array([1.0, 0, 0]))
        np.testing.assert_allclose(f, np.r_[fx[0], R @ fx[1:4], fx[4]], rtol=1e-12, atol=1e-12)
        # the flux differs from HLLC's on a jump (a different scheme is evaluated)
        prm.inv_surf_flux = 0
        assert np.abs(pyoracle.flux(pp, 0, ocs, ncs, [1, 0, 0]) - fx).max() > 1e-3
    finally:
        prm.inv_surf_flux = old
