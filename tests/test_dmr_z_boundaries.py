"""The z boundaries of the double Mach reflection (oracle, CPU).

On a one-cell-thick periodic mesh each cell's -z face is paired with its own +z face. For a
z-invariant state the periodic ghost is then the state itself, as the symmetry ghost is when the
z-momentum vanishes (IBCs/periodic.cc:69-114, IBCs/symmetry.cc:53-59): the two right-hand sides
must agree to round-off, and a wrong face-dof pairing across the self-paired faces would show as
an O(1) difference. The positivity failure of the periodic configuration near t = 0.1 is
therefore not the pairing; it is the growth of z-dependent modes of the flow from round-off (see
the GPU test of the horizon).
"""
import numpy as np

from helpers import make
from oracle.pyoracle import Oracle
from plens_gb300 import configs


def _rhs(z_bc, nz=1):
    case = make(configs.dmr(nx=24, ny=6, z_bc=z_bc, noise=0.0, nz=nz))
    o = Oracle(case, threads=2)
    U = case.initial_state()
    o.set_state(U, 0.0)
    R, alpha, _ = o.rhs()
    return case, U, R, alpha


def test_dmr_initial_state_is_z_invariant():
    case, U, _, _ = _rhs("periodic")
    P = case.degree + 1
    Ur = U.reshape(5, case.n_cells, P, P * P)  # [var][cell][z layer][x-y node]
    assert np.array_equal(Ur, np.broadcast_to(Ur[:, :, :1, :], Ur.shape))
    assert not U[3].any()


def test_periodic_and_symmetry_z_agree_on_a_z_invariant_state():
    _, _, Rp, ap = _rhs("periodic")
    _, _, Rs, as_ = _rhs("symmetry")
    scale = np.abs(Rs).max()
    assert np.abs(Rp - Rs).max() <= 1e-15 * scale
    assert np.array_equal(Rp[3], Rs[3])
    assert np.abs(Rp[3]).max() <= 1e-14 * scale  # no z-momentum source beyond round-off
    assert np.abs(ap - as_).max() <= 1e-13


def test_two_cell_periodic_z_agrees_with_one_cell():
    """Two cells across z: the -z face of the lower cell pairs with the +z face of the upper one.
    Each x-y column of the two-cell mesh reproduces the one-cell right-hand side."""
    case1, _, R1, _ = _rhs("periodic", nz=1)
    case2, _, R2, _ = _rhs("periodic", nz=2)
    P = case1.degree + 1
    n1 = case1.n_cells
    r1 = R1.reshape(5, n1, P ** 3)
    # the box generator numbers cells x fastest, then y, then z
    r2 = R2.reshape(5, 2, n1, P ** 3)
    scale = np.abs(R1).max()
    for k in range(2):
        assert np.abs(r2[:, k] - r1).max() <= 1e-15 * scale


def _z_dependent(U, P, seed):
    """U with seeded per-dof perturbations of density and z-momentum (varying along z and across
    each face), the specific internal energy kept positive."""
    rng = np.random.default_rng(seed)
    V = U.copy()
    rho = V[0] * (1 + 1e-2 * rng.uniform(-1, 1, V.shape[1]))
    u = V[1:4] / V[0]
    e = (V[4] - 0.5 * (V[1:4] ** 2).sum(axis=0) / V[0]) / V[0]
    u[2] = 0.1 * rng.uniform(-1, 1, V.shape[1])
    V[0] = rho
    V[1:4] = rho * u
    V[4] = rho * e + 0.5 * rho * (u ** 2).sum(axis=0)
    return V


def test_self_paired_faces_on_a_z_dependent_state():
    """A z-dependent state (random density and z-velocity per dof) on the one-cell periodic mesh,
    and the same state in both cells of the two-cell periodic mesh, which then is the one-cell
    state's periodic continuation: every cell's right-hand side agrees. A wrong pairing of the
    self-paired -z/+z face dofs (a transposed or shifted face numbering) gives O(1) differences."""
    case1 = make(configs.dmr(nx=24, ny=6, z_bc="periodic", noise=0.0, nz=1))
    case2 = make(configs.dmr(nx=24, ny=6, z_bc="periodic", noise=0.0, nz=2))
    P = case1.degree + 1
    n1 = case1.n_cells
    U1 = _z_dependent(case1.initial_state(), P, 5)
    U2 = np.concatenate([U1.reshape(5, n1, P ** 3)] * 2, axis=1).reshape(5, -1)
    o1, o2 = Oracle(case1, threads=2), Oracle(case2, threads=2)
    o1.set_state(U1, 0.0)
    o2.set_state(U2, 0.0)
    R1, a1, _ = o1.rhs()
    R2, a2, _ = o2.rhs()
    r1 = R1.reshape(5, n1, P ** 3)
    r2 = R2.reshape(5, 2, n1, P ** 3)
    scale = np.abs(R1).max(axis=1, keepdims=True)
    for k in range(2):
        assert (np.abs(r2[:, k] - r1).max(axis=2) / scale).max() <= 1e-13
        assert np.abs(a2.reshape(2, n1)[k] - a1).max() <= 1e-13
    # the z-momentum residual is O(1) here, not round-off: the test sees the z faces
    assert np.abs(R1[3]).max() > 1e-3 * np.abs(R1[1:4]).max()
