"""The modal indicator of the mixed forms at degree 3 with the change of basis on the tensor cores
(k_blender_tc: tcgen05.mma in 3xTF32 form, blender_calculator.cc:123-177 with the change of basis
matrix of change_of_basis_matrix.h:74-98; the default of such contexts) against the separable
transform on the CUDA cores.

Both are FP32-accurate; their sums run in different orders, so alpha agrees to 5e-4 (absolute;
the Hennemann sigmoid amplifies the relative difference of the energy ratios, ~1e-6, by its slope)
and the troubled-cell lists agree except for cells at the alpha_min cut. The states after 20 steps
agree to 1e-6 relative L1; the parity of each path with the FP64 oracle is the mixed form's."""
import numpy as np
import pytest

from helpers import make, rel_l1
from oracle.pyoracle import Oracle
from plens_gb300 import configs
from plens_gb300.api import GpuSolver, PlensError

pytestmark = pytest.mark.gpu


def _state(nx, ny, steps):
    case = make(configs.dmr(nx=nx, ny=ny))
    o = Oracle(case)
    o.set_state(case.initial_state(), 0.0)
    o.advance(steps)
    U, t, _, _ = o.get_state()
    return U, t


def _check_alpha(a_cc, a_tc, amin):
    assert np.abs(a_tc - a_cc).max() <= 5e-4
    flip = (a_cc > 0) != (a_tc > 0)
    assert np.all(np.maximum(a_cc, a_tc)[flip] <= amin + 5e-4)
    assert (a_cc > 0).sum() > 20  # the state has troubled cells


@pytest.mark.parametrize("prec", ["mixed", "mixed_r32"])
def test_tensor_core_indicator_matches_cuda_cores(prec):
    U, t = _state(48, 12, 10)
    case = make(configs.dmr(nx=48, ny=12, precision=prec))
    amin = case.params.alpha_min
    g = GpuSolver(case)
    g.set_indicator_tensor_cores(False)
    g.set_state(U, t)
    R_cc = g.rhs()
    a_cc = g.cell_scalars()[0]
    g.set_indicator_tensor_cores(True)
    g.set_state(U, t)
    R_tc = g.rhs()
    a_tc = g.cell_scalars()[0]
    _check_alpha(a_cc, a_tc, amin)
    assert rel_l1(R_tc, R_cc).max() <= 1e-5
    # 20 steps each way from the same state
    g.set_state(U, t)
    g.advance(20)
    U_tc = g.get_state()
    g.set_indicator_tensor_cores(False)
    g.set_state(U, t)
    g.advance(20)
    U_cc = g.get_state()
    assert rel_l1(U_tc, U_cc).max() <= 1e-6


def test_tensor_core_indicator_full_size_and_partial_tile():
    """The full double Mach reflection (14,400 cells: 112 full tiles of 128 cells and one of 64)."""
    case = make(configs.dmr(precision="mixed"))
    g = GpuSolver(case)
    g.set_indicator_tensor_cores(False)
    g.set_state(case.initial_state(), 0.0)
    g.advance(30)
    g.rhs()
    a_cc = g.cell_scalars()[0]
    g.set_indicator_tensor_cores(True)
    g.rhs()
    a_tc = g.cell_scalars()[0]
    _check_alpha(a_cc, a_tc, case.params.alpha_min)


def test_tensor_core_indicator_needs_a_mixed_degree_3_modal_context():
    for spec in (configs.dmr(nx=24, ny=6), configs.dmr(nx=24, ny=6, precision="mixed", degree=2),
                 configs.dmr(nx=24, ny=6, precision="mixed", sensor="learned")):
        g = GpuSolver(make(spec))
        with pytest.raises(PlensError):
            g.set_indicator_tensor_cores(True)
