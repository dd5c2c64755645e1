"""State I/O through the C ABI (plens_gpu_set_state / plens_gpu_get_state): a page-locked host
buffer is read and written by the GPU through its device mapping in one pass (which also writes
the mixed form's FP32 state image); any other buffer goes through the copy engines. Both must
give the same state and the same steps."""
import numpy as np
import pytest

from helpers import make
from plens_gb300 import configs
from plens_gb300.api import GpuSolver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pinned_and_pageable_state_io_agree(precision):
    torch = pytest.importorskip("torch")
    case = make(configs.dmr(nx=24, ny=6, precision=precision))
    U0 = case.initial_state()
    pageable, pinned = GpuSolver(case), GpuSolver(case)
    pageable.set_state(U0, 0.0)
    src = torch.empty(U0.shape, dtype=torch.float64).pin_memory()
    src.numpy()[:] = U0
    pinned.set_state(src.numpy(), 0.0)
    out = torch.empty(U0.shape, dtype=torch.float64).pin_memory()
    pinned.get_state(out.numpy())
    assert np.array_equal(out.numpy(), U0)
    pageable.advance(3)
    pinned.advance(3)
    Ua = pageable.get_state()
    pinned.get_state(out.numpy())
    assert np.array_equal(Ua, out.numpy())
    assert not np.array_equal(Ua, U0)
