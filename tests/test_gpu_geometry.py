"""Geometry setup on the GPU (plens_gpu_setup_geometry): with ``GB300/geometry setup = gpu`` the
metric terms (calc_metric_terms / MetricTerms<3>::reinit, dgsem/metric_terms.cc:67-142), the
face-dof matches and normals (form_neighbor_face_matchings, dgsem/plens.cc:1574-1627) and the
error-norm quadrature must be the host setup's bits, on straight, split, periodic and curved
(cylinder manifold, mapping degree 3) meshes, and a mesh error must read the same."""
import numpy as np
import pytest

from helpers import mirrored_box_prm
from plens_gb300 import configs
from plens_gb300.api import Case, PlensError

pytestmark = pytest.mark.gpu


def _bits_equal(a, b):
    if a is None or b is None:
        return a is None and b is None
    a, b = np.asarray(a), np.asarray(b)
    if a.shape != b.shape:
        return False
    if a.dtype.kind == "f":
        return np.array_equal(a.view(np.uint64 if a.itemsize == 8 else np.uint32),
                              b.view(np.uint64 if b.itemsize == 8 else np.uint32))
    return np.array_equal(a, b)


def _compare(spec, mapping_degree=3):
    host = configs.make_case(spec, mapping_degree=mapping_degree)
    gpu = configs.make_case(configs.with_gpu_geometry(spec), mapping_degree=mapping_degree)
    mh, mg = host.mesh_arrays(), gpu.mesh_arrays()
    assert mh.keys() == mg.keys()
    diff = [k for k in mh if not _bits_equal(mh[k], mg[k])]
    assert not diff, f"GPU geometry differs from the host's in {diff}"
    assert _bits_equal(host.dof_xyz(), gpu.dof_xyz())
    assert _bits_equal(host.initial_state(), gpu.initial_state())
    return mh


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5])
def test_box_with_split_boundary(degree):
    m = _compare(configs.dmr(nx=24, ny=6, degree=degree))
    assert m["n_face_tasks"] > 0


def test_periodic_box():
    _compare(configs.sod(n=12))
    _compare(configs.shock_vortex(n=5))


def test_curved_cylinder_with_error_norm_quadrature():
    spec = configs.with_error_norms(configs.cylinder(n_radial=10, n_azimuthal=12), conv_exact="1 + x*y")
    m = _compare(spec)
    assert m["q_wJ"] is not None and m["q_xyz"] is not None
    # curved cells: the metric terms vary inside a cell
    assert np.ptp(m["detJ"][:64]) > 0


def test_curved_mapping_degrees():
    for mdeg in (1, 2, 4):
        _compare(configs.cylinder(n_radial=6, n_azimuthal=8), mapping_degree=mdeg)


def test_non_positive_jacobian_is_reported(tmp_path):
    with pytest.raises(PlensError, match="cell 0 has a non-positive Jacobian"):
        Case(mirrored_box_prm(tmp_path, "gpu"), 2, base_dir=str(tmp_path))
