"""Host setup chain: input.prm parsing, expressions, 1D operators, mesh tables and metric terms,
including the reference's own known-answer checks (face_dof_info.h:82-90,
metric_terms.cc:228-235)."""
import math

import numpy as np
import pytest

from helpers import make, mirrored_box_prm
from plens_gb300 import configs
from plens_gb300.api import Case, PlensError, eval_expression, gll_1d


# ------------------------------------------------------------------------- expressions

@pytest.mark.parametrize("src,vars_,val", [
    ("1+2*3", {}, 7.0),
    ("-2^2", {}, -4.0),                       # muparser: unary minus binds weaker than ^
    ("2^3^2", {}, 512.0),                     # right associative
    ("(x > 1 ? 3 : 4)", {"x": 2}, 3.0),
    ("(x > 1 ? 3 : 4)", {"x": 0}, 4.0),
    ("sin(pi/2) + cos(0) + sqrt(16)", {}, 6.0),
    ("min(3, x, 1) + max(2, y)", {"x": 0.5, "y": 7}, 7.5),
    ("x - 1.3213672 - 11.547005*t > 0 ? 1 : 116.5", {"x": 2.0, "t": 0.01}, 1.0),
    ("x - 1.3213672 - 11.547005*t > 0 ? 1 : 116.5", {"x": 1.0, "t": 0.01}, 116.5),
    ("t < 1e-3 ? abs(y-10e-3) : -1", {"y": 0.02, "t": 0.0}, 0.01),
    ("if(x < 0, -1, 1) * exp(log(2))", {"x": -3}, -2.0),
    ("x>=1 && y<=2 || z==3", {"x": 0, "y": 0, "z": 3}, 1.0),
])
def test_expression_values(src, vars_, val):
    assert eval_expression(src, **vars_) == pytest.approx(val, rel=1e-14, abs=1e-14)


@pytest.mark.parametrize("src", ["1+", "foo(2)", "(1", "x ? 1", "1 2"])
def test_expression_errors(src):
    with pytest.raises(PlensError):
        eval_expression(src)


# -------------------------------------------------------------------------- 1D operators

@pytest.mark.parametrize("n", [2, 3, 4, 5, 6])
def test_gll_rule(n):
    x, w = gll_1d(n)
    assert x[0] == 0 and x[-1] == 1
    np.testing.assert_allclose(x + x[::-1], 1.0, atol=1e-15)
    np.testing.assert_allclose(w.sum(), 1.0, rtol=1e-15)
    for k in range(2 * n - 2):  # exact up to degree 2N-1 = 2n-3
        assert (w * x ** k).sum() == pytest.approx(1.0 / (k + 1), rel=1e-13)


# ------------------------------------------------------------------------------- prm

def test_prm_errors_name_the_line():
    prm, files, deg = configs.sod(n=4)
    with pytest.raises(PlensError, match="undeclared entry"):
        make((prm + "\nsubsection mesh\n  set colour = red\nend\n", files, deg))
    with pytest.raises(PlensError, match="missing 'end'"):
        make((prm + "\nsubsection mesh\n", files, deg))
    bad = prm.replace("set type = free", "set type = none", 1)
    with pytest.raises(PlensError, match="'none' type BC"):
        make((bad, files, deg))


def test_prm_echo_round_trip():
    c = make(configs.dmr(nx=4, ny=2))
    echo = c.prm_echo()
    assert "set prescribed p = ( x - 1.3213672 - 11.547005*t > 0 ? 1 : 116.5 )" in echo
    assert "subsection blender parameters" in echo
    # the echo parses back into an identical case
    c2 = Case(echo, 3)
    np.testing.assert_array_equal(c2.initial_state(), c.initial_state())


# ---------------------------------------------------------------------- face dof maps
# FaceDoFInfo known answer for N=2 (dgsem/face_dof_info.h:82-90)
KAT_N2 = [
    [0, 3, 6, 9, 12, 15, 18, 21, 24],
    [2, 5, 8, 11, 14, 17, 20, 23, 26],
    [0, 1, 2, 9, 10, 11, 18, 19, 20],
    [6, 7, 8, 15, 16, 17, 24, 25, 26],
    [0, 1, 2, 3, 4, 5, 6, 7, 8],
    [18, 19, 20, 21, 22, 23, 24, 25, 26],
]


def test_face_dof_map_known_answer():
    """Face tasks carry the location of each face dof; it must be the cell dof the reference's
    N=2 face map names."""
    c = make(configs.dmr(nx=3, ny=2, degree=2))
    m = c.mesh_arrays()
    X = c.dof_xyz()
    seen = set()
    for ti in range(m["n_face_tasks"]):
        cell, f = m["ft_cell"][ti], m["ft_face"][ti]
        for q in range(9):
            dof = cell * 27 + KAT_N2[f][q]
            np.testing.assert_array_equal(m["ft_xyz"][ti, q], X[:, dof])
        seen.add(f)
    assert seen == set(range(6))


def test_interior_faces_match_neighbour_locations():
    c = make(configs.cylinder(n_radial=4, n_azimuthal=8))
    m = c.mesh_arrays()
    X = c.dof_xyz()
    P = 4
    fmap = {f: [0] * 16 for f in range(6)}
    for f in range(6):
        for q in range(16):
            a, b = q % P, q // P
            fmap[f][q] = [P * q, 3 + P * q, a + 16 * b, 12 + a + 16 * b, q, 48 + q][f]
    n_int = 0
    for ti in range(m["n_face_tasks"]):
        if m["ft_bc"][ti] >= 0:
            continue
        n_int += 1
        c0, f0, c1, f1 = m["ft_cell"][ti], m["ft_face"][ti], m["ft_nbr_cell"][ti], m["ft_nbr_face"][ti]
        assert c0 < c1
        for q in range(16):
            q1 = m["ft_nbr_fdof"][ti, q]
            np.testing.assert_allclose(X[:, c0 * 64 + fmap[f0][q]], X[:, c1 * 64 + fmap[f1][q1]], atol=1e-12)
    # O-mesh: every interior face appears once (radial + azimuthal incl. the seam)
    assert n_int == 3 * 8 + 4 * 8


def test_periodic_partners_and_outward_normals():
    c = make(configs.sod(n=6))
    m = c.mesh_arrays()
    for ti in range(m["n_face_tasks"]):
        f = m["ft_face"][ti]
        sgn = -1 if f % 2 == 0 else 1
        n = m["ft_normal"][ti]
        expect = np.zeros(3)
        expect[f // 2] = sgn
        np.testing.assert_allclose(n, np.tile(expect, (9, 1)), atol=1e-15)
        if m["ft_bc"][ti] in (3, 4, 5, 6):  # periodic: 1-cell wide, partner is the same cell
            assert m["ft_nbr_cell"][ti] == m["ft_cell"][ti]
            assert m["ft_nbr_face"][ti] == f ^ 1


# ---------------------------------------------------------------------- metric terms

def _rotated_box_msh(path, r):
    """One hexahedron: the box [0,4]x[0,2]x[0,1] rotated by r about z (metric_terms.cc:148-236)."""
    c, s = math.cos(r), math.sin(r)
    pts = [(x, y, z) for z in (0, 1) for y in (0, 2) for x in (0, 4)]  # lexicographic
    rot = [(c * x - s * y, s * x + c * y, z) for (x, y, z) in pts]
    gm = [0, 1, 3, 2, 4, 5, 7, 6]  # gmsh hexahedron order from lexicographic
    faces = {1: (0, 2, 6, 4), 2: (1, 3, 7, 5), 3: (0, 1, 5, 4), 4: (2, 3, 7, 6), 5: (0, 1, 3, 2), 6: (4, 5, 7, 6)}
    lines = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$Nodes", "8"]
    lines += [f"{i + 1} {p[0]!r} {p[1]!r} {p[2]!r}" for i, p in enumerate(rot)]
    lines += ["$EndNodes", "$Elements", "7"]
    eid = 1
    for bid, f in faces.items():
        lines.append(f"{eid} 3 2 {bid} {bid} " + " ".join(str(v + 1) for v in f))
        eid += 1
    lines.append(f"{eid} 5 2 1 1 " + " ".join(str(gm[k] + 1) for k in range(8)))
    lines.append("$EndElements")
    path.write_text("\n".join(lines) + "\n")


def test_metric_terms_rotated_box_known_answer(tmp_path):
    r = math.radians(30)
    _rotated_box_msh(tmp_path / "box.msh", r)
    prm = """
subsection mesh
  set type = straight
  set format = msh
  set file name = box.msh
end
subsection Navier-Stokes
  set gas name = air
end
subsection IC
  set type = uniform
end
subsection BCs
""" + "".join(f"  subsection bid{b}\n    set type = free\n  end\n" for b in range(1, 7)) + "end\n"
    c = Case(prm, 2, base_dir=str(tmp_path))
    m = c.mesh_arrays()
    Ja = m["Ja"]  # [dir][comp][dof]
    expect = np.array([[2 * math.cos(r), 2 * math.sin(r), 0], [-4 * math.sin(r), 4 * math.cos(r), 0], [0, 0, 8]])
    for d in range(3):
        np.testing.assert_allclose(Ja[d].T, np.tile(expect[d], (27, 1)), atol=1e-13)
    np.testing.assert_allclose(m["detJ"], 8.0, rtol=1e-14)
    assert m["h_min"][0] == pytest.approx(1.0)


# ------------------------------------------------------------------- geometry setup switch

def test_geometry_setup_switch(tmp_path):
    """"GB300/geometry setup" takes host|gpu; gpu needs the GPU library's geometry function, which
    plens_case_create (without _ex) does not pass; the host computes a non-positive Jacobian
    error as the reference's setup would stop on it."""
    from plens_gb300.api import host_lib
    prm, files, deg = configs.sod(n=4)
    with pytest.raises(PlensError, match="must be host[|]gpu"):
        make((prm.replace("subsection GB300\n", "subsection GB300\n    set geometry setup = cpu\n"), files, deg))
    L = host_lib()
    import ctypes
    h = ctypes.c_void_p()
    gprm = configs.with_gpu_geometry((prm, files, deg))[0]
    assert L.plens_case_create(gprm.encode(), b".", 3, deg, ctypes.byref(h)) != 0
    assert b"needs the GPU library's geometry function" in L.plens_case_last_error()
    with pytest.raises(PlensError, match="cell 0 has a non-positive Jacobian"):
        Case(mirrored_box_prm(tmp_path, "host"), 2, base_dir=str(tmp_path))


def test_setup_phase_times():
    """The setup reports its phase times (mesh, geometry, topology, initial condition)."""
    c = make(configs.dmr(nx=12, ny=4))
    t = c.setup_times()
    assert list(t) == ["mesh", "geometry", "topology", "initial_condition"]
    assert all(v >= 0 for v in t.values()) and t["geometry"] > 0
