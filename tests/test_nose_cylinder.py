"""The nose-cylinder manifold of the host setup (manifolds/nose_cylinder.cc:15-78): cells beyond
the plane through the separation point normal to the axis are spherical about the nose centre,
the others cylindrical about the axis through the separation point.

- With the plane beyond every cell, the metric terms are those of the cylinder manifold.
- A spherical shell patch read from a gmsh file, all beyond the plane, bounded by two spheres and
  four planes through the centre (great circles: the directions (1, a, b)/|.| of a rectangle
  a x b): its volume from the metric terms (sum of det J times the GLL weights) approaches the
  exact one, (r2^3 - r1^3)/3 times the patch's solid angle, to 2e-6 with the cubic mapping on
  2 x 3 x 2 cells against 3e-2 for the straight (trilinear) mesh -- the support points lie on the spheres and the planes.
- The reference's two checks: the nose centre on the spherical side, a cell centre on the plane.
"""
import math

import numpy as np
import pytest

from plens_gb300 import configs
from plens_gb300.api import Case, PlensError, gll_1d

R1, R2, AA, BB = 1.0, 2.0, (-0.3, 0.3), (-0.2, 0.4)


def _cyl_prm(subtype_block: str) -> tuple:
    prm, files, deg = configs.cylinder(n_radial=4, n_azimuthal=12)
    old = """    set curved subtype = cylinder
    subsection cylinder
        set axis direction = 0 0 1
        set axis point = 0 0 0
    end"""
    assert old in prm
    return prm.replace(old, subtype_block), files, deg


def test_nose_cylinder_before_the_plane_is_the_cylinder_manifold():
    prm_c, _, deg = _cyl_prm("""    set curved subtype = cylinder
    subsection cylinder
        set axis direction = 0 0 1
        set axis point = 0 0 0
    end""")
    prm_n, _, _ = _cyl_prm("""    set curved subtype = nose cylinder
    subsection nose cylinder
        set axis direction = 0 0 1
        set separation point = 0 0 10
        set nose center = 0 0 5
    end""")
    a = Case(prm_c, deg, 3).mesh_arrays()
    b = Case(prm_n, deg, 3).mesh_arrays()
    for k in ("detJ", "Ja", "Jinv"):
        np.testing.assert_allclose(b[k], a[k], rtol=1e-12, atol=1e-12 * np.abs(a[k]).max())


def _shell_msh(path, nr=2, nt=3, npp=2):
    """A structured shell patch r x a x b (direction (1, a, b)/|.|), cells numbered r fastest;
    every boundary face tagged 1..6 (-r, +r, -a, +a, -b, +b)."""
    def node(i, j, k):
        return 1 + i + (nr + 1) * (j + (nt + 1) * k)
    lines = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$Nodes", str((nr + 1) * (nt + 1) * (npp + 1))]
    for k in range(npp + 1):
        for j in range(nt + 1):
            for i in range(nr + 1):
                r = R1 + (R2 - R1) * i / nr
                a = AA[0] + (AA[1] - AA[0]) * j / nt
                b = BB[0] + (BB[1] - BB[0]) * k / npp
                n = math.sqrt(1 + a * a + b * b)
                lines.append(f"{node(i, j, k)} {r / n!r} {r * a / n!r} {r * b / n!r}")
    lines += ["$EndNodes", "$Elements"]
    gm = [0, 1, 3, 2, 4, 5, 7, 6]
    faces = {1: (0, 2, 6, 4), 2: (1, 3, 7, 5), 3: (0, 1, 5, 4), 4: (2, 3, 7, 6), 5: (0, 1, 3, 2), 6: (4, 5, 7, 6)}
    elems = []
    for k in range(npp):
        for j in range(nt):
            for i in range(nr):
                corners = [node(i + (v & 1), j + ((v >> 1) & 1), k + (v >> 2)) for v in range(8)]
                on = {1: i == 0, 2: i == nr - 1, 3: j == 0, 4: j == nt - 1, 5: k == 0, 6: k == npp - 1}
                for bid, f in faces.items():
                    if on[bid]:
                        elems.append(f"3 2 {bid} {bid} " + " ".join(str(corners[v]) for v in f))
                elems.append("5 2 1 1 " + " ".join(str(corners[gm[v]]) for v in range(8)))
    lines.append(str(len(elems)))
    lines += [f"{n + 1} {e}" for n, e in enumerate(elems)]
    lines.append("$EndElements")
    (path / "shell.msh").write_text("\n".join(lines) + "\n")


def _shell_prm(curved: bool, nose="0 0 0", sep="0.1 0 0") -> str:
    mesh = ("    set type = curved\n    set curved subtype = nose cylinder\n    subsection nose cylinder\n"
            f"        set axis direction = 1 0 0\n        set separation point = {sep}\n"
            f"        set nose center = {nose}\n    end\n") if curved else "    set type = straight\n"
    bcs = "".join(f"  subsection bid{b}\n    set type = free\n  end\n" for b in range(1, 7))
    return ("subsection mesh\n" + mesh + "    set format = msh\n    set file name = shell.msh\nend\n"
            "subsection Navier-Stokes\n  set gas name = air\nend\nsubsection IC\n  set type = uniform\nend\n"
            "subsection BCs\n" + bcs + "end\n")


def _volume(case: Case, degree: int) -> float:
    m = case.mesh_arrays()
    _, w = gll_1d(degree + 1)
    w3 = np.einsum("i,j,k->kji", w, w, w).ravel()
    return float((m["detJ"].reshape(-1, (degree + 1) ** 3) * w3).sum())


def test_spherical_shell_sector_volume(tmp_path):
    _shell_msh(tmp_path)
    F = lambda a, b: math.atan(a * b / math.sqrt(1 + a * a + b * b))  # noqa: E731
    omega = F(AA[1], BB[1]) - F(AA[0], BB[1]) - F(AA[1], BB[0]) + F(AA[0], BB[0])
    exact = (R2 ** 3 - R1 ** 3) / 3 * omega
    curved = _volume(Case(_shell_prm(True), 3, 3, base_dir=str(tmp_path)), 3)
    straight = _volume(Case(_shell_prm(False), 3, 1, base_dir=str(tmp_path)), 3)
    e_c, e_s = abs(curved / exact - 1), abs(straight / exact - 1)
    print(f"\nshell sector volume: exact {exact:.12f}, nose-cylinder manifold rel err {e_c:.2e}, straight {e_s:.2e}")
    assert e_c < 2e-6  # the cubic mapping's error on 2 x 3 x 2 cells
    assert e_s > 1e4 * e_c


def test_nose_cylinder_checks(tmp_path):
    _shell_msh(tmp_path)
    with pytest.raises(PlensError, match="nose center lies in spherical region"):
        Case(_shell_prm(True, nose="1 0 0"), 3, 3, base_dir=str(tmp_path))
    # a cell centre on the plane: one box cell [1, 2] x [0, 1]^2 (centre x = 1.5 exactly)
    bcs = "".join(f"  subsection bid{b}\n    set type = free\n  end\n" for b in range(1, 7))
    prm = ("subsection mesh\n    set type = curved\n    set format = builtin\n"
           "    set curved subtype = nose cylinder\n    subsection nose cylinder\n"
           "        set axis direction = 1 0 0\n        set separation point = 1.5 0 0\n"
           "        set nose center = 0 0 0\n    end\n    subsection builtin\n        set generator = box\n"
           "        set lower corner = 1 0 0\n        set upper corner = 2 1 1\n        set subdivisions = 1 1 1\n"
           "        set boundary ids = 1 2 3 4 5 6\n    end\nend\n"
           "subsection Navier-Stokes\n  set gas name = air\nend\nsubsection IC\n  set type = uniform\nend\n"
           "subsection BCs\n" + bcs + "end\n")
    with pytest.raises(PlensError, match="bifurcation plane"):
        Case(prm, 3, 3)
