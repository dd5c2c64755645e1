"""Shared helpers of the test suite: workload construction and the parity metrics."""
from __future__ import annotations

import numpy as np

from plens_gb300 import configs


def make(spec):
    return configs.make_case(spec)


def var_scales(X: np.ndarray) -> np.ndarray:
    """Per-equation scale of a [5][ndof] field: max |.| of rho, of the momentum vector (the three
    components jointly, so a component that is pure round-off noise in a quasi-1D flow is
    measured against the momentum it belongs to), and of rho E."""
    a = np.abs(X)
    m = a[1:4].max()
    return np.array([a[0].max(), m, m, m, a[4].max()])


def max_rel_err(X: np.ndarray, ref: np.ndarray) -> float:
    """max over equations of max_dof |X - ref| / scale(ref)."""
    s = var_scales(ref)
    s = np.where(s > 0, s, 1.0)
    return float(max(np.abs(X[v] - ref[v]).max() / s[v] for v in range(5)))


def rel_l1(X: np.ndarray, ref: np.ndarray) -> np.ndarray:
    """Relative L1 error of rho, momentum (jointly) and rho E."""
    d = np.abs(X - ref)
    a = np.abs(ref)
    return np.array([d[0].sum() / a[0].sum(), d[1:4].sum() / max(a[1:4].sum(), 1e-300), d[4].sum() / a[4].sum()])


def mirrored_box_prm(tmp_path, setup):
    """One hexahedron whose vertices are listed mirrored in x: det J < 0 everywhere."""
    pts = [(-x, y, z) for z in (0, 1) for y in (0, 2) for x in (0, 4)]
    gm = [0, 1, 3, 2, 4, 5, 7, 6]
    faces = {1: (0, 2, 6, 4), 2: (1, 3, 7, 5), 3: (0, 1, 5, 4), 4: (2, 3, 7, 6), 5: (0, 1, 3, 2), 6: (4, 5, 7, 6)}
    lines = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$Nodes", "8"]
    lines += [f"{i + 1} {p[0]!r} {p[1]!r} {p[2]!r}" for i, p in enumerate(pts)]
    lines += ["$EndNodes", "$Elements", "7"]
    for eid, (bid, f) in enumerate(faces.items(), start=1):
        lines.append(f"{eid} 3 2 {bid} {bid} " + " ".join(str(v + 1) for v in f))
    lines.append("7 5 2 1 1 " + " ".join(str(gm[k] + 1) for k in range(8)))
    lines.append("$EndElements")
    (tmp_path / "box.msh").write_text("\n".join(lines) + "\n")
    return """
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
""" + "".join(f"  subsection bid{b}\n    set type = free\n  end\n" for b in range(1, 7)) + \
        f"end\nsubsection GB300\n  set geometry setup = {setup}\nend\n"
