"""The synthetic workloads, written as input.prm text in the reference's format.

Each function returns ``(prm_text, files, fe_degree)`` where ``files`` maps file names (relative
to the case directory) to their contents, e.g. the piecewise-function IC file
(IBCs/piecewise_function.cc:100-190 format). Sizes default to the full configurations; smaller
``n`` values give the parity-test cases of the same physics.

- ``sod``: 3D Sod shock tube, 200x1x1 cells, N=2, periodic y/z, seeded density noise 1e-4.
- ``dmr``: double Mach reflection, [0,4]x[0,1]x[0,0.0167], 240x60x1 cells, N=3, periodic z,
  BCs of study1/dmr/scripts/base_input.prm:17-50, pre-shock density noise 1e-6.
- ``cylinder``: Mach 8, Re_D=1e5 laminar flow over a cylinder of radius 1 (cylinder manifold),
  160 radial x 128 azimuthal x 1 O-mesh clustered to 1e-3 R, N=3, isothermal 300 K wall,
  Sutherland viscosity, Pr=0.72, velocity noise 1e-5.
- ``shock_vortex``: periodic cube [0,2pi]^3, 64^3 cells, N=3, mu=1e-4 constant, random-phase
  solenoidal field at Mt=0.6 plus a Mach-3 shock at x=pi.
"""
from __future__ import annotations

import math
import tempfile
from pathlib import Path

SOD_IC = """p
2
1
1
0.5


1
0
0
0
1
0.125
0
0
0
0.1
"""


def _gb300(precision: str, sensor: str, extra: str = "") -> str:
    return f"""
subsection GB300
    set precision = {precision}
    set sensor = {sensor}
    set judge every = 25
    set judge alpha tolerance = 0.05
{extra}end
"""


def sod(n: int = 200, precision="fp64", sensor="modal", courant=0.5, end_time=1.0, noise=1e-4):
    prm = f"""
subsection mesh
    set type = straight
    set format = builtin
    subsection builtin
        set generator = box
        set lower corner = 0 0 0
        set upper corner = 1 0.005 0.005
        set subdivisions = {n} 1 1
        set boundary ids = 1 2 3 4 5 6
    end
end
subsection Navier-Stokes
    set gas name = air
    set inviscid = true
    set inviscid surface flux scheme = HLLC
    set inviscid volume flux scheme = Chandrashekhar
end
subsection IC
    set type = piecewise function
    set file name = ic.dat
    subsection noise
        set variable = rho
        set amplitude = {noise}
        set seed = 1
    end
end
subsection BCs
    subsection bid1
        set type = free
    end
    subsection bid2
        set type = free
    end
    subsection bid3
        set type = periodic
        set periodic direction = 1
        set periodic orientation = left
        set other surface boundary id = 4
    end
    subsection bid4
        set type = periodic
        set periodic direction = 1
        set periodic orientation = right
        set other surface boundary id = 3
    end
    subsection bid5
        set type = periodic
        set periodic direction = 2
        set periodic orientation = left
        set other surface boundary id = 6
    end
    subsection bid6
        set type = periodic
        set periodic direction = 2
        set periodic orientation = right
        set other surface boundary id = 5
    end
end
subsection blender parameters
    set variable = pxrho
    set blender max value = 0.5
end
subsection time integration
    set RK order = 4
    set Courant number = {courant}
    set end time = {end_time}
end
subsection data output
    set write frequency = 1000000
end
""" + _gb300(precision, sensor)
    return prm, {"ic.dat": SOD_IC}, 2


def dmr(nx: int = 240, ny: int = 60, precision="fp64", sensor="modal", end_time=0.2, noise=1e-6,
        degree=3, z_bc="periodic", nz: int = 1, plens_2d: bool = False):
    """Double Mach reflection. z_bc: "periodic" (the benchmark configuration) or "symmetry" (the
    z boundaries of the reference's own input, study1/dmr/scripts/base_input.prm:43-48); nz cells
    of 0.0167 each across z; plens_2d: the reference's PLENS_2D switch (the z-momentum RHS set to
    zero, dgsem/plens.cc:3772-3774), which keeps the flow two-dimensional."""
    if z_bc == "periodic":
        z_bcs = """    subsection bid5
        set type = periodic
        set periodic direction = 2
        set periodic orientation = left
        set other surface boundary id = 6
    end
    subsection bid6
        set type = periodic
        set periodic direction = 2
        set periodic orientation = right
        set other surface boundary id = 5
    end"""
    elif z_bc == "symmetry":
        z_bcs = """    subsection bid5
        set type = symmetry
    end
    subsection bid6
        set type = symmetry
    end"""
    else:
        raise ValueError(z_bc)
    prm = f"""
subsection mesh
    set type = straight
    set format = builtin
    subsection builtin
        set generator = box
        set lower corner = 0 0 0
        set upper corner = 4 1 {0.0167 * nz!r}
        set subdivisions = {nx} {ny} {nz}
        set boundary ids = 1 3 1 2 5 6
        set split -y side at x = 0.16666666666666666
        set split boundary id = 4
    end
end
subsection Navier-Stokes
    set gas name = air
    set inviscid = true
    set inviscid surface flux scheme = HLLC
    set inviscid volume flux scheme = Chandrashekhar
end
subsection IC
    set type = double mach reflection
    subsection noise
        set variable = pre-shock rho
        set amplitude = {noise}
        set seed = 2
    end
end
subsection BCs
    subsection bid1
        set type = uniform inflow
        set prescribed p = 116.5
        set prescribed velocity = 7.144709581221619 -4.125 0
        set prescribed T = 0.050792519
    end
    subsection bid2
        set type = varying inflow
        set prescribed p = ( x - 1.3213672 - 11.547005*t > 0 ? 1 : 116.5 )
        set prescribed T = ( x - 1.3213672 - 11.547005*t > 0 ? 0.0024913559 : 0.050792519 )
        set prescribed velocity = ( x - 1.3213672 - 11.547005*t > 0 ? 0 : 7.144709581221619 );\\
                                  ( x - 1.3213672 - 11.547005*t > 0 ? 0 : -4.125);\\
                                  0
    end
    subsection bid3
        set type = uniform inflow
        set prescribed p = 1
        set prescribed velocity = 0 0 0
        set prescribed T = 0.0024913559
    end
    subsection bid4
        set type = uniform temp wall
    end
{z_bcs}
end
subsection blender parameters
    set variable = pxrho
    set wall blender limit = 0
end
subsection time integration
    set RK order = 4
    set Courant number = 0.5
    set end time = {end_time}
end
subsection data output
    set write frequency = 1000000
end
""" + _gb300(precision, sensor, "    set 2d = true\n" if plens_2d else "")
    return prm, {}, degree


def _local_stepping(local: dict | None) -> str:
    """The "time integration" lines of local time stepping: ``local`` = dict(start=t0,
    limit=bool, neighbor=factor, global_=factor); None keeps global stepping."""
    if not local:
        return ""
    return (f"    set request local stepping = true\n"
            f"    set local stepping start time = {local.get('start', 0.0)!r}\n"
            f"    set limit local time step = {'true' if local.get('limit', False) else 'false'}\n"
            f"    set local step neighbor factor = {local.get('neighbor', 1.05)!r}\n"
            f"    set local step global factor = {local.get('global_', 1000.0)!r}\n")


def cylinder(n_radial: int = 160, n_azimuthal: int = 128, precision="fp64", sensor="modal",
             end_time=1e9, courant=0.3, mapping_degree_note=True, local: dict | None = None,
             wall_bc="uniform temp wall", inflow_bc="uniform inflow", z_bc="periodic"):
    """Laminar Mach-8 cylinder. The boundary types can be swapped for the BC parity cases:
    wall_bc "uniform temp wall" | "insulated wall", inflow_bc "uniform inflow" | "ZPG inflow",
    z_bc "periodic" | "symmetry" | "empty"."""
    gamma, Rgas, Tinf, Mach, Re, D = 1.4, 287.0, 200.0, 8.0, 1e5, 2.0
    pinf = 100.0
    rho = pinf / (Rgas * Tinf)
    u = Mach * math.sqrt(gamma * Rgas * Tinf)
    mu_inf = rho * u * D / Re
    T0, S = 273.0, 111.0
    mu0 = mu_inf / ((Tinf / T0) ** 1.5 * (T0 + S) / (Tinf + S))
    MW = 8.314462618 / Rgas
    if z_bc == "periodic":
        z_bcs = """    subsection bid4
        set type = periodic
        set periodic direction = 2
        set periodic orientation = left
        set other surface boundary id = 5
    end
    subsection bid5
        set type = periodic
        set periodic direction = 2
        set periodic orientation = right
        set other surface boundary id = 4
    end"""
    elif z_bc in ("symmetry", "empty"):
        z_bcs = f"""    subsection bid4
        set type = {z_bc}
    end
    subsection bid5
        set type = {z_bc}
    end"""
    else:
        raise ValueError(z_bc)
    prm = f"""
subsection mesh
    set type = curved
    set format = builtin
    set curved subtype = cylinder
    subsection cylinder
        set axis direction = 0 0 1
        set axis point = 0 0 0
    end
    subsection builtin
        set generator = o-mesh
        set inner radius = 1
        set outer radius = 10
        set radial cells = {n_radial}
        set azimuthal cells = {n_azimuthal}
        set first cell height = 1e-3
        set z cells = 1
        set z length = 0.05
        set o-mesh boundary ids = 1 2 3 4 5
    end
end
subsection Navier-Stokes
    set gas name = custom
    set gamma = {gamma}
    set molecular weight = {MW!r}
    set Prandtl number = 0.72
    set mu0 = {mu0!r}
    set T0 = {T0}
    set S = {S}
    set inviscid surface flux scheme = HLLC
    set inviscid volume flux scheme = Chandrashekhar
end
subsection IC
    set type = uniform
    subsection uniform
        set primitive state = {rho!r} {u!r} 0 0 {pinf!r}
        set wall damping radius = 1
        set wall damping length = 0.5
    end
    subsection noise
        set variable = velocity
        set amplitude = 1e-5
        set seed = 3
    end
end
subsection BCs
    subsection bid1
        set type = {wall_bc}
        set prescribed T = 300
        set prescribed velocity = 0 0 0
    end
    subsection bid2
        set type = {inflow_bc}
        set prescribed p = {pinf!r}
        set prescribed T = {Tinf!r}
        set prescribed velocity = {u!r} 0 0
    end
    subsection bid3
        set type = outflow
        set prescribed p = {pinf!r}
    end
{z_bcs}
end
subsection blender parameters
    set variable = pxrho
    set wall blender limit = 0
end
subsection time integration
    set RK order = 4
    set Courant number = {courant}
    set end time = {end_time}
{_local_stepping(local)}end
subsection data output
    set write frequency = 1000000
end
""" + _gb300(precision, sensor)
    return prm, {}, 3


def shock_vortex(n: int = 64, precision="fp64", sensor="modal", end_time=1e9, modes=8):
    L = 2 * math.pi
    prm = f"""
subsection mesh
    set type = straight
    set format = builtin
    subsection builtin
        set generator = box
        set lower corner = 0 0 0
        set upper corner = {L!r} {L!r} {L!r}
        set subdivisions = {n} {n} {n}
        set boundary ids = 1 2 3 4 5 6
    end
end
subsection Navier-Stokes
    set gas name = custom
    set gamma = 1.4
    set molecular weight = 0.028
    set Prandtl number = 0.72
    set mu0 = 1e-4
    set inviscid surface flux scheme = HLLC
    set inviscid volume flux scheme = Chandrashekhar
end
subsection IC
    set type = shock vortex
    subsection shock vortex
        set turbulent Mach number = 0.6
        set shock Mach number = 3
        set shock x = {math.pi!r}
        set modes = {modes}
    end
    subsection noise
        set seed = 4
    end
end
subsection BCs
""" + "".join(
        f"""    subsection bid{2 * d + 1}
        set type = periodic
        set periodic direction = {d}
        set periodic orientation = left
        set other surface boundary id = {2 * d + 2}
    end
    subsection bid{2 * d + 2}
        set type = periodic
        set periodic direction = {d}
        set periodic orientation = right
        set other surface boundary id = {2 * d + 1}
    end
""" for d in range(3)) + f"""end
subsection blender parameters
    set variable = pxrho
end
subsection time integration
    set RK order = 4
    set Courant number = 0.3
    set end time = {end_time}
end
subsection data output
    set write frequency = 1000000
end
""" + _gb300(precision, sensor, "    set constant viscosity = true\n")
    return prm, {}, 3


def with_error_norms(spec, ss_error: bool = True, conv_exact: str | None = None):
    """``spec`` with the error norms of the output steps set: the steady-state error on or off,
    and the density convergence error against ``conv_exact`` (an expression of x, y, z, t)."""
    prm, files, degree = spec
    lines = f"    set calculate steady state error = {'true' if ss_error else 'false'}\n"
    if conv_exact is not None:
        lines += ("    subsection convergence\n        set calculate error = true\n"
                  "        set variable = density\n"
                  f"        set exact solution = {conv_exact}\n    end\n")
    key = "subsection data output\n"
    assert prm.count(key) == 1
    return prm.replace(key, key + lines), files, degree


def with_gpu_geometry(spec):
    """``spec`` with the metric terms and face dofs computed on the GPU (``GB300/geometry setup``)."""
    prm, files, degree = spec
    key = "subsection GB300\n"
    assert prm.count(key) == 1
    return prm.replace(key, key + "    set geometry setup = gpu\n"), files, degree


def make_case(spec, mapping_degree: int = 3):
    """Writes the auxiliary files of ``spec`` into a temporary directory and builds the Case."""
    from .api import Case

    prm, files, degree = spec
    d = Path(tempfile.mkdtemp(prefix="plens_case_"))
    for name, text in files.items():
        (d / name).write_text(text)
    (d / "input.prm").write_text(prm)
    return Case(prm, degree, mapping_degree=mapping_degree, base_dir=str(d))
