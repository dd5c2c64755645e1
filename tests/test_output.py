"""Data output and restart (PLENS::write / post_process, dgsem/plens.cc:4170-4322, 3950-3963, and the
"from archive restart" initial condition, IBCs/from_archive_restart.cc:23-73): the VTU file decodes
to the mesh's GLL nodes, the state and the post-processed p, T, velocity; an archive round-trips
the state bit for bit and restarts a case with it."""
import base64
import struct
import xml.etree.ElementTree as ET

import numpy as np

from helpers import make
from plens_gb300 import configs
from plens_gb300.api import write_pvd

DTYPES = {"Float64": "<f8", "Float32": "<f4", "Int64": "<i8", "UInt8": "u1"}


def _decode(da):
    """A binary inline DataArray: base64 UInt64 byte count, then base64 data."""
    txt = "".join(da.text.split())
    nbytes = struct.unpack("<Q", base64.b64decode(txt[:12]))[0]
    data = base64.b64decode(txt[12:])
    assert len(data) == nbytes
    return np.frombuffer(data, dtype=DTYPES[da.get("type")])


def _arrays(path):
    root = ET.parse(path).getroot()
    piece = root.find("UnstructuredGrid/Piece")
    out = {}
    for sec in ("PointData", "CellData", "Points", "Cells"):
        for da in piece.find(sec).findall("DataArray"):
            out[da.get("Name") or sec] = _decode(da)
    return int(piece.get("NumberOfPoints")), int(piece.get("NumberOfCells")), out


def test_vtu_decodes_to_state_and_post_processed_fields(tmp_path):
    case = make(configs.sod(n=12))  # N = 2
    U = case.initial_state()
    alpha = np.linspace(0, 0.5, case.n_cells)
    path = tmp_path / "out.vtu"
    case.write_vtu(path, U, alpha=alpha, alpha_d=alpha / 0.5, loc_dt=1e-3)
    npts, ncells, a = _arrays(path)
    N = 2
    assert npts == case.n_dofs and ncells == case.n_cells * N ** 3
    np.testing.assert_array_equal(a["Points"].reshape(-1, 3), case.dof_xyz().T)
    np.testing.assert_array_equal(a["rho"], U[0])
    g = case.params.gamma
    p = (g - 1) * (U[4] - 0.5 * (U[1] ** 2 + U[2] ** 2 + U[3] ** 2) / U[0])
    np.testing.assert_allclose(a["p"], p, rtol=1e-15, atol=0)
    np.testing.assert_allclose(a["u"], U[1] / U[0], rtol=1e-15, atol=0)
    np.testing.assert_allclose(a["T"], p / (U[0] * case.params.R), rtol=1e-13)
    assert np.all(a["types"] == 12)
    np.testing.assert_array_equal(a["offsets"], 8 * np.arange(1, ncells + 1))
    conn = a["connectivity"].reshape(-1, 8)
    assert conn.min() == 0 and conn.max() == case.n_dofs - 1
    # each sub-hexahedron's vertices are nodes of one cell, in VTK order (x, then y, then z)
    P = N + 1
    assert np.all(conn // P ** 3 == (conn[:, :1] // P ** 3))
    np.testing.assert_array_equal(conn[0], [0, 1, 1 + P, P, P * P, 1 + P * P, 1 + P + P * P, P + P * P])
    np.testing.assert_allclose(a["alpha"], np.repeat(alpha, N ** 3).astype(np.float32))
    assert np.all(a["loc_dt"] == np.float32(1e-3))


def test_pvd_record(tmp_path):
    write_pvd(tmp_path / "o.pvd", [(0.0, "o_000000.vtu"), (0.25, "o_000001.vtu")])
    ds = ET.parse(tmp_path / "o.pvd").getroot().findall("Collection/DataSet")
    assert [(float(d.get("timestep")), d.get("file")) for d in ds] == [(0.0, "o_000000.vtu"), (0.25, "o_000001.vtu")]


def test_archive_round_trip_and_restart_ic(tmp_path):
    case = make(configs.sod(n=12))
    U = case.initial_state() * (1 + 1e-3 * np.random.default_rng(0).uniform(-1, 1, (5, case.n_dofs)))
    ar = tmp_path / "state.ar"
    case.write_archive(ar, U, 0.125, 37, 4)
    U2, t, n, k = case.read_archive(ar)
    assert (t, n, k) == (0.125, 37, 4)
    np.testing.assert_array_equal(U2, U)
    prm, files, deg = configs.sod(n=12)
    prm = (prm.replace("set type = piecewise function", "set type = from archive restart", 1)
           .replace("set file name = ic.dat", f"set file name = {ar}", 1)
           .replace("set variable = rho", "set variable = none", 1))
    restarted = make((prm, files, deg))
    np.testing.assert_array_equal(restarted.initial_state(), U)
    # another mesh is rejected
    other = make(configs.sod(n=14))
    try:
        other.read_archive(ar)
        raise AssertionError("archive of another mesh accepted")
    except Exception as e:  # noqa: BLE001
        assert "another mesh" in str(e)
