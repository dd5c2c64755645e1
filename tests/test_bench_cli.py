"""bench.py's host-side pieces on CPU: the committed profile's traffic line that the roofline
reads, the byte counts it reports, the --mesh option of the single-form runs and its checks."""
import subprocess
import sys
from pathlib import Path

import bench
from plens_gb300 import configs

ROOT = Path(__file__).resolve().parent.parent


def test_traffic_line_of_the_volume_profile_parses():
    t = bench._traffic_from_profile("k_volume_mx_dmr.md")
    assert t is not None and t > 0
    # a stage-1 launch moves less than the 282 B per DoF-stage average of all five stages plus
    # the register reads it does not make, and more than its reads alone
    assert 134 * 921600 * 0.9 < t < 282 * 921600


def test_byte_counts():
    assert bench.BYTES_PER_DOF_STAGE["learned"] == 280 - 40 // 5
    assert bench.MOVED_BYTES_MIXED == 80 + 56 + 32 + 36 + 8 + 40 + 30


def test_mesh_option_replaces_the_cell_counts():
    case = configs.make_case(bench._spec("shock_vortex", "mixed", "learned", (8,)))
    assert case.n_cells == 8 ** 3
    case = configs.make_case(bench._spec("dmr", "mixed", "modal", (24, 6)))
    assert case.n_cells == 24 * 6


def test_mesh_option_is_checked():
    for extra in (["--mesh", "8"], ["--form", "learned", "--workload", "shock_vortex", "--mesh", "8,8"]):
        r = subprocess.run([sys.executable, str(ROOT / "bench.py"), *extra], capture_output=True, text=True,
                           timeout=120)
        assert r.returncode == 2, r.stderr
        assert "--mesh" in r.stderr
