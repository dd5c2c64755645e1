"""The C-ABI libraries load and export every function their headers declare (no GPU needed: the
CUDA library is loaded, not called)."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _declared(header: str):
    text = (ROOT / "include" / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(plens_[a-z0-9_]+)\s*\(", text)))


def test_host_library_exports_header():
    from plens_gb300.api import host_lib
    L = host_lib()
    names = _declared("plens_host.h")
    assert "plens_case_create" in names
    for n in names:
        assert hasattr(L, n), n


def test_gpu_library_exports_header():
    from plens_gb300 import build
    lib = build.LIB / "libplens_gpu.so"
    if not lib.exists():
        build.build_gpu()
    try:
        L = C.CDLL(str(lib))
    except OSError as e:  # the CUDA runtime is part of the toolkit image; report if missing
        pytest.skip(f"CUDA runtime not loadable here: {e}")
    names = _declared("plens_gpu.h")
    assert "plens_gpu_create" in names and "plens_gpu_advance" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_gpu_library_rejects_bad_arguments_without_a_device():
    """Argument checks run before any CUDA call: null pointers are E_INVALID."""
    from plens_gb300 import build
    lib = build.LIB / "libplens_gpu.so"
    if not lib.exists():
        build.build_gpu()
    try:
        L = C.CDLL(str(lib))
    except OSError as e:
        pytest.skip(f"CUDA runtime not loadable here: {e}")
    L.plens_gpu_create.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    assert L.plens_gpu_create(None, None, None) == 1
