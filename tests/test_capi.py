"""The C-ABI library: builds for sm_103a, loads, and exports every symbol that
include/bem_gb300.h declares (no GPU needed: no compute calls)."""
import ctypes
import os
import pathlib
import re

from mesh2hrtf_gb300 import build, capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = pathlib.Path(os.path.join(ROOT, "include", "bem_gb300.h")).read_text()
    return sorted(set(re.findall(r"\b(bem_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_the_binding():
    assert sorted(capi.EXPORTED) == _declared()


def test_library_exports_every_declared_symbol():
    build.build_library()
    lib = ctypes.CDLL(build.LIB)
    for name in _declared():
        assert hasattr(lib, name), name


def test_footprint_without_device():
    lib = capi.load()
    n = 20480
    fp = lib.bem_footprint_bytes(n, capi.PREC_MIXED, 60)
    assert fp > n * n * 8
    assert lib.bem_footprint_bytes(n, capi.PREC_FP64, 60) > 1.9 * n * n * 8
    assert lib.bem_version().decode().startswith("mesh2hrtf_gb300")
