"""The C-ABI library loads and exports every entry point include/gbims.h declares
(no compute calls: this runs without a GPU)."""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def header_symbols():
    text = (ROOT / "include" / "gbims.h").read_text()
    return sorted(set(re.findall(r"\b(gb(?:ims|npf|sln|mpnn)_[a-z_0-9]+)\s*\(", text)))


def test_header_symbols_bound_in_python():
    from modflow6_gb300 import _lib
    assert sorted(_lib.EXPORTED) == header_symbols()


def test_library_builds_and_exports():
    import shutil
    if shutil.which("nvcc") is None:
        pytest.skip("nvcc not available")
    from modflow6_gb300 import build
    lib = build.build()
    import ctypes
    so = ctypes.CDLL(str(lib))
    for name in header_symbols():
        assert hasattr(so, name), name
