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


def _build_c_driver(tmp_path):
    """Compiles tests/c_abi/drive_gbims.c with gcc against include/gbims.h
    and links it to libgbims.so: the C ABI as a C caller sees it."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None or shutil.which("nvcc") is None:
        pytest.skip("gcc or nvcc not available")
    from modflow6_gb300 import build
    lib = build.build()
    cuda = Path(shutil.which("nvcc")).resolve().parents[1]
    libdir = next((p for p in (cuda / "lib64", cuda / "lib", cuda / "targets" / "sbsa-linux" / "lib")
                   if (p / "libcudart.so").exists()), cuda / "lib64")
    exe = tmp_path / "drive_gbims"
    cmd = ["gcc", "-O2", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "c_abi" / "drive_gbims.c"), "-o", str(exe), "-L", str(lib.parent),
           "-lgbims", "-L", str(libdir), "-lcudart", "-lm", f"-Wl,-rpath,{lib.parent}",
           f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_c_caller_compiles_and_links(tmp_path):
    assert _build_c_driver(tmp_path).exists()


@pytest.mark.gpu
def test_c_caller_runs(gblib, tmp_path):
    """The C program's allocate / apply / records / destroy sequence, PCG and
    BiCGSTAB, on the GPU."""
    import subprocess
    exe = _build_c_driver(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0 and "drive_gbims ok" in r.stdout, r.stdout + r.stderr
