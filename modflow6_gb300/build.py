"""Builds the GB300 IMS library (libgbims.so) in-tree with nvcc for sm_103a.

Each CUDA translation unit is compiled in parallel; the shared library is
written next to this file so that the package loads it from the source tree.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "libgbims.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code without contraction of a*b+c, so that host-side setup arithmetic
# rounds as the oracle's C does on both x86-64 and aarch64
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "--expt-relaxed-constexpr"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the GB300 library cannot be built")
    return exe


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def extra_flags() -> list[str]:
    """Build-time tuning definitions from GBIMS_NVCC_EXTRA (for example
    "-DGB_DIA64_S=1"); a change of them rebuilds every object."""
    return os.environ.get("GBIMS_NVCC_EXTRA", "").split()


def _compile(src: Path, verbose: bool, stale: bool) -> Path:
    out = OBJ / (src.stem + ".o")
    deps = [src] + sorted(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "gbims.h"]
    if not stale and out.exists() and out.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return out
    cmd = [nvcc(), *ARCH, *FLAGS, *extra_flags(), "-c", str(src), "-o", str(out)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        print(r.stderr)
    return out


def build(verbose: bool = False) -> Path:
    """Compiles every .cu under csrc/ and links libgbims.so; returns its path."""
    OBJ.mkdir(exist_ok=True)
    srcs = sources()
    stamp = OBJ / "flags.txt"
    flags = " ".join(FLAGS + extra_flags())
    stale = not stamp.exists() or stamp.read_text() != flags
    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose, stale), srcs))
    stamp.write_text(flags)
    newest = max(o.stat().st_mtime for o in objs)
    if stale or not LIB.exists() or LIB.stat().st_mtime < newest:
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    import sys

    print(build(verbose="-v" in sys.argv))
