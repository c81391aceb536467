"""MODFLOW 6 binary output files: heads (and other dependent variables).

MODFLOW 6 opens its binary output with ACCESS='STREAM', FORM='UNFORMATTED'
(src/Utilities/OpenSpec.f90:17-25), so a file is a plain byte stream with no
Fortran record markers, in the writing machine's byte order (little-endian on
every platform MODFLOW 6 is built for).

A dependent-variable file (HEAD) holds, for each saved time step, one record
per layer of a DIS grid (DisType%record_array, src/Model/Discretization/
Dis.f90:1401-1486), each written by `ulasav` (src/Utilities/InputOutput.f90:
924-940):

    kstp  int32, kper int32, pertim float64, totim float64,
    text  16 bytes (space-padded, e.g. "HEAD            "),
    ncol  int32, nrow int32, ilay int32          -- 52 bytes in all
    ncol*nrow float64 values, column index fastest

`read_dependent_variable` and `write_dependent_variable` read and write that
layout for full DIS grids, so heads computed on the GPU can be compared with
a file MODFLOW 6 wrote, and a file written here can be read by the tools that
read MODFLOW 6's.
"""
from __future__ import annotations

from dataclasses import dataclass
from pathlib import Path

import numpy as np

HEADER = np.dtype([("kstp", "<i4"), ("kper", "<i4"), ("pertim", "<f8"), ("totim", "<f8"),
                   ("text", "S16"), ("ncol", "<i4"), ("nrow", "<i4"), ("ilay", "<i4")])
assert HEADER.itemsize == 52


@dataclass
class LayerRecord:
    kstp: int
    kper: int
    pertim: float
    totim: float
    text: str
    ncol: int
    nrow: int
    ilay: int
    data: np.ndarray  # (nrow, ncol) float64


def read_dependent_variable(src) -> list[LayerRecord]:
    """All `ulasav` records of a binary dependent-variable file (a path or the
    file's bytes), in file order."""
    buf = src if isinstance(src, (bytes, bytearray, memoryview)) else Path(src).read_bytes()
    buf = memoryview(buf)
    out: list[LayerRecord] = []
    pos = 0
    while pos < len(buf):
        if len(buf) - pos < HEADER.itemsize:
            raise ValueError(f"truncated header at byte {pos}")
        h = np.frombuffer(buf, HEADER, count=1, offset=pos)[0]
        ncol, nrow = int(h["ncol"]), int(h["nrow"])
        if ncol <= 0 or nrow <= 0:
            raise ValueError(f"bad record shape {nrow}x{ncol} at byte {pos}")
        pos += HEADER.itemsize
        nval = ncol * nrow
        if len(buf) - pos < 8 * nval:
            raise ValueError(f"truncated data at byte {pos}")
        data = np.frombuffer(buf, "<f8", count=nval, offset=pos).reshape(nrow, ncol).copy()
        pos += 8 * nval
        out.append(LayerRecord(int(h["kstp"]), int(h["kper"]), float(h["pertim"]),
                               float(h["totim"]), h["text"].decode("ascii").strip(), ncol, nrow,
                               int(h["ilay"]), data))
    return out


def read_heads(src, text: str = "HEAD") -> dict[tuple[int, int], np.ndarray]:
    """{(kper, kstp): heads (nlay, nrow, ncol)} from a binary head file; the
    layers of one time step are stacked in `ilay` order."""
    steps: dict[tuple[int, int], dict[int, np.ndarray]] = {}
    for r in read_dependent_variable(src):
        if r.text != text:
            continue
        steps.setdefault((r.kper, r.kstp), {})[r.ilay] = r.data
    return {k: np.stack([v[i] for i in sorted(v)]) for k, v in steps.items()}


def write_dependent_variable(path, values: np.ndarray, nlay: int, nrow: int, ncol: int,
                             kstp: int = 1, kper: int = 1, pertim: float = 1.0,
                             totim: float = 1.0, text: str = "HEAD", append: bool = False) -> None:
    """Writes one time step of a full DIS grid (node order layer, row, column)
    as `nlay` `ulasav` records."""
    v = np.ascontiguousarray(values, dtype="<f8").reshape(nlay, nrow * ncol)
    if len(text) > 16:
        raise ValueError("text is at most 16 characters")
    with open(path, "ab" if append else "wb") as f:
        for k in range(nlay):
            h = np.zeros(1, HEADER)
            h["kstp"], h["kper"], h["pertim"], h["totim"] = kstp, kper, pertim, totim
            h["text"] = text.ljust(16).encode("ascii")
            h["ncol"], h["nrow"], h["ilay"] = ncol, nrow, k + 1
            f.write(h.tobytes())
            f.write(v[k].tobytes())
