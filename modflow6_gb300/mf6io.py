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


# ---- cell-by-cell budget files -------------------------------------------
#
# A budget file (OC BUDGET FILEOUT) holds, for each saved time step, one
# record per flow term in the order the model saves them (gwf_ot_flow,
# src/Model/GroundWaterFlow/gwf.f90:911-931: STO-SS and STO-SY when the
# model has STO, FLOW-JA-FACE, then each boundary package in name-file
# order).  Every record starts with
#
#     kstp int32, kper int32, text 16 bytes (right-justified), ndim1 int32,
#     ndim2 int32, -ndim3 int32;  imeth int32, delt, pertim, totim float64
#
# and then, for imeth 1 (`ubdsv1`, src/Utilities/InputOutput.f90:945-974),
# ndim1*ndim2*ndim3 float64 values; for imeth 6 (`ubdsv06`, :981-1024, with
# `ubdsvd` per entry, :1051-1072) the four 16-byte names (model, package,
# destination model, destination package), naux+1 int32, naux 16-byte
# auxiliary names, nlist int32 and nlist entries (node int32, node2 int32,
# q float64, naux float64).  Arrays are written with the grid's shape
# (DIS: ncol, nrow, nlay; DISV: ncpl, 1, nlay; DISU: nodes, 1, 1), and
# FLOW-JA-FACE as (nja, 1, 1) (record_connection_array,
# src/Model/ModelUtilities/DiscretizationBase.f90:955-969).

BUDGET_HEADER = np.dtype([("kstp", "<i4"), ("kper", "<i4"), ("text", "S16"), ("ndim1", "<i4"),
                          ("ndim2", "<i4"), ("ndim3", "<i4"), ("imeth", "<i4"),
                          ("delt", "<f8"), ("pertim", "<f8"), ("totim", "<f8")])
assert BUDGET_HEADER.itemsize == 64


@dataclass
class BudgetRecord:
    kstp: int
    kper: int
    text: str
    ndim1: int
    ndim2: int
    ndim3: int
    imeth: int
    delt: float
    pertim: float
    totim: float
    data: np.ndarray | None = None          # imeth 1: ndim1*ndim2*ndim3 values
    names: tuple = ("", "", "", "")         # imeth 6: model, package, model2, package2
    auxnames: tuple = ()
    node: np.ndarray | None = None          # imeth 6: 1-based
    node2: np.ndarray | None = None
    q: np.ndarray | None = None
    aux: np.ndarray | None = None           # (nlist, naux)


def _s16(text: str, right: bool = True) -> bytes:
    if len(text) > 16:
        raise ValueError("a name is at most 16 characters")
    return (text.rjust(16) if right else text.ljust(16)).encode("ascii")


def write_budget(path, records: list[BudgetRecord], append: bool = False) -> None:
    """Writes the records as MODFLOW 6's budget file does."""
    with open(path, "ab" if append else "wb") as f:
        for r in records:
            h = np.zeros(1, BUDGET_HEADER)
            h["kstp"], h["kper"], h["text"] = r.kstp, r.kper, _s16(r.text)
            h["ndim1"], h["ndim2"], h["ndim3"] = r.ndim1, r.ndim2, -r.ndim3
            h["imeth"], h["delt"], h["pertim"], h["totim"] = r.imeth, r.delt, r.pertim, r.totim
            f.write(h.tobytes())
            if r.imeth == 1:
                d = np.ascontiguousarray(r.data, "<f8").ravel()
                if d.size != r.ndim1 * r.ndim2 * r.ndim3:
                    raise ValueError(f"{r.text}: {d.size} values for a "
                                     f"{r.ndim1}x{r.ndim2}x{r.ndim3} record")
                f.write(d.tobytes())
            elif r.imeth == 6:
                for nm in r.names:
                    f.write(_s16(nm, right=False))
                naux = len(r.auxnames)
                f.write(np.int32(naux + 1).tobytes())
                for a in r.auxnames:
                    f.write(_s16(a, right=False))
                nlist = 0 if r.q is None else len(r.q)
                f.write(np.int32(nlist).tobytes())
                ent = np.zeros(nlist, [("node", "<i4"), ("node2", "<i4"), ("q", "<f8")]
                               + [(f"a{k}", "<f8") for k in range(naux)])
                if nlist:
                    ent["node"], ent["node2"], ent["q"] = r.node, r.node2, r.q
                    for k in range(naux):
                        ent[f"a{k}"] = np.asarray(r.aux)[:, k]
                f.write(ent.tobytes())
            else:
                raise ValueError(f"imeth {r.imeth} is not written here")


def read_budget(src) -> list[BudgetRecord]:
    """All imeth 1 and imeth 6 records of a budget file (a path or bytes)."""
    buf = src if isinstance(src, (bytes, bytearray, memoryview)) else Path(src).read_bytes()
    buf = memoryview(buf)
    out: list[BudgetRecord] = []
    pos = 0
    while pos < len(buf):
        if len(buf) - pos < BUDGET_HEADER.itemsize:
            raise ValueError(f"truncated header at byte {pos}")
        h = np.frombuffer(buf, BUDGET_HEADER, count=1, offset=pos)[0]
        pos += BUDGET_HEADER.itemsize
        r = BudgetRecord(int(h["kstp"]), int(h["kper"]), h["text"].decode("ascii").strip(),
                         int(h["ndim1"]), int(h["ndim2"]), -int(h["ndim3"]), int(h["imeth"]),
                         float(h["delt"]), float(h["pertim"]), float(h["totim"]))
        if r.imeth == 1:
            nval = r.ndim1 * r.ndim2 * r.ndim3
            r.data = np.frombuffer(buf, "<f8", count=nval, offset=pos).copy()
            pos += 8 * nval
        elif r.imeth == 6:
            names = []
            for _ in range(4):
                names.append(bytes(buf[pos:pos + 16]).decode("ascii").strip())
                pos += 16
            r.names = tuple(names)
            naux = int(np.frombuffer(buf, "<i4", count=1, offset=pos)[0]) - 1
            pos += 4
            aux = []
            for _ in range(naux):
                aux.append(bytes(buf[pos:pos + 16]).decode("ascii").strip())
                pos += 16
            r.auxnames = tuple(aux)
            nlist = int(np.frombuffer(buf, "<i4", count=1, offset=pos)[0])
            pos += 4
            dt = np.dtype([("node", "<i4"), ("node2", "<i4"), ("q", "<f8")]
                          + [(f"a{k}", "<f8") for k in range(naux)])
            ent = np.frombuffer(buf, dt, count=nlist, offset=pos)
            pos += dt.itemsize * nlist
            r.node, r.node2, r.q = ent["node"].copy(), ent["node2"].copy(), ent["q"].copy()
            r.aux = np.stack([ent[f"a{k}"] for k in range(naux)], axis=1) if naux else None
        else:
            raise ValueError(f"imeth {r.imeth} at byte {pos} is not read here")
        out.append(r)
    return out


def gwf_budget_records(m, name: str, flowja, cells: dict, kstp: int = 1, kper: int = 1,
                       delt: float = 1.0, pertim: float = 1.0, totim: float = 1.0) -> list:
    """The records one time step of a GWF model saves (gwf_ot_flow order):
    STO-SS and STO-SY (sto_save_model_flows, gwf-sto.f90:615-640, STO-SY when
    a cell is convertible), FLOW-JA-FACE, then CHD, WEL and RCH as the input
    writer lists them, each entry (user node, list index, rate) as
    save_print_model_flows writes it (BoundaryPackage.f90:1753-1900).
    cells holds sto_ss, sto_sy (per cell) and chd, wel, rch (per entry)."""
    if getattr(m, "disu", False):
        shape = (m.nodes, 1, 1)
    elif getattr(m, "disv", False):
        shape = (m.ncpl, 1, m.nlay)
    else:
        shape = (m.ncol, m.nrow, m.nlay)
    name = name.upper()
    base = dict(kstp=kstp, kper=kper, delt=delt, pertim=pertim, totim=totim)
    recs = []
    if m.ss is not None and m.sy is not None:
        recs.append(BudgetRecord(text="STO-SS", ndim1=shape[0], ndim2=shape[1], ndim3=shape[2],
                                 imeth=1, data=np.asarray(cells["sto_ss"]), **base))
        if np.any(np.asarray(m.icelltype) != 0):
            recs.append(BudgetRecord(text="STO-SY", ndim1=shape[0], ndim2=shape[1],
                                     ndim3=shape[2], imeth=1, data=np.asarray(cells["sto_sy"]),
                                     **base))
    fj = np.asarray(flowja)
    recs.append(BudgetRecord(text="FLOW-JA-FACE", ndim1=fj.size, ndim2=1, ndim3=1, imeth=1,
                             data=fj, **base))
    nodeuser = getattr(m, "nodeuser", None)
    for key, nodes in (("chd", m.chd_node), ("wel", m.wel_node), ("rch", m.rch_node)):
        if not len(nodes):
            continue
        nu = np.asarray(nodes) if nodeuser is None else np.asarray(nodeuser)[nodes]
        recs.append(BudgetRecord(text=key.upper(), ndim1=shape[0], ndim2=shape[1],
                                 ndim3=shape[2], imeth=6,
                                 names=(name, name, name, key.upper()),
                                 node=nu + 1, node2=np.arange(1, len(nodes) + 1),
                                 q=np.asarray(cells[key]), **base))
    return recs
