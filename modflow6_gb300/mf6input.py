"""MODFLOW 6 input files for a single GWF DIS model and its IMS solution.

`write_simulation` writes the files the `mf6` program reads for the models
this library solves (GwfDisModel: DIS, IC, NPF, STO, CHD, WEL, RCH, with the
IMS and TDIS settings), so the same model can be run by the reference program
on any machine that has it, and its binary head file compared with ours
(modflow6_gb300.mf6io).  The blocks and keywords follow the input definition
files of the reference (doc/mf6io/mf6ivar/dfn/*.dfn); arrays are written
INTERNAL with full precision (repr of each float), node order layer, row,
column; cell ids are 1-based (layer, row, column).

`read_blocks` parses the block structure back (BEGIN name ... END name) for
the round-trip tests.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from .dis import GwfDisModel

_RCLOSE_OPTION = {0: "", 1: " STRICT", 2: " L2NORM_RCLOSE", 3: " RELATIVE_RCLOSE",
                  4: " L2NORM_RELATIVE_RCLOSE"}
_UNDER_RELAXATION = {0: "NONE", 1: "SIMPLE", 2: "COOLEY", 3: "DBD"}
_SCALING = {0: "NONE", 1: "DIAGONAL", 2: "L2NORM"}
_REORDERING = {0: "NONE", 1: "RCM", 2: "MD"}
_CELL_AVERAGING = {1: "LOGARITHMIC", 2: "AMT-LMK", 3: "AMT-HMK"}


def _fmt(v) -> str:
    return repr(float(v))


def _array(name: str, values, layered_shape=None, ints=False, per_line=10) -> list[str]:
    """An INTERNAL array, either whole or, with layered_shape (nlay, ncpl),
    one INTERNAL block per layer."""
    v = np.asarray(values).ravel()
    f = (lambda x: str(int(x))) if ints else _fmt
    out = []

    def body(a):
        for i in range(0, a.size, per_line):
            out.append("      " + " ".join(f(x) for x in a[i:i + per_line]))

    if layered_shape is None:
        out.append(f"  {name}")
        out.append("    INTERNAL FACTOR 1" + ("" if ints else ".0"))
        body(v)
    else:
        nlay, ncpl = layered_shape
        out.append(f"  {name} LAYERED")
        for k in range(nlay):
            out.append("    INTERNAL FACTOR 1" + ("" if ints else ".0"))
            body(v[k * ncpl:(k + 1) * ncpl])
    return out


def _block(name: str, lines: list[str], suffix: str = "") -> list[str]:
    head = f"BEGIN {name}{(' ' + suffix) if suffix else ''}"
    return [head] + lines + [f"END {name}", ""]


def _cellid(m: GwfDisModel, node: int) -> str:
    nrc = m.nrow * m.ncol
    k, rem = divmod(int(node), nrc)
    i, j = divmod(rem, m.ncol)
    return f"{k + 1} {i + 1} {j + 1}"


def write_simulation(ws, m: GwfDisModel, ims, nl, periods=((1.0, 1, 1.0, True),),
                     name: str = "gwf", ptc: bool = True) -> dict:
    """Writes mfsim.nam, the TDIS, IMS and GWF name files and the package
    files into directory `ws`; returns {package: path}.

    ims: an ImsLinearSettings (LINEAR block); nl: a solution.Nonlinear
    (NONLINEAR block); periods: (perlen, nstp, tsmult, steady) per stress
    period, with the stresses of the model applied in period 1 and kept;
    ptc False writes NO_PTC ALL."""
    ws = Path(ws)
    ws.mkdir(parents=True, exist_ok=True)
    files = {}

    def write(key, fname, lines):
        p = ws / fname
        p.write_text("\n".join(lines) + "\n")
        files[key] = p

    nper = len(periods)
    write("sim", "mfsim.nam",
          _block("options", [])
          + _block("timing", [f"  TDIS6 {name}.tdis"])
          + _block("models", [f"  gwf6 {name}.nam {name}"])
          + _block("exchanges", [])
          + _block("solutiongroup", [f"  ims6 {name}.ims {name}"], "1"))
    write("tdis", f"{name}.tdis",
          _block("options", ["  TIME_UNITS days"])
          + _block("dimensions", [f"  NPER {nper}"])
          + _block("perioddata", [f"  {_fmt(p[0])} {int(p[1])} {_fmt(p[2])}" for p in periods]))
    opts = []
    if not ptc or getattr(nl, "iallowptc", 1) == 0:
        opts.append("  NO_PTC ALL")
    nonlin = [f"  OUTER_DVCLOSE {_fmt(nl.dvclose)}", f"  OUTER_MAXIMUM {int(nl.mxiter)}",
              f"  UNDER_RELAXATION {_UNDER_RELAXATION[int(nl.nonmeth)]}"]
    if nl.nonmeth > 0:
        nonlin += [f"  UNDER_RELAXATION_THETA {_fmt(nl.theta)}",
                   f"  UNDER_RELAXATION_KAPPA {_fmt(nl.akappa)}",
                   f"  UNDER_RELAXATION_GAMMA {_fmt(nl.gamma)}",
                   f"  UNDER_RELAXATION_MOMENTUM {_fmt(nl.amomentum)}"]
    if nl.numtrack > 0:
        nonlin += [f"  BACKTRACKING_NUMBER {int(nl.numtrack)}",
                   f"  BACKTRACKING_TOLERANCE {_fmt(nl.btol)}",
                   f"  BACKTRACKING_REDUCTION_FACTOR {_fmt(nl.breduc)}",
                   f"  BACKTRACKING_RESIDUAL_LIMIT {_fmt(nl.res_lim)}"]
    lin = [f"  INNER_MAXIMUM {int(ims.iter1)}", f"  INNER_DVCLOSE {_fmt(ims.dvclose)}",
           f"  INNER_RCLOSE {_fmt(ims.rclose)}{_RCLOSE_OPTION[int(ims.icnvgopt)]}",
           f"  LINEAR_ACCELERATION {'CG' if ims.ilinmeth == 1 else 'BICGSTAB'}",
           f"  RELAXATION_FACTOR {_fmt(ims.relax)}",
           f"  PRECONDITIONER_LEVELS {int(ims.level)}",
           f"  PRECONDITIONER_DROP_TOLERANCE {_fmt(ims.droptol)}",
           f"  NUMBER_ORTHOGONALIZATIONS {int(ims.north)}",
           f"  SCALING_METHOD {_SCALING[int(ims.iscl)]}",
           f"  REORDERING_METHOD {_REORDERING[int(ims.iord)]}"]
    write("ims", f"{name}.ims", _block("options", opts) + _block("nonlinear", nonlin)
          + _block("linear", lin))
    # GWF name file
    gopts = []
    if m.inewton:
        gopts.append("  NEWTON" + (" UNDER_RELAXATION" if m.inewtonur else ""))
    transient = m.ss is not None and m.sy is not None
    pk = [f"  DIS6 {name}.dis dis", f"  IC6 {name}.ic ic", f"  NPF6 {name}.npf npf"]
    if transient:
        pk.append(f"  STO6 {name}.sto sto")
    if m.chd_node.size:
        pk.append(f"  CHD6 {name}.chd chd")
    if m.wel_node.size:
        pk.append(f"  WEL6 {name}.wel wel")
    if m.rch_node.size:
        pk.append(f"  RCH6 {name}.rch rch")
    pk.append(f"  OC6 {name}.oc oc")
    write("nam", f"{name}.nam", _block("options", gopts) + _block("packages", pk))
    nrc = m.nrow * m.ncol
    write("dis", f"{name}.dis",
          _block("options", ["  LENGTH_UNITS meters"])
          + _block("dimensions", [f"  NLAY {m.nlay}", f"  NROW {m.nrow}", f"  NCOL {m.ncol}"])
          + _block("griddata", _array("DELR", m.delr) + _array("DELC", m.delc)
                   + _array("TOP", m.top) + _array("BOTM", m.botm, (m.nlay, nrc))))
    write("ic", f"{name}.ic", _block("options", [])
          + _block("griddata", _array("STRT", m.strt, (m.nlay, nrc))))
    nopts = ["  SAVE_FLOWS"]
    if m.icellavg:
        nopts.append(f"  ALTERNATIVE_CELL_AVERAGING {_CELL_AVERAGING[int(m.icellavg)]}")
    if m.ivarcv:
        nopts.append("  VARIABLECV" + (" DEWATERED" if m.idewatcv else ""))
    write("npf", f"{name}.npf", _block("options", nopts)
          + _block("griddata", _array("ICELLTYPE", m.icelltype, (m.nlay, nrc), ints=True)
                   + _array("K", m.k11, (m.nlay, nrc)) + _array("K33", m.k33, (m.nlay, nrc))))
    if transient:
        sper = []
        for ip, p in enumerate(periods, start=1):
            sper += _block("period", ["  STEADY-STATE" if p[3] else "  TRANSIENT"], str(ip))
        write("sto", f"{name}.sto", _block("options", ["  SAVE_FLOWS"])
              + _block("griddata", _array("ICONVERT", m.icelltype, (m.nlay, nrc), ints=True)
                       + _array("SS", m.ss, (m.nlay, nrc)) + _array("SY", m.sy, (m.nlay, nrc)))
              + sper)

    def listpkg(key, nodes, vals):
        lines = [f"  {_cellid(m, n)} {_fmt(v)}" for n, v in zip(nodes, vals)]
        write(key, f"{name}.{key}", _block("options", ["  SAVE_FLOWS"])
              + _block("dimensions", [f"  MAXBOUND {len(lines)}"]) + _block("period", lines, "1"))

    if m.chd_node.size:
        listpkg("chd", m.chd_node, m.chd_head)
    if m.wel_node.size:
        listpkg("wel", m.wel_node, m.wel_q)
    if m.rch_node.size:
        listpkg("rch", m.rch_node, m.rch_rate)
    write("oc", f"{name}.oc",
          _block("options", [f"  BUDGET FILEOUT {name}.cbc", f"  HEAD FILEOUT {name}.hds"])
          + _block("period", ["  SAVE HEAD ALL", "  SAVE BUDGET ALL"], "1"))
    return files


def read_blocks(path) -> list[tuple[str, str, list[str]]]:
    """(block name, suffix, lines) of every BEGIN ... END block of a MODFLOW 6
    input file, in file order; comments (#, !) and blank lines dropped."""
    out = []
    cur = None
    for raw in Path(path).read_text().splitlines():
        line = raw.split("#")[0].split("!")[0].strip()
        if not line:
            continue
        w = line.split()
        if w[0].upper() == "BEGIN":
            cur = (w[1].lower(), " ".join(w[2:]), [])
        elif w[0].upper() == "END":
            if cur is None or w[1].lower() != cur[0]:
                raise ValueError(f"unbalanced END {w[1]} in {path}")
            out.append(cur)
            cur = None
        elif cur is not None:
            cur[2].append(line)
    if cur is not None:
        raise ValueError(f"block {cur[0]} not closed in {path}")
    return out


def read_array(lines: list[str], name: str) -> np.ndarray:
    """The values of array `name` (INTERNAL, whole or LAYERED) from a griddata
    block's lines."""
    vals, on = [], False
    for line in lines:
        w = line.split()
        if w[0].upper() in ("INTERNAL", "CONSTANT", "OPEN/CLOSE"):
            if on and w[0].upper() != "INTERNAL":
                raise ValueError("only INTERNAL arrays are read")
            continue
        try:
            float(w[0])
        except ValueError:  # an array name opens the next array
            on = w[0].upper() == name.upper()
            continue
        if on:
            vals += [float(x) for x in w]
    return np.array(vals)
