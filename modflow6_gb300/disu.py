"""DISU (unstructured) grids: cells and connections given by the user.

`disu_connections` turns the DISU input arrays into the connectivity the
solution uses, as MODFLOW 6 does:

* Disu.f90:325-425 (disu_ck): each row's first JA entry is the cell itself
  (it may be given negative), the other entries name valid cells, IDOMAIN is
  0 or 1, active cells have positive thickness and area, and a cell below
  (ihc 0, higher number) has its top no more than VERTICAL_OFFSET_TOLERANCE
  above the bottom of the cell above;
* Disu.f90:218-266: the reduced numbering of the cells with IDOMAIN 1
  (nodereduced, nodeuser);
* Connections.f90:801-928 (disuconnections): for a reduced grid the rows of
  the kept cells, each with its diagonal first and the kept neighbours
  ascending (Sparse.f90:217-239), and the per-entry arrays compressed in
  input order;
* Connections.f90:160-316 (con_finalize) and :1205-1268 (fillisym,
  filljas): the checks (diagonal first, ascending rows, every connection
  with its counterpart, IHC and HWVA symmetric, IHC in 0..2), then IHC,
  CL12 and HWVA moved into one value per connection n < m: CL1 from the
  entry in row n, CL2 from the entry in row m.

All numbers here are 0-based; JA in the input is 1-based as in the DISU
file (IAC, JA, IHC, CL12, HWVA, ANGLDEGX blocks).  ANGLDEGX is not read:
the horizontal anisotropy it serves (K22, XT3D) is not part of this build.
The evaluation is vectorised over entries and equals the oracle's loops
(or_disu_connect) array for array.  `DisuModel` carries a GWF model on such
a grid with the attributes the NPF fill and the oracle read.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


class DisuError(ValueError):
    """The DISU input fails one of the reference's checks; `messages` lists
    every failure found (the reference stores them all before stopping)."""

    def __init__(self, messages: list[str]):
        super().__init__("; ".join(messages))
        self.messages = messages


def iac_to_ia(iac) -> np.ndarray:
    """IA (0-based offsets, nodes + 1) from IAC, the number of entries of each
    row including the diagonal."""
    iac = np.asarray(iac, np.int64)
    ia = np.zeros(iac.size + 1, np.int64)
    np.cumsum(iac, out=ia[1:])
    return ia


def disu_check(top, bot, area, iac, ja, ihc, idomain=None, voffsettol: float = 0.0) -> np.ndarray:
    """disu_ck (Disu.f90:325-425).  Returns JA (1-based) with a negative
    diagonal entry made positive; raises DisuError listing every failure."""
    top, bot, area = (np.asarray(a, float) for a in (top, bot, area))
    ia = iac_to_ia(iac)
    ja = np.array(ja, np.int64)
    ihc = np.asarray(ihc, np.int64)
    n = ia.size - 1
    idomain = np.ones(n, np.int64) if idomain is None else np.asarray(idomain, np.int64)
    errs = []
    rows = np.arange(n)
    d = ia[:-1]
    ja[d] = np.abs(ja[d])
    for r in np.flatnonzero(ja[d] != rows + 1):
        errs.append(f"Cell {r + 1} must have its first connection be itself.  Found: {ja[d[r]]}")
    off = np.ones(ja.size, bool)
    off[d] = False
    rown = np.repeat(rows, np.diff(ia))
    bad = off & ((ja < 0) | (ja > n))
    for p in np.flatnonzero(bad):
        errs.append(f"Cell {rown[p] + 1} has invalid connection in JA.  Found: {ja[p]}")
    if errs:
        raise DisuError(errs)
    for r in np.flatnonzero((idomain > 1) | (idomain < 0)):
        errs.append(f"Invalid idomain value {idomain[r]} specified for node {r + 1}")
    act = idomain == 1
    for r in np.flatnonzero(act & (top - bot <= 0.0)):
        errs.append(f"CELL ({r + 1}) THICKNESS <= 0. TOP, BOT: {top[r]} {bot[r]}")
    for r in np.flatnonzero(act & (area <= 0.0)):
        errs.append(f"Cell {r + 1} with area <= 0. Area: {area[r]}")
    if voffsettol < 0.0:
        errs.append(f"Vertical offset tolerance must be greater than zero. Found {voffsettol}")
    m = np.where(off, ja - 1, 0)
    below = off & (ihc == 0) & (m > rown)
    for p in np.flatnonzero(below & (top[m] - bot[rown] > voffsettol)):
        errs.append(f"Top elevation ({top[m[p]]}) for cell {m[p] + 1} is above bottom elevation "
                    f"({bot[rown[p]]}) for cell {rown[p] + 1}.")
    if errs:
        raise DisuError(errs)
    return ja


def _finalize(n, ia, ja, ihct, cl12t, hwvat, angt=None) -> dict:
    """con_finalize (Connections.f90:160-316) on 0-based ia/ja (nja) and the
    per-entry arrays in the same order."""
    nja = ja.size
    rown = np.repeat(np.arange(n), np.diff(ia))
    errs = []
    d = ia[:-1]
    for r in np.flatnonzero(ja[d] != np.arange(n)):
        errs.append(f"JA: First value for cell : {r + 1} must equal {r + 1}. Found {ja[d[r]] + 1} instead.")
    nxt = np.arange(nja - 1)
    unsorted = (rown[nxt] == rown[nxt + 1]) & (nxt > d[rown[nxt]]) & (ja[nxt] > ja[nxt + 1])
    for p in np.flatnonzero(unsorted):
        errs.append(f"JA: Entries not sorted for row: {rown[p] + 1}. Offending entries are: "
                    f"{ja[p] + 1} and {ja[p + 1] + 1}")
    if errs:
        raise DisuError(errs)
    # fillisym: the first position of (m, n) in row m
    key = rown * n + ja
    order = np.argsort(key, kind="stable")
    sk = key[order]
    want = ja * n + rown
    at = np.searchsorted(sk, want)
    found = (at < nja) & (sk[np.minimum(at, nja - 1)] == want)
    isym = np.where(found, order[np.minimum(at, nja - 1)], -1)
    self_ = ja == rown
    isym[self_] = np.flatnonzero(self_)
    for p in np.flatnonzero(isym < 0):
        errs.append(f"JA: Array does not have symmetric counterpart in position {p + 1} "
                    f"for cell {rown[p] + 1} connected to cell {ja[p] + 1}")
    if errs:
        raise DisuError(errs)
    # filljas
    upper = ja > rown
    lower = ja < rown
    njas = int(upper.sum())
    jas = np.full(nja, -1, np.int64)
    jas[upper] = np.arange(njas)
    jas[lower] = jas[isym[lower]]
    off = upper | lower
    for p in np.flatnonzero(off & (ihct != ihct[isym])):
        errs.append(f"IHC: Array is not symmetric in positions: {p + 1} and {isym[p] + 1}")
    for p in np.flatnonzero(off & (hwvat != hwvat[isym])):
        errs.append(f"HWVA: Array is not symmetric in positions: {p + 1} and {isym[p] + 1}")
    for p in np.flatnonzero(off & ((ihct < 0) | (ihct > 2))):
        errs.append(f"IHC must be 0, 1, or 2.  Found: {ihct[p]}")
    if errs:
        raise DisuError(errs)
    ihc = np.zeros(njas, np.int64)
    cl1, cl2, hwva = np.zeros(njas), np.zeros(njas), np.zeros(njas)
    ihc[jas[off]] = ihct[off]
    cl1[jas[upper]] = cl12t[upper]
    cl2[jas[lower]] = cl12t[lower]
    hwva[jas[off]] = hwvat[off]
    # anglex: the upper triangle's ANGLDEGX in radians (:300-312)
    anglex = np.zeros(njas)
    if angt is not None:
        anglex[jas[upper]] = angt[upper] * (math.atan(1.0) / 45.0)
    return dict(nodes=n, nja=nja, njas=njas, ia=ia.astype(np.int32), ja=ja.astype(np.int32),
                isym=isym.astype(np.int32), jas=jas.astype(np.int32), ihc=ihc.astype(np.int32),
                cl1=cl1, cl2=cl2, hwva=hwva, anglex=anglex)


def disu_connections(iac, ja, ihc, cl12, hwva, idomain=None, angldegx=None) -> dict:
    """The connectivity of a DISU grid from its input arrays (JA 1-based; a
    negative diagonal entry allowed), reduced to the cells with IDOMAIN 1,
    with anglex (radians, per connection n < m) from ANGLDEGX when given.
    The result also holds `nodeuser` (reduced -> user, 0-based) and
    `nodereduced` (user -> reduced, -1 for a removed cell)."""
    ia_u = iac_to_ia(iac)
    ja_u = np.abs(np.asarray(ja, np.int64)) - 1
    ihc_u = np.asarray(ihc, np.int64)
    cl12_u = np.asarray(cl12, float)
    hwva_u = np.asarray(hwva, float)
    ang_u = None if angldegx is None else np.asarray(angldegx, float)
    nu = ia_u.size - 1
    idomain = np.ones(nu, np.int64) if idomain is None else np.asarray(idomain, np.int64)
    keep = idomain > 0
    n = int(keep.sum())
    if n == 0:
        raise DisuError(["Model does not have any active nodes. Ensure IDOMAIN array has some "
                         "values greater than zero."])
    nodereduced = np.full(nu, -1, np.int64)
    nodereduced[keep] = np.arange(n)
    nodeuser = np.flatnonzero(keep)
    if n == nu:
        out = _finalize(n, ia_u, ja_u, ihc_u, cl12_u, hwva_u, ang_u)
    else:
        row_u = np.repeat(np.arange(nu), np.diff(ia_u))
        sel = keep[row_u] & keep[ja_u]
        rr, cc = nodereduced[row_u[sel]], nodereduced[ja_u[sel]]
        # sparse%addconnection per row (no duplicates), then sort: the
        # diagonal first, the rest ascending
        k = np.unique(rr * n + cc)
        r2, c2 = k // n, k % n
        srt = np.lexsort((c2, c2 != r2, r2))
        r2, c2 = r2[srt], c2[srt]
        if r2.size != rr.size:
            raise DisuError(["JA: a row names the same cell twice"])
        ia = np.zeros(n + 1, np.int64)
        np.cumsum(np.bincount(r2, minlength=n), out=ia[1:])
        out = _finalize(n, ia, c2, ihc_u[sel], cl12_u[sel], hwva_u[sel],
                        None if ang_u is None else ang_u[sel])
    out.update(nodeuser=nodeuser.astype(np.int32), nodereduced=nodereduced.astype(np.int32))
    return out


def dis_as_disu(nlay: int, nrow: int, ncol: int, delr, delc, top, botm):
    """The DISU input arrays (IAC, JA 1-based, IHC, CL12, HWVA, TOP, BOT,
    AREA, all per user cell or entry) of a full DIS grid, with the DIS node
    numbering and the DIS geometry (Connections.f90:463-698): a DISU written
    this way must give the DIS connectivity."""
    delr, delc = np.asarray(delr, float), np.asarray(delc, float)
    nrc = nrow * ncol
    n = nlay * nrc
    cell_top = np.concatenate([np.asarray(top, float).ravel(), np.asarray(botm, float).ravel()[:-nrc]])
    cell_bot = np.asarray(botm, float).ravel().copy()
    iac, ja, ihc, cl12, hwva = [], [], [], [], []
    for k in range(nlay):
        for i in range(nrow):
            for j in range(ncol):
                p = j + i * ncol + k * nrc
                ent = [(p, 1, 0.0, 0.0)]
                if k > 0:
                    ent.append((p - nrc, 0, 0.5 * (cell_top[p] - cell_bot[p]), delr[j] * delc[i]))
                if i > 0:
                    ent.append((p - ncol, 1, 0.5 * delc[i], delr[j]))
                if j > 0:
                    ent.append((p - 1, 1, 0.5 * delr[j], delc[i]))
                if j < ncol - 1:
                    ent.append((p + 1, 1, 0.5 * delr[j], delc[i]))
                if i < nrow - 1:
                    ent.append((p + ncol, 1, 0.5 * delc[i], delr[j]))
                if k < nlay - 1:
                    ent.append((p + nrc, 0, 0.5 * (cell_top[p] - cell_bot[p]), delr[j] * delc[i]))
                iac.append(len(ent))
                for m, h, c, w in ent:
                    ja.append(m + 1)
                    ihc.append(h)
                    cl12.append(c)
                    hwva.append(w)
    area = np.tile(np.outer(delc, delr).ravel(), nlay)
    return dict(iac=np.array(iac), ja=np.array(ja), ihc=np.array(ihc), cl12=np.array(cl12),
                hwva=np.array(hwva), top=cell_top, bot=cell_bot, area=area)


def refined_grid(nlay: int, nrow: int, ncol: int, size: float, box: tuple, thick: float = 10.0,
                 stagger: float = 0.0, seed: int = 0):
    """A seeded quadtree-style DISU grid: nrow x ncol square cells of side
    `size` in every layer, those inside box = (i0, i1, j0, j1) (half-open)
    split into 2 x 2 cells of side size/2.  Cells are numbered layer by
    layer, row by row of the coarse grid, a split cell's four children in
    place (upper row first).  A coarse cell beside the box connects to the
    two fine cells along the shared face (width size/2, CL12 size/2 from the
    coarse cell and size/4 from the fine one).  With stagger > 0 the layer
    elevations vary from column to column by up to `stagger`, and horizontal
    connections between cells whose vertical ranges differ get IHC 2.
    Returns the DISU input dict (as dis_as_disu) plus the cell centres."""
    rng = np.random.default_rng(seed)
    i0, i1, j0, j1 = box
    fine = np.zeros((nrow, ncol), bool)
    fine[i0:i1, j0:j1] = True
    # sub-cells of one layer: (i, j, a, b) with a, b in {0, 1} for split
    # cells and (0, 0) for a coarse cell
    cells = []
    for i in range(nrow):
        for j in range(ncol):
            if fine[i, j]:
                cells += [(i, j, a, b) for a in (0, 1) for b in (0, 1)]
            else:
                cells.append((i, j, 0, 0))
    ncpl = len(cells)
    idx = {c: q for q, c in enumerate(cells)}
    # cell centre, extent and elevation per layer cell
    xc = np.array([(j + (0.25 + 0.5 * b if fine[i, j] else 0.5)) * size for i, j, a, b in cells])
    yc = np.array([(nrow - i - (0.25 + 0.5 * a if fine[i, j] else 0.5)) * size for i, j, a, b in cells])
    half = np.array([0.25 * size if fine[i, j] else 0.5 * size for i, j, a, b in cells])
    shift = rng.uniform(0.0, stagger, (nlay + 1, ncol)) if stagger > 0 else np.zeros((nlay + 1, ncol))
    top = np.empty(nlay * ncpl)
    bot = np.empty(nlay * ncpl)
    for k in range(nlay):
        for q, (i, j, a, b) in enumerate(cells):
            top[q + k * ncpl] = thick * (nlay - k) - shift[k, j] * (k > 0)
            bot[q + k * ncpl] = thick * (nlay - k - 1) - shift[k + 1, j] * (k + 1 < nlay)

    # ANGLDEGX of a face by its direction (rows grow southward): east 0,
    # north 90, west 180, south 270 degrees
    face_angle = {(0, 1): 0.0, (-1, 0): 90.0, (0, -1): 180.0, (1, 0): 270.0}

    def horiz(q):
        """(neighbour, width, face angle) over the four faces of layer cell q"""
        i, j, a, b = cells[q]
        out = []
        if fine[i, j]:
            # within the parent, then across the parent's faces
            for da, db in ((-1, 0), (1, 0), (0, -1), (0, 1)):
                ang = face_angle[(da, db)]
                na, nb = a + da, b + db
                if 0 <= na <= 1 and 0 <= nb <= 1:
                    out.append((idx[(i, j, na, nb)], 0.5 * size, ang))
                    continue
                ii, jj = i + (na > 1) - (na < 0), j + (nb > 1) - (nb < 0)
                if not (0 <= ii < nrow and 0 <= jj < ncol):
                    continue
                if fine[ii, jj]:
                    out.append((idx[(ii, jj, na % 2, nb % 2)], 0.5 * size, ang))
                else:
                    out.append((idx[(ii, jj, 0, 0)], 0.5 * size, ang))
        else:
            for di, dj in ((-1, 0), (1, 0), (0, -1), (0, 1)):
                ang = face_angle[(di, dj)]
                ii, jj = i + di, j + dj
                if not (0 <= ii < nrow and 0 <= jj < ncol):
                    continue
                if fine[ii, jj]:
                    # the two children along the shared face
                    if di:
                        a2 = 1 if di < 0 else 0
                        out += [(idx[(ii, jj, a2, b2)], 0.5 * size, ang) for b2 in (0, 1)]
                    else:
                        b2 = 1 if dj < 0 else 0
                        out += [(idx[(ii, jj, a2, b2)], 0.5 * size, ang) for a2 in (0, 1)]
                else:
                    out.append((idx[(ii, jj, 0, 0)], size, ang))
        return out

    iac, ja, ihc, cl12, hwva, angx = [], [], [], [], [], []
    for k in range(nlay):
        for q in range(ncpl):
            p = q + k * ncpl
            ent = [(p, 1, 0.0, 0.0, 0.0)]
            area_q = (2 * half[q]) ** 2
            if k > 0:
                ent.append((p - ncpl, 0, 0.5 * (top[p] - bot[p]), area_q, 0.0))
            if k < nlay - 1:
                ent.append((p + ncpl, 0, 0.5 * (top[p] - bot[p]), area_q, 0.0))
            for q2, w, ang in horiz(q):
                p2 = q2 + k * ncpl
                stag = top[p] != top[p2] or bot[p] != bot[p2]
                ent.append((p2, 2 if stag else 1, half[q], w, ang))
            ent = [ent[0]] + sorted(ent[1:])
            iac.append(len(ent))
            for m, h, c, w, ang in ent:
                ja.append(m + 1)
                ihc.append(h)
                cl12.append(c)
                hwva.append(w)
                angx.append(ang)
    area = np.tile((2 * half) ** 2, nlay)
    return dict(iac=np.array(iac), ja=np.array(ja), ihc=np.array(ihc), cl12=np.array(cl12),
                hwva=np.array(hwva), angldegx=np.array(angx), top=top, bot=bot, area=area,
                xc=np.tile(xc, nlay), yc=np.tile(yc, nlay), ncpl=ncpl)


@dataclass
class DisuModel:
    """A GWF model on a DISU grid (NPF, IC, STO, CHD, WEL, RCH).  Cell arrays
    (k11, k33, icelltype, strt, ss, sy) and boundary node numbers are in the
    reduced numbering; top, bot, area, idomain and the connection arrays are
    per user cell and entry, as in the DISU file.  nlay and nrow are 1 and
    ncol is the number of cells, so the per-column rules written for DIS
    read the same cells."""

    top_u: np.ndarray
    bot_u: np.ndarray
    area_u: np.ndarray
    iac: np.ndarray
    ja: np.ndarray              # 1-based, as in the file
    ihc_u: np.ndarray
    cl12: np.ndarray
    hwva_u: np.ndarray
    k11: np.ndarray
    k33: np.ndarray
    icelltype: np.ndarray
    strt: np.ndarray
    idomain: np.ndarray | None = None
    voffsettol: float = 0.0
    ss: np.ndarray | None = None
    sy: np.ndarray | None = None
    chd_node: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    chd_head: np.ndarray = field(default_factory=lambda: np.zeros(0))
    wel_node: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    wel_q: np.ndarray = field(default_factory=lambda: np.zeros(0))
    rch_node: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    rch_rate: np.ndarray = field(default_factory=lambda: np.zeros(0))
    inewton: int = 0
    inewtonur: int = 0
    ivarcv: int = 0
    idewatcv: int = 0
    icellavg: int = 0
    name: str = ""
    disu: bool = True
    angldegx: np.ndarray | None = None  # per entry, degrees (ANGLDEGX)
    xc_u: np.ndarray | None = None      # per user cell: the cell centre (CELL2D)
    yc_u: np.ndarray | None = None
    ixt3d: int = 0          # NPF XT3D: 0 off, 1 XT3D, 2 XT3D RHS
    iavgkeff: int = 0       # effective K of K22/ANGLE1..3 without XT3D: 0 harmonic, 1 arithmetic
    k22: np.ndarray | None = None
    angle1: np.ndarray | None = None    # degrees
    angle2: np.ndarray | None = None
    angle3: np.ndarray | None = None

    def __post_init__(self):
        self.ja = disu_check(self.top_u, self.bot_u, self.area_u, self.iac, self.ja, self.ihc_u,
                             self.idomain, self.voffsettol)
        self._con = disu_connections(self.iac, self.ja, self.ihc_u, self.cl12, self.hwva_u,
                                     self.idomain, self.angldegx)

    @property
    def xc(self) -> np.ndarray:
        return np.asarray(self.xc_u, float)[self.nodeuser]

    @property
    def yc(self) -> np.ndarray:
        return np.asarray(self.yc_u, float)[self.nodeuser]

    @property
    def nlay(self) -> int:
        return 1

    @property
    def nrow(self) -> int:
        return 1

    @property
    def ncol(self) -> int:
        return self.nodes

    @property
    def nodes(self) -> int:
        return int(self._con["nodes"])

    @property
    def nodeuser(self) -> np.ndarray:
        return self._con["nodeuser"]

    @property
    def cell_top(self) -> np.ndarray:
        return np.asarray(self.top_u, float)[self.nodeuser]

    @property
    def cell_bot(self) -> np.ndarray:
        return np.asarray(self.bot_u, float)[self.nodeuser]

    @property
    def area(self) -> np.ndarray:
        return np.asarray(self.area_u, float)[self.nodeuser]

    def connections(self) -> dict:
        return self._con

    @property
    def ibound(self) -> np.ndarray:
        ib = np.ones(self.nodes, dtype=np.int32)
        ib[self.chd_node] = -1
        return ib


def make_disu_model(nlay: int = 2, nrow: int = 12, ncol: int = 16, seed: int = 0,
                    stagger: float = 0.0, transient: bool = False, newton: bool = False,
                    idomain_holes: int = 0) -> DisuModel:
    """A seeded DISU workload on the refined grid: lognormal K, CHD on the
    first and last coarse columns of every layer, wells and recharge on the
    top layer; `stagger` > 0 offsets the layer elevations column by column
    (IHC 2 connections); `idomain_holes` removes that many interior cells
    (IDOMAIN 0)."""
    from .dis import lognormal_field

    rng = np.random.default_rng(seed)
    box = (nrow // 3, nrow // 3 + max(1, nrow // 3), ncol // 3, ncol // 3 + max(1, ncol // 3))
    g = refined_grid(nlay, nrow, ncol, 50.0, box, thick=10.0, stagger=stagger, seed=seed)
    nu = g["iac"].size
    ncpl = g["ncpl"]
    x = g["xc"][:ncpl]
    west = np.flatnonzero(x < 50.0)
    east = np.flatnonzero(x > 50.0 * (ncol - 1))
    chd_u = np.concatenate([west + k * ncpl for k in range(nlay)] +
                           [east + k * ncpl for k in range(nlay)])
    idomain = np.ones(nu, np.int64)
    if idomain_holes:
        cand = np.setdiff1d(np.arange(nu), chd_u)
        idomain[rng.choice(cand, size=idomain_holes, replace=False)] = 0
    red = np.full(nu, -1)
    red[idomain > 0] = np.arange(int((idomain > 0).sum()))
    n = int((idomain > 0).sum())
    kf = lognormal_field(rng, (1, nu), 1.0, 3.0).ravel()[:nu]
    k = kf[idomain > 0]
    ict = np.full(n, 1 if newton else 0, np.int32)
    strt = np.full(n, 8.0 * nlay)
    chd_head_u = np.concatenate([np.full(west.size * nlay, 9.0 * nlay),
                                 np.full(east.size * nlay, 7.0 * nlay)])
    m = DisuModel(g["top"], g["bot"], g["area"], g["iac"], g["ja"], g["ihc"], g["cl12"], g["hwva"],
                  k, 0.1 * k, ict, strt, idomain=idomain if idomain_holes else None,
                  inewton=1 if newton else 0, name="disu-refined", angldegx=g["angldegx"],
                  xc_u=g["xc"], yc_u=g["yc"])
    if transient:
        m.ss, m.sy = np.full(n, 1e-5), np.full(n, 0.15)
    m.chd_node = red[chd_u].astype(np.int32)
    m.chd_head = chd_head_u
    chd = np.zeros(n, bool)
    chd[m.chd_node] = True
    top_layer = np.flatnonzero(red[:ncpl] >= 0)
    free = np.setdiff1d(red[top_layer], m.chd_node)
    m.wel_node = np.sort(rng.choice(free, size=max(1, free.size // 40), replace=False)).astype(np.int32)
    m.wel_q = rng.uniform(-300.0, -20.0, m.wel_node.size)
    m.rch_node = red[top_layer].astype(np.int32)
    m.rch_rate = np.full(m.rch_node.size, 2.0e-4)
    return m
