"""DISV (vertex) grids: layered grids of arbitrary polygons.

`disv_connections` builds the connectivity of a full DISV grid as MODFLOW 6
does (src/Model/ModelUtilities/Connections.f90:702-796 disvconnections and
:1272-1361 vertexconnect; DisvGeom.f90:136-202 cprops, :302-332
shared_edge, :339-386 get_area, :416-445 distance / distance_normal):

* node n = j + k*ncpl (cell j of layer k, 0-based);
* each row: the diagonal, the cell above and below, and every cell of the
  same layer with which the cell shares an edge (an edge of one cell's
  vertex list that appears reversed in the other's); the off-diagonals in
  ascending order (Sparse.f90:217-239);
* a cell's vertex list is closed by repeating its first vertex, as
  Disv.f90:548-585 define_cellverts does;
* vertical connections: ihc 0, hwva the cell's area, cl1/cl2 half the cell
  thicknesses; horizontal: ihc 1, hwva the shared edge's length, cl1/cl2 the
  normal distances from the two cell centres to that edge (the edge taken in
  the lower-numbered cell's vertex order).

The arithmetic follows the reference's expressions term by term, so the
arrays equal the oracle's bit for bit; the numpy evaluation is vectorised
over cells and connections.  `DisvModel` carries a GWF model on such a grid
with the attributes the NPF fill and the oracle read.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


def close_vertex_lists(icvert: list) -> tuple[np.ndarray, np.ndarray]:
    """iavert (ncpl + 1) and javert (0-based vertex numbers) with each cell's
    list closed by its first vertex unless it is closed already."""
    ia = [0]
    ja = []
    for verts in icvert:
        v = list(int(x) for x in verts)
        if v[-1] != v[0]:
            v.append(v[0])
        ja += v
        ia.append(len(ja))
    return np.array(ia, np.int64), np.array(ja, np.int64)


def _cell_area(iavert, javert, vx, vy) -> np.ndarray:
    """get_area for every cell, term by term in the reference's order."""
    ncpl = iavert.size - 1
    nv = np.diff(iavert)
    x1 = vx[javert[iavert[:-1]]]
    y1 = vy[javert[iavert[:-1]]]
    area = np.zeros(ncpl)
    for t in range(int(nv.max())):
        on = t < nv
        q = iavert[:-1] + np.minimum(t, nv - 1)
        nxt = np.where(t + 1 < nv, q + 1, iavert[:-1])
        x = vx[javert[q]]
        y = vy[javert[nxt]]
        area = np.where(on, area + (x - x1) * (y - y1), area)
    for t in range(int(nv.max())):
        on = t < nv
        q = iavert[:-1] + np.minimum(t, nv - 1)
        nxt = np.where(t + 1 < nv, q + 1, iavert[:-1])
        y = vy[javert[q]]
        x = vx[javert[nxt]]
        area = np.where(on, area - (x - x1) * (y - y1), area)
    return np.abs(area) * 0.5


def _shared_edges(iavert, javert, nvert):
    """(j1, j2, a, b) for every ordered pair of cells sharing an edge: a, b
    the first consecutive vertices of j1's list found reversed in j2's."""
    ncpl = iavert.size - 1
    cell = np.repeat(np.arange(ncpl), np.diff(iavert) - 1)
    first = np.concatenate([np.arange(iavert[j], iavert[j + 1] - 1) for j in range(ncpl)])
    a, b = javert[first], javert[first + 1]
    pos = first - iavert[cell]
    key = a * nvert + b
    rkey = b * nvert + a
    order = np.argsort(key, kind="stable")
    ks = key[order]
    lo = np.searchsorted(ks, rkey, side="left")
    hi = np.searchsorted(ks, rkey, side="right")
    out = []
    for t in np.flatnonzero(hi > lo):
        for u in order[lo[t]:hi[t]]:
            if cell[u] != cell[t]:
                out.append((cell[t], cell[u], pos[t], a[t], b[t]))
    if not out:
        return np.zeros((0, 4), np.int64)
    e = np.array(out, np.int64)
    # the first matching pair in j1's vertex order
    o = np.lexsort((e[:, 2], e[:, 1], e[:, 0]))
    e = e[o]
    keep = np.ones(len(e), bool)
    keep[1:] = (e[1:, 0] != e[:-1, 0]) | (e[1:, 1] != e[:-1, 1])
    e = e[keep]
    return e[:, [0, 1, 3, 4]]


def disv_nodereduced(idomain) -> np.ndarray:
    """nodereduced in the reference's convention (Disv.f90 grid finalize):
    the 1-based reduced number of a cell with IDOMAIN > 0, 0 for IDOMAIN 0
    (removed), -1 for IDOMAIN < 0 (a vertical pass-through cell)."""
    idomain = np.asarray(idomain, np.int64)
    red = np.where(idomain > 0, 0, np.where(idomain < 0, -1, 0)).astype(np.int64)
    act = idomain > 0
    red[act] = np.arange(1, int(act.sum()) + 1)
    return red


def disv_connections(nlay: int, iavert, javert, vx, vy, xc, yc, top, bot, idomain=None) -> dict:
    """CSR connectivity and symmetric-connection geometry of a DISV grid
    (top/bot per user node, layer-major), reduced to the cells with IDOMAIN
    > 0 as vertexconnect (Connections.f90:1272-1361) does: a vertical
    connection passes through cells with IDOMAIN < 0 to the next cell above
    or below that is not one, and exists if that cell is active; also the
    cell areas (ncpl) and nodeuser (reduced -> user, 0-based)."""
    iavert = np.asarray(iavert, np.int64)
    javert = np.asarray(javert, np.int64)
    vx, vy = np.asarray(vx, float), np.asarray(vy, float)
    xc, yc = np.asarray(xc, float), np.asarray(yc, float)
    top, bot = np.asarray(top, float), np.asarray(bot, float)
    ncpl = iavert.size - 1
    nu = nlay * ncpl
    red = disv_nodereduced(np.ones(nu) if idomain is None else idomain)
    nodeuser = np.flatnonzero(red > 0)
    n = nodeuser.size
    nvert = int(javert.max()) + 1
    edges = _shared_edges(iavert, javert, nvert)  # (j1, j2, a, b)
    # horizontal neighbours per cell, ascending
    nbr = [[] for _ in range(ncpl)]
    eab = {}
    for j1, j2, a, b in edges:
        nbr[j1].append(j2)
        eab[(j1, j2)] = (a, b)
    rows = []
    for u in nodeuser:
        k, j = divmod(int(u), ncpl)
        off = []
        for step in (-1, 1):
            kk = k + step
            while 0 <= kk < nlay and red[j + kk * ncpl] < 0:
                kk += step
            if 0 <= kk < nlay and red[j + kk * ncpl] > 0:
                off.append(int(red[j + kk * ncpl]) - 1)
        off += [int(red[j2 + k * ncpl]) - 1 for j2 in nbr[j] if red[j2 + k * ncpl] > 0]
        rows.append([int(red[u]) - 1] + sorted(set(off)))
    ia = np.zeros(n + 1, np.int64)
    ia[1:] = np.cumsum([len(r) for r in rows])
    ja = np.concatenate([np.array(r, np.int64) for r in rows])
    nja = int(ia[-1])
    rown = np.repeat(np.arange(n), np.diff(ia))
    # isym: position of (m, n) in row m
    pos_of = {}
    for p in range(nja):
        pos_of[(int(rown[p]), int(ja[p]))] = p
    isym = np.array([pos_of[(int(ja[p]), int(rown[p]))] for p in range(nja)], np.int64)
    upper = ja > rown
    jas = np.full(nja, -1, np.int64)
    njas = int(upper.sum())
    jas[upper] = np.arange(njas)
    lower = ja < rown
    jas[lower] = jas[isym[lower]]
    area = _cell_area(iavert, javert, vx, vy)
    ihc = np.zeros(njas, np.int64)
    cl1, cl2, hwva = np.zeros(njas), np.zeros(njas), np.zeros(njas)
    pu = np.flatnonzero(upper)
    nn, mm = rown[pu], ja[pu]
    s = jas[pu]
    un, um = nodeuser[nn], nodeuser[mm]
    jn, jm = un % ncpl, um % ncpl
    vert = jn == jm
    sv = s[vert]
    ihc[sv] = 0
    hwva[sv] = area[jn[vert]]
    cl1[sv] = 0.5 * (top[un[vert]] - bot[un[vert]])
    cl2[sv] = 0.5 * (top[um[vert]] - bot[um[vert]])
    hz = ~vert
    sh = s[hz]
    ihc[sh] = 1
    ab = np.array([eab[(int(x), int(y))] for x, y in zip(jn[hz], jm[hz])], np.int64).reshape(-1, 2)
    x1, y1 = vx[ab[:, 0]], vy[ab[:, 0]]
    x2, y2 = vx[ab[:, 1]], vy[ab[:, 1]]
    dist = np.sqrt((x1 - x2) * (x1 - x2) + (y1 - y2) * (y1 - y2))
    hwva[sh] = dist

    def dnorm(x0, y0):
        d = np.abs((x2 - x1) * (y1 - y0) - (x1 - x0) * (y2 - y1))
        return d / dist

    cl1[sh] = dnorm(xc[jn[hz]], yc[jn[hz]])
    cl2[sh] = dnorm(xc[jm[hz]], yc[jm[hz]])
    # anglex (DisvGeom.f90:193-199, 394-412): the angle of the shared edge's
    # normal, atan2(dx, -dy) of the edge in the lower-numbered cell's vertex
    # order, in [0, 2 pi); evaluated with the C library's atan2 one value at
    # a time, as the Fortran does
    anglex = np.zeros(njas)
    two_pi = 2.0 * (4.0 * math.atan(1.0))
    ax = [math.atan2(float(a), float(-b)) for a, b in zip(x2 - x1, y2 - y1)]
    anglex[sh] = [v if v >= 0.0 else two_pi + v for v in ax]
    return dict(nodes=n, nja=nja, njas=njas, ia=ia.astype(np.int32), ja=ja.astype(np.int32),
                isym=isym.astype(np.int32), jas=jas.astype(np.int32), ihc=ihc.astype(np.int32),
                cl1=cl1, cl2=cl2, hwva=hwva, area=area, anglex=anglex,
                nodeuser=nodeuser.astype(np.int32), nodereduced=red.astype(np.int32))


@dataclass
class DisvModel:
    """A GWF model on a DISV grid (NPF, IC, STO, CHD, WEL, RCH), node order
    layer-major.  nrow is 1 and ncol is ncpl, so the per-column rules written
    for DIS (the bottom cell of a column) read the same cells."""

    nlay: int
    vertices: np.ndarray        # (nvert, 2)
    icvert: list                # per cell its vertex numbers (0-based, clockwise)
    xc: np.ndarray              # cell centres (ncpl)
    yc: np.ndarray
    top: np.ndarray             # (ncpl) model top
    botm: np.ndarray            # (nlay*ncpl)
    k11: np.ndarray
    k33: np.ndarray
    icelltype: np.ndarray
    strt: np.ndarray
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
    disv: bool = True
    idomain: np.ndarray | None = None  # per user cell; the cell arrays are per active cell
    ixt3d: int = 0          # NPF XT3D: 0 off, 1 XT3D, 2 XT3D RHS
    iavgkeff: int = 0       # effective K of K22/ANGLE1..3 without XT3D: 0 harmonic, 1 arithmetic
    k22: np.ndarray | None = None
    angle1: np.ndarray | None = None   # degrees
    angle2: np.ndarray | None = None
    angle3: np.ndarray | None = None

    @property
    def ncpl(self) -> int:
        return len(self.icvert)

    @property
    def nrow(self) -> int:
        return 1

    @property
    def ncol(self) -> int:
        return self.ncpl

    @property
    def nodeuser(self) -> np.ndarray:
        nu = self.nlay * self.ncpl
        if self.idomain is None:
            return np.arange(nu)
        return np.flatnonzero(np.asarray(self.idomain) > 0)

    @property
    def nodes(self) -> int:
        return int(self.nodeuser.size)

    @property
    def vertex_lists(self):
        return close_vertex_lists(self.icvert)

    @property
    def user_top(self) -> np.ndarray:
        t = np.empty(self.nlay * self.ncpl)
        t[:self.ncpl] = self.top
        t[self.ncpl:] = self.botm[:-self.ncpl]
        return t

    @property
    def cell_top(self) -> np.ndarray:
        return self.user_top[self.nodeuser]

    @property
    def cell_bot(self) -> np.ndarray:
        return np.asarray(self.botm)[self.nodeuser]

    def connections(self) -> dict:
        iav, jav = self.vertex_lists
        return disv_connections(self.nlay, iav, jav, self.vertices[:, 0], self.vertices[:, 1],
                                self.xc, self.yc, self.user_top, self.botm, self.idomain)

    @property
    def area(self) -> np.ndarray:
        return np.tile(self.connections()["area"], self.nlay)[self.nodeuser]

    @property
    def xcn(self) -> np.ndarray:
        """cell centres per active cell"""
        return np.tile(self.xc, self.nlay)[self.nodeuser]

    @property
    def ycn(self) -> np.ndarray:
        return np.tile(self.yc, self.nlay)[self.nodeuser]

    @property
    def ibound(self) -> np.ndarray:
        ib = np.ones(self.nodes, dtype=np.int32)
        ib[self.chd_node] = -1
        return ib


def hex_mesh(nx: int, ny: int, size: float = 10.0, seed: int = 0, jitter: float = 0.15):
    """A seeded mesh of hexagons in `nx` columns and `ny` rows (offset rows,
    shared vertices, clockwise lists) with jittered interior vertices, so that
    edge lengths and normal distances vary from cell to cell: (vertices,
    icvert, xc, yc)."""
    rng = np.random.default_rng(seed)
    h = size * np.sqrt(3.0) / 2.0
    verts = {}
    vx, vy = [], []

    def vid(x, y):
        key = (round(x, 6), round(y, 6))
        if key not in verts:
            verts[key] = len(vx)
            vx.append(x)
            vy.append(y)
        return verts[key]

    icvert, xc, yc = [], [], []
    for r in range(ny):
        for c in range(nx):
            cx = c * 1.5 * size
            cy = r * 2 * h + (h if c % 2 else 0.0)
            ang = np.deg2rad(np.array([120.0, 60.0, 0.0, -60.0, -120.0, 180.0]))
            pts = [vid(cx + size * np.cos(a), cy + size * np.sin(a)) for a in ang]
            icvert.append(pts)
            xc.append(cx)
            yc.append(cy)
    vx, vy = np.array(vx), np.array(vy)
    # jitter the vertices used by three cells (interior), keep the centres
    use = np.zeros(len(vx), int)
    for pts in icvert:
        for p in pts:
            use[p] += 1
    inner = use >= 3
    vx[inner] += rng.uniform(-jitter, jitter, inner.sum()) * size
    vy[inner] += rng.uniform(-jitter, jitter, inner.sum()) * size
    return np.stack([vx, vy], axis=1), icvert, np.array(xc), np.array(yc)


def make_disv_model(nlay: int = 3, nx: int = 30, ny: int = 20, seed: int = 0,
                    transient: bool = False, newton: bool = False,
                    idomain: np.ndarray | None = None) -> DisvModel:
    """A seeded DISV workload on the hexagon mesh: lognormal K per layer,
    CHD on the cells of the first and last columns of every layer, wells and
    recharge."""
    from .dis import lognormal_field

    rng = np.random.default_rng(seed)
    verts, icvert, xc, yc = hex_mesh(nx, ny, seed=seed)
    ncpl = len(icvert)
    n = nlay * ncpl
    top = np.full(ncpl, 10.0 * nlay)
    botm = np.repeat(10.0 * (nlay - 1 - np.arange(nlay)), ncpl).astype(float)
    k = np.concatenate([lognormal_field(rng, (ny, nx), 1.0, 3.0).ravel() for _ in range(nlay)])
    ict = np.full(n, 1 if newton else 0, np.int32)
    m = DisvModel(nlay, verts, icvert, xc, yc, top, botm, k, 0.1 * k, ict, np.full(n, 8.0 * nlay),
                  inewton=1 if newton else 0, name="disv-hex")
    if transient:
        m.ss, m.sy = np.full(n, 1e-5), np.full(n, 0.15)
    col = np.arange(ncpl) % nx
    west = np.flatnonzero(col == 0)
    east = np.flatnonzero(col == nx - 1)
    m.chd_node = np.concatenate([west + k2 * ncpl for k2 in range(nlay)] +
                                [east + k2 * ncpl for k2 in range(nlay)]).astype(np.int32)
    m.chd_head = np.concatenate([np.full(west.size * nlay, 9.0 * nlay),
                                 np.full(east.size * nlay, 7.0 * nlay)])
    chd = np.zeros(n, bool)
    chd[m.chd_node] = True
    m.wel_node = np.sort(rng.choice(np.flatnonzero(~chd), size=max(1, ncpl // 40),
                                    replace=False)).astype(np.int32)
    m.wel_q = rng.uniform(-300.0, -20.0, m.wel_node.size)
    m.rch_node = np.arange(ncpl, dtype=np.int32)
    m.rch_rate = np.full(ncpl, 2.0e-4)
    if idomain is not None:
        # keep the active cells: cell arrays and boundaries in the reduced
        # numbering (boundaries on removed cells dropped)
        idomain = np.asarray(idomain)
        keep = idomain > 0
        red = np.full(n, -1)
        red[keep] = np.arange(int(keep.sum()))
        m.idomain = idomain
        for f in ("k11", "k33", "icelltype", "strt", "ss", "sy"):
            v = getattr(m, f)
            if v is not None:
                setattr(m, f, np.asarray(v)[keep])
        for nf, vf in (("chd_node", "chd_head"), ("wel_node", "wel_q"), ("rch_node", "rch_rate")):
            nodes = getattr(m, nf)
            ok = keep[nodes]
            setattr(m, nf, red[nodes[ok]].astype(np.int32))
            setattr(m, vf, np.asarray(getattr(m, vf))[ok])
    return m
