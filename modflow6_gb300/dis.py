"""Structured DIS grid models for the GB300 IMS path.

* `dis_connections` builds the grid connectivity exactly as MODFLOW 6 does for
  a full DIS grid (Connections.f90:463-698 `disconnections`, Sparse.f90:217-239
  sort with the diagonal first, `fillisym`/`filljas` :1205-1268), vectorised.
  Node n = j + i*ncol + k*nrow*ncol (GeomUtil.f90:82-95), 0-based.
* `GwfDisModel` is a single GWF model (DIS, IC, NPF, STO, CHD, WEL, RCH).
* `make_config` generates the seeded synthetic workloads: lognormal K fields
  (white noise, Gaussian filter with the correlation length in cells,
  re-standardised, scaled by sigma_lnK, exponentiated), CHD faces, wells and
  recharge.  No external data set is used.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


def dis_connections(nlay: int, nrow: int, ncol: int, delr: np.ndarray, delc: np.ndarray,
                    top: np.ndarray, bot: np.ndarray) -> dict:
    """CSR connectivity and symmetric-connection geometry of a full DIS grid."""
    nrc = nrow * ncol
    n = nlay * nrc
    node = np.arange(n, dtype=np.int64)
    k, rem = np.divmod(node, nrc)
    i, j = np.divmod(rem, ncol)
    # neighbours in sorted order: up(k-1), back(i-1), left(j-1), right, front, down
    offs = [-nrc, -ncol, -1, 1, ncol, nrc]
    has = [k > 0, i > 0, j > 0, j < ncol - 1, i < nrow - 1, k < nlay - 1]
    cnt = 1 + np.sum(np.stack(has), axis=0)
    ia = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(cnt, out=ia[1:])
    nja = int(ia[-1])
    ja = np.empty(nja, dtype=np.int64)
    ja[ia[:-1]] = node
    pos = ia[:-1] + 1
    slot = []  # per direction: CSR position of that neighbour in each row, or -1
    for o, h in zip(offs, has):
        ja[pos[h]] = node[h] + o
        slot.append(np.where(h, pos, -1))
        pos = pos + h
    # isym: position of (m, n) in row m; direction d pairs with 5 - d
    isym = np.empty(nja, dtype=np.int64)
    isym[ia[:-1]] = ia[:-1]
    for d, o in enumerate(offs):
        p = slot[d]
        h = p >= 0
        isym[p[h]] = slot[5 - d][node[h] + o]
    # jas: upper connections numbered in (node, JA) order, i.e. right, front, down
    upper = np.zeros(nja, dtype=bool)
    for d in (3, 4, 5):
        p = slot[d]
        upper[p[p >= 0]] = True
    jas = np.full(nja, -1, dtype=np.int64)
    njas = int(upper.sum())
    jas[upper] = np.arange(njas)
    lower = np.zeros(nja, dtype=bool)
    for d in (0, 1, 2):
        p = slot[d]
        lower[p[p >= 0]] = True
    jas[lower] = jas[isym[lower]]
    # symmetric geometry (ihc, cl1, cl2, hwva) per jas
    ihc = np.zeros(njas, dtype=np.int64)
    cl1 = np.zeros(njas)
    cl2 = np.zeros(njas)
    hwva = np.zeros(njas)
    thick = top - bot
    p = slot[3]; h = p >= 0; s = jas[p[h]]
    ihc[s] = 1; cl1[s] = 0.5 * delr[j[h]]; cl2[s] = 0.5 * delr[j[h] + 1]; hwva[s] = delc[i[h]]
    p = slot[4]; h = p >= 0; s = jas[p[h]]
    ihc[s] = 1; cl1[s] = 0.5 * delc[i[h]]; cl2[s] = 0.5 * delc[i[h] + 1]; hwva[s] = delr[j[h]]
    p = slot[5]; h = p >= 0; s = jas[p[h]]
    ihc[s] = 0; cl1[s] = 0.5 * thick[node[h]]; cl2[s] = 0.5 * thick[node[h] + nrc]
    hwva[s] = delr[j[h]] * delc[i[h]]
    return dict(nodes=n, nja=nja, njas=njas, ia=ia.astype(np.int32), ja=ja.astype(np.int32),
                isym=isym.astype(np.int32), jas=jas.astype(np.int32), ihc=ihc.astype(np.int32),
                cl1=cl1, cl2=cl2, hwva=hwva)


def lognormal_field(rng: np.random.Generator, shape: tuple, sigma_ln: float, corr: float,
                    kgeo: float = 1.0) -> np.ndarray:
    """exp(sigma_ln * standardised Gaussian-filtered white noise) * kgeo."""
    from scipy.ndimage import gaussian_filter

    w = rng.standard_normal(shape)
    if corr > 0:
        w = gaussian_filter(w, sigma=corr, mode="reflect")
    sd = w.std()
    w = (w - w.mean()) / (sd if sd > 0 else 1.0)
    return kgeo * np.exp(sigma_ln * w)


@dataclass
class GwfDisModel:
    nlay: int
    nrow: int
    ncol: int
    delr: np.ndarray
    delc: np.ndarray
    top: np.ndarray                # (nrow*ncol,) model top
    botm: np.ndarray               # (nlay*nrow*ncol,)
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
    inewtonur: int = 0      # NEWTON UNDER_RELAXATION (gwf.f90:181)
    ivarcv: int = 0         # NPF VARIABLECV
    idewatcv: int = 0       # NPF VARIABLECV DEWATERED
    icellavg: int = 0       # ALTERNATIVE_CELL_AVERAGING: 0 harmonic, 1 LOGARITHMIC, 2 AMT-LMK, 3 AMT-HMK
    name: str = ""
    ixt3d: int = 0          # NPF XT3D: 0 off, 1 XT3D, 2 XT3D RHS
    iavgkeff: int = 0       # effective K of K22/ANGLE1..3 without XT3D: 0 harmonic, 1 arithmetic
    k22: np.ndarray | None = None      # NPF K22 (default K11)
    angle1: np.ndarray | None = None   # NPF ANGLE1..3 in degrees; XT3D without ANGLE2
    angle2: np.ndarray | None = None   # has no z component in its horizontal terms
    angle3: np.ndarray | None = None

    @property
    def nodes(self) -> int:
        return self.nlay * self.nrow * self.ncol

    @property
    def cell_top(self) -> np.ndarray:
        nrc = self.nrow * self.ncol
        t = np.empty(self.nodes)
        t[:nrc] = self.top
        t[nrc:] = self.botm[:-nrc]
        return t

    @property
    def cell_bot(self) -> np.ndarray:
        return self.botm

    @property
    def area(self) -> np.ndarray:
        a2 = np.outer(self.delc, self.delr).ravel()
        return np.tile(a2, self.nlay)

    def connections(self) -> dict:
        return dis_connections(self.nlay, self.nrow, self.ncol, self.delr, self.delc,
                               self.cell_top, self.cell_bot)

    @property
    def ibound(self) -> np.ndarray:
        ib = np.ones(self.nodes, dtype=np.int32)
        ib[self.chd_node] = -1
        return ib


def _faces_chd(nlay, nrow, ncol, hwest, heast):
    nrc = nrow * ncol
    k, i = np.meshgrid(np.arange(nlay), np.arange(nrow), indexing="ij")
    west = (k * nrc + i * ncol).ravel()
    east = (k * nrc + i * ncol + ncol - 1).ravel()
    nodes = np.concatenate([west, east]).astype(np.int32)
    heads = np.concatenate([np.full(west.size, hwest), np.full(east.size, heast)])
    return nodes, heads


def make_config(name: str, seed: int = 0, scale: float = 1.0) -> GwfDisModel:
    """Seeded synthetic workloads.

    c1 : 100x100x1 confined, lnK~N(0,1) corr 5, CHD 10/0 on columns 1/100,
         recharge 1e-4 m/d (CG+ILU0, FP64).
    c2 : 1000x1000x10 confined, per-layer lnKh~N(0,1.5^2) corr 20, Kv=0.1 Kh,
         CHD 20 m west face / 0 m east face, 5000 wells U(-500,-50) m3/d.
    c3 : 500x500x5 convertible (Newton), Sy 0.15, Ss 1e-5, top 50, bottom
         sloping 0 to -40, 2000 wells U(-1000,0), recharge U(0,5e-4).
    c5 : 256x256x3 transient confined, 50 wells U(-800,0).
    xt3d : 200x200x3 confined, full-tensor (NPF XT3D): lnK11~N(0,1) corr 10,
         K22 0.2 K11, K33 0.05 K11, ANGLE1/2/3 30/15/5 degrees, CHD 28/22 m
         on the west/east faces, 200 wells U(-200,-20) m3/d.
    `scale` < 1 shrinks nrow/ncol for CPU-sized parity cases of c2/c3/c5.
    """
    rng = np.random.default_rng(seed)
    if name == "c1":
        nlay, nrow, ncol = 1, 100, 100
        delr = np.full(ncol, 10.0); delc = np.full(nrow, 10.0)
        top = np.full(nrow * ncol, 10.0); botm = np.zeros(nlay * nrow * ncol)
        k = lognormal_field(rng, (nrow, ncol), 1.0, 5.0).ravel()
        m = GwfDisModel(nlay, nrow, ncol, delr, delc, top, botm, k.copy(), k.copy(),
                        np.zeros(nrow * ncol, np.int32), np.full(nrow * ncol, 10.0), name="c1")
        m.chd_node, m.chd_head = _faces_chd(nlay, nrow, ncol, 10.0, 0.0)
        m.rch_node = np.arange(nrow * ncol, dtype=np.int32)
        m.rch_rate = np.full(nrow * ncol, 1.0e-4)
        return m
    if name == "c2":
        nlay = 10
        nrow = ncol = max(4, int(round(1000 * scale)))
        nrc = nrow * ncol
        delr = np.full(ncol, 10.0); delc = np.full(nrow, 10.0)
        top = np.full(nrc, 100.0)
        botm = np.repeat(100.0 - 10.0 * np.arange(1, nlay + 1), nrc)
        corr = 20.0 * scale if scale < 1 else 20.0
        kh = np.concatenate([lognormal_field(rng, (nrow, ncol), 1.5, corr).ravel() for _ in range(nlay)])
        m = GwfDisModel(nlay, nrow, ncol, delr, delc, top, botm, kh, 0.1 * kh,
                        np.zeros(nlay * nrc, np.int32), np.full(nlay * nrc, 10.0), name="c2")
        m.chd_node, m.chd_head = _faces_chd(nlay, nrow, ncol, 20.0, 0.0)
        nwel = max(1, int(round(5000 * scale * scale)))
        chd = np.zeros(m.nodes, bool); chd[m.chd_node] = True
        cand = np.flatnonzero(~chd)
        m.wel_node = np.sort(rng.choice(cand, size=nwel, replace=False)).astype(np.int32)
        m.wel_q = rng.uniform(-500.0, -50.0, nwel)
        return m
    if name == "c3":
        nlay = 5
        nrow = ncol = max(4, int(round(500 * scale)))
        nrc = nrow * ncol
        delr = np.full(ncol, 10.0); delc = np.full(nrow, 10.0)
        top = np.full(nrc, 50.0)
        bottom = np.tile(np.linspace(0.0, -40.0, ncol), nrow)
        frac = np.arange(1, nlay + 1) / nlay
        botm = np.concatenate([50.0 + f * (bottom - 50.0) for f in frac])
        k = np.concatenate([lognormal_field(rng, (nrow, ncol), 1.0, 10.0).ravel() for _ in range(nlay)])
        m = GwfDisModel(nlay, nrow, ncol, delr, delc, top, botm, k, k.copy(),
                        np.ones(nlay * nrc, np.int32), np.full(nlay * nrc, 45.0),
                        ss=np.full(nlay * nrc, 1.0e-5), sy=np.full(nlay * nrc, 0.15),
                        inewton=1, name="c3")
        nwel = max(1, int(round(2000 * scale * scale)))
        m.wel_node = np.sort(rng.choice(m.nodes, size=nwel, replace=False)).astype(np.int32)
        m.wel_q = rng.uniform(-1000.0, 0.0, nwel)
        m.rch_node = np.arange(nrc, dtype=np.int32)
        m.rch_rate = rng.uniform(0.0, 5.0e-4, nrc)
        return m
    if name == "c5":
        nlay = 3
        nrow = ncol = max(4, int(round(256 * scale)))
        nrc = nrow * ncol
        delr = np.full(ncol, 10.0); delc = np.full(nrow, 10.0)
        top = np.full(nrc, 30.0)
        botm = np.repeat(np.array([20.0, 10.0, 0.0]), nrc)
        k = np.concatenate([lognormal_field(rng, (nrow, ncol), 1.0, 8.0).ravel() for _ in range(nlay)])
        m = GwfDisModel(nlay, nrow, ncol, delr, delc, top, botm, k, 0.1 * k,
                        np.zeros(nlay * nrc, np.int32), np.full(nlay * nrc, 25.0),
                        ss=np.full(nlay * nrc, 1.0e-5), sy=np.full(nlay * nrc, 0.15), name="c5")
        m.chd_node, m.chd_head = _faces_chd(nlay, nrow, ncol, 25.0, 20.0)
        chd = np.zeros(m.nodes, bool); chd[m.chd_node] = True
        nwel = 50
        m.wel_node = np.sort(rng.choice(np.flatnonzero(~chd), size=nwel, replace=False)).astype(np.int32)
        m.wel_q = rng.uniform(-800.0, 0.0, nwel)
        return m
    if name == "xt3d":
        nlay = 3
        nrow = ncol = max(6, int(round(200 * scale)))
        nrc = nrow * ncol
        n = nlay * nrc
        delr = np.full(ncol, 10.0); delc = np.full(nrow, 10.0)
        top = np.full(nrc, 30.0)
        botm = np.repeat(np.array([20.0, 10.0, 0.0]), nrc)
        k = np.concatenate([lognormal_field(rng, (nrow, ncol), 1.0, 10.0).ravel() for _ in range(nlay)])
        m = GwfDisModel(nlay, nrow, ncol, delr, delc, top, botm, k, 0.05 * k,
                        np.zeros(n, np.int32), np.full(n, 25.0), name="xt3d")
        m.ixt3d = 1
        m.k22 = 0.2 * k
        m.angle1, m.angle2, m.angle3 = np.full(n, 30.0), np.full(n, 15.0), np.full(n, 5.0)
        m.chd_node, m.chd_head = _faces_chd(nlay, nrow, ncol, 28.0, 22.0)
        chd = np.zeros(n, bool); chd[m.chd_node] = True
        nwel = max(1, int(round(200 * scale * scale)))
        m.wel_node = np.sort(rng.choice(np.flatnonzero(~chd), size=nwel, replace=False)).astype(np.int32)
        m.wel_q = rng.uniform(-200.0, -20.0, nwel)
        return m
    raise ValueError(f"unknown config {name!r}")
