"""Device-resident NumericalSolution for one GWF model (gbsln_* C ABI) on a
DIS grid, or on a DISV or DISU grid through its connectivity
(gbsln_create_grid).

`GwfSolution` mirrors the per-time-step use of NumericalSolutionType
(src/Solution/NumericalSolution.f90: sln_ca :1287, solve :1482-1837) for a
single GWF model with the DIS, IC, NPF, STO, CHD, WEL and RCH packages: the
fill, the sln_ls fix-ups, the IMS apply, dxmax and under-relaxation all run in
HBM; only per-outer-iteration scalars return to the host.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .dis import GwfDisModel
from .ims import ImsLinearSettings


@dataclass
class Nonlinear:
    """IMS NONLINEAR block (defaults: COMPLEXITY SIMPLE, sln_setouter :2626-2637)."""

    dvclose: float = 1.0e-3   # OUTER_DVCLOSE
    mxiter: int = 25          # OUTER_MAXIMUM
    nonmeth: int = 0          # UNDER_RELAXATION: 0 none, 1 simple, 2 cooley, 3 dbd
    theta: float = 1.0
    akappa: float = 0.0
    gamma: float = 1.0
    amomentum: float = 0.0
    iallowptc: int = 1
    numtrack: int = 0         # BACKTRACKING_NUMBER (0: no backtracking)
    btol: float = 0.0         # BACKTRACKING_TOLERANCE
    breduc: float = 0.0       # BACKTRACKING_REDUCTION_FACTOR
    res_lim: float = 0.0      # BACKTRACKING_RESIDUAL_LIMIT

    @classmethod
    def preset(cls, complexity: str, **kw) -> "Nonlinear":
        c = complexity.upper()
        if c == "SIMPLE":
            n = cls(1e-3, 25, 0, 1.0, 0.0, 1.0, 0.0)
        elif c == "MODERATE":
            n = cls(1e-2, 50, 3, 0.9, 1e-4, 0.0, 0.0)
        elif c == "COMPLEX":
            # sln_setouter (NumericalSolution.f90:2657-2668), with backtracking
            n = cls(1e-1, 100, 3, 0.8, 1e-4, 0.0, 0.0, 1, 20, 1.05, 0.1, 0.002)
        else:
            raise ValueError(complexity)
        for k, v in kw.items():
            setattr(n, k, v)
        return n


def sln_ls_fixups(ia, ja, active, amat, rhs, x, isymmetric=True):
    """Host form of the sln_ls loose ends (NumericalSolution.f90:2434-2478) for
    callers that assemble on the host and call the C ABI with host arrays."""
    amat = amat.copy()
    rhs = rhs.copy()
    n = ia.size - 1
    diag = ia[:-1]
    act = active > 0
    small = act & (np.abs(amat[diag]) < 1e-15)
    amat[diag[small]] = -1.0
    rhs[small] = rhs[small] + (-1.0) * x[small]
    rows = np.repeat(np.arange(n), np.diff(ia))
    inactive = ~act
    off = rows != ja
    kill = inactive[rows] & off
    amat[kill] = 0.0
    amat[diag[inactive]] = 1.0
    rhs[inactive] = x[inactive]
    if isymmetric:
        elim = off & act[rows] & (active[ja] < 0)
        idx = np.flatnonzero(elim)
        # per row, in JA order: rhs -= a * x(col)
        for p in idx:
            r = rows[p]
            rhs[r] = rhs[r] - amat[p] * x[ja[p]]
        amat[idx] = 0.0
    return amat, rhs


class LsFixups:
    """The sln_ls loose ends (NumericalSolution.f90:2434-2478) for one matrix
    structure and IBOUND, applied in place to host arrays each outer
    iteration: the positions they touch are found once, so an application
    costs a pass over the diagonal and the few CHD-related entries.  Results
    equal `sln_ls_fixups` bit for bit (the CHD columns are moved to the
    right-hand side row by row in JA order, as the reference loops)."""

    def __init__(self, ia, ja, active, isymmetric=True):
        ia = np.asarray(ia, np.int64)
        ja = np.asarray(ja, np.int64)
        n = ia.size - 1
        self.diag = ia[:-1]
        self.act = np.asarray(active) > 0
        rows = np.repeat(np.arange(n), np.diff(ia))
        off = rows != ja
        self.inactive = np.flatnonzero(~self.act)
        self.kill = np.flatnonzero(~self.act[rows] & off)
        if isymmetric:
            e = np.flatnonzero(off & self.act[rows] & (np.asarray(active)[ja] < 0))
        else:
            e = np.zeros(0, np.int64)
        self.eidx, self.erow, self.ecol = e, rows[e], ja[e]

    def apply(self, amat, rhs, x):
        d = amat[self.diag]
        small = np.flatnonzero(self.act & (np.abs(d) < 1e-15))
        amat[self.diag[small]] = -1.0
        rhs[small] = rhs[small] + (-1.0) * x[small]
        amat[self.kill] = 0.0
        amat[self.diag[self.inactive]] = 1.0
        rhs[self.inactive] = x[self.inactive]
        if self.eidx.size:
            np.subtract.at(rhs, self.erow, amat[self.eidx] * x[self.ecol])
            amat[self.eidx] = 0.0
        return amat, rhs


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class GwfSolution:
    def __init__(self, m: GwfDisModel, ims: ImsLinearSettings, nl: Nonlinear,
                 satomega: float = 1.0e-6):
        lib = _lib.load()
        self.m = m
        general = bool(getattr(m, "disv", False) or getattr(m, "disu", False))
        if general:
            con = m.connections()
            keep = dict(delr=_f([0.0]), delc=_f([0.0]), top=_f([0.0]), botm=_f([0.0]),
                        g_ia=_i(con["ia"]), g_ja=_i(con["ja"]), g_ihc=_i(con["ihc"]),
                        g_cl1=_f(con["cl1"]), g_cl2=_f(con["cl2"]), g_hwva=_f(con["hwva"]),
                        g_top=_f(m.cell_top), g_bot=_f(m.cell_bot), g_area=_f(m.area))
            grid = _lib.GbslnGrid(int(m.nodes), int(con["nja"]), _lib.iptr(keep["g_ia"]),
                                  _lib.iptr(keep["g_ja"]), _lib.iptr(keep["g_ihc"]),
                                  _lib.dptr(keep["g_cl1"]), _lib.dptr(keep["g_cl2"]),
                                  _lib.dptr(keep["g_hwva"]), _lib.dptr(keep["g_top"]),
                                  _lib.dptr(keep["g_bot"]), _lib.dptr(keep["g_area"]))
        else:
            keep = dict(delr=_f(m.delr), delc=_f(m.delc), top=_f(m.top), botm=_f(m.botm))
        keep.update(k11=_f(m.k11), k33=_f(m.k33), ict=_i(m.icelltype),
                    chd_node=_i(m.chd_node), chd_head=_f(m.chd_head), wel_node=_i(m.wel_node),
                    wel_q=_f(m.wel_q), rch_node=_i(m.rch_node), rch_rate=_f(m.rch_rate),
                    strt=_f(m.strt))
        ss = sy = None
        if m.ss is not None and m.sy is not None:
            keep["ss"], keep["sy"] = _f(m.ss), _f(m.sy)
            ss, sy = _lib.dptr(keep["ss"]), _lib.dptr(keep["sy"])
        self._keep = keep
        cm = _lib.GbslnModel(m.nlay, m.nrow, m.ncol, _lib.dptr(keep["delr"]), _lib.dptr(keep["delc"]),
                             _lib.dptr(keep["top"]), _lib.dptr(keep["botm"]), _lib.dptr(keep["k11"]),
                             _lib.dptr(keep["k33"]), _lib.iptr(keep["ict"]), ss, sy,
                             int(m.chd_node.size), _lib.iptr(keep["chd_node"]), _lib.dptr(keep["chd_head"]),
                             int(m.wel_node.size), _lib.iptr(keep["wel_node"]), _lib.dptr(keep["wel_q"]),
                             int(m.rch_node.size), _lib.iptr(keep["rch_node"]), _lib.dptr(keep["rch_rate"]))
        npf = _lib.GbnpfOptions(int(m.inewton), int(m.ivarcv), int(m.idewatcv), int(m.icellavg),
                                satomega, 0, int(m.inewtonur))
        cs = ims.to_c(0)
        cnl = _lib.GbslnNonlinear(nl.dvclose, nl.mxiter, nl.nonmeth, nl.theta, nl.akappa, nl.gamma,
                                  nl.amomentum, nl.iallowptc, nl.numtrack, nl.btol, nl.breduc,
                                  nl.res_lim)
        self._h = C.c_void_p()
        ixt3d = int(getattr(m, "ixt3d", 0))
        # the conductivity tensor: XT3D, or K22/ANGLE2 in the standard form
        tensor = ixt3d != 0 or getattr(m, "k22", None) is not None or \
            getattr(m, "angle2", None) is not None
        if tensor:
            con = m.connections()
            if ixt3d == 1:
                from .xt3d import xt3d_pattern
                self._nja = int(xt3d_pattern(con["ia"], con["ja"])[1].size)

            def opt(name):
                v = getattr(m, name, None)
                if v is None:
                    return None
                keep["kt_" + name] = _f(v)
                return _lib.dptr(keep["kt_" + name])

            cx = _lib.GbslnKTensor(opt("k22"), opt("angle1"), opt("angle2"), opt("angle3"), ixt3d,
                                   int(getattr(m, "iavgkeff", 0)))
        if tensor and general:
            # the connection geometry: cell centres and face-normal angles
            disu = bool(getattr(m, "disu", False))
            if disu:
                xcn, ycn = m.xc, m.yc
            else:
                xcn, ycn = m.xcn, m.ycn
            keep.update(x_xc=_f(xcn), x_yc=_f(ycn), x_ax=_f(con["anglex"]))
            cg = _lib.GbslnGeometry(_lib.dptr(keep["x_xc"]), _lib.dptr(keep["x_yc"]),
                                    _lib.dptr(keep["x_ax"]), int(disu))
            rc = lib.gbsln_create_grid_tensor(C.byref(grid), C.byref(cm), C.byref(cx), C.byref(cg),
                                              C.byref(npf), C.byref(cs), C.byref(cnl),
                                              _lib.dptr(keep["strt"]), C.byref(self._h))
        elif tensor:
            rc = lib.gbsln_create_tensor(C.byref(cm), C.byref(cx), C.byref(npf), C.byref(cs),
                                         C.byref(cnl), _lib.dptr(keep["strt"]), C.byref(self._h))
        elif general:
            rc = lib.gbsln_create_grid(C.byref(grid), C.byref(cm), C.byref(npf), C.byref(cs),
                                       C.byref(cnl), _lib.dptr(keep["strt"]), C.byref(self._h))
        else:
            rc = lib.gbsln_create(C.byref(cm), C.byref(npf), C.byref(cs), C.byref(cnl),
                                  _lib.dptr(keep["strt"]), C.byref(self._h))
        if rc < 0:
            msg = lib.gbsln_last_error(self._h).decode() if self._h else ""
            lib.gbsln_destroy(self._h)
            self._h = C.c_void_p()
            raise _lib.GbimsError(rc, msg)
        self.nodes = m.nodes

    def timestep(self, kper: int = 1, kstp: int = 1, delt: float = 1.0, guess=None) -> dict:
        """One time step to closure.  `guess`: optional device address (int)
        of a float64 array of initial heads for the active cells (a warm
        start, gbsln_timestep_guess); the previous heads stay the storage
        reference."""
        lib = _lib.load()
        st = _lib.GbslnStats()
        if guess is None:
            rc = lib.gbsln_timestep(self._h, kper, kstp, delt, C.byref(st))
        else:
            rc = lib.gbsln_timestep_guess(self._h, kper, kstp, delt, C.c_void_p(guess), C.byref(st))
        if rc < 0:
            raise _lib.GbimsError(rc, lib.gbsln_last_error(self._h).decode())
        return {f: getattr(st, f) for f, _ in st._fields_}

    def formulate(self, delt: float = 0.0, hold: np.ndarray | None = None):
        """Assembled (amat, rhs) at the current heads, before the sln_ls fix-ups."""
        lib = _lib.load()
        nja = int(self.m.connections()["nja"]) if not hasattr(self, "_nja") else self._nja
        self._nja = nja
        amat = np.zeros(nja)
        rhs = np.zeros(self.nodes)
        hp = _lib.dptr(_f(hold)) if hold is not None else None
        if hold is not None:
            self._hold = _f(hold)
            hp = _lib.dptr(self._hold)
        rc = lib.gbsln_formulate(self._h, delt, hp, _lib.dptr(amat), _lib.dptr(rhs))
        if rc < 0:
            raise _lib.GbimsError(rc, lib.gbsln_last_error(self._h).decode())
        return amat, rhs

    BUDGET_ENTRIES = ("STO-SS", "STO-SY", "CHD", "WEL", "RCH")

    def budget_cells(self) -> dict:
        """The rates the packages save to the budget file for the last time
        step (gbsln_budget_cells): sto_ss and sto_sy per cell; chd, wel and
        rch per list entry."""
        lib = _lib.load()
        m = self.m
        out = dict(sto_ss=np.zeros(self.nodes), sto_sy=np.zeros(self.nodes),
                   chd=np.zeros(len(m.chd_node)), wel=np.zeros(len(m.wel_node)),
                   rch=np.zeros(len(m.rch_node)))
        rc = lib.gbsln_budget_cells(self._h, *[_lib.dptr(out[k]) for k in
                                               ("sto_ss", "sto_sy", "chd", "wel", "rch")])
        if rc < 0:
            raise _lib.GbimsError(rc, lib.gbsln_last_error(self._h).decode())
        return out

    def save_budget(self, path, name: str = "gwf", kstp: int = 1, kper: int = 1,
                    delt: float = 1.0, pertim: float = 1.0, totim: float = 1.0,
                    append: bool = False) -> None:
        """Writes the last time step's flows as MODFLOW 6's budget file does
        (OC SAVE BUDGET; mf6io.write_budget)."""
        from .mf6io import gwf_budget_records, write_budget
        fj, _ = self.budget(flowja=True)
        recs = gwf_budget_records(self.m, name, fj, self.budget_cells(), kstp, kper, delt,
                                  pertim, totim)
        write_budget(path, recs, append=append)

    def budget(self, flowja: bool = False):
        """Model budget of the last time step (gbsln_budget): rates in/out per
        entry, totals, percent discrepancy and the largest cell imbalance;
        with flowja=True also FLOW-JA-FACE (nja, CSR order)."""
        lib = _lib.load()
        t = _lib.GbslnBudgetTable()
        m = self.m
        if getattr(m, "disv", False) or getattr(m, "disu", False):
            nja = int(m.connections()["nja"])
        else:
            nja = m.nodes + 2 * (m.nlay * (m.nrow * (m.ncol - 1) + m.ncol * (m.nrow - 1))
                                 + (m.nlay - 1) * m.nrow * m.ncol)
        fj = np.zeros(nja) if flowja else None
        rc = lib.gbsln_budget(self._h, _lib.dptr(fj) if fj is not None else None, C.byref(t))
        if rc < 0:
            raise _lib.GbimsError(rc, lib.gbsln_last_error(self._h).decode())
        out = dict(rate_in=np.array(t.rate_in[:]), rate_out=np.array(t.rate_out[:]),
                   total_in=t.total_in, total_out=t.total_out,
                   percent_discrepancy=t.percent_discrepancy,
                   max_cell_imbalance=t.max_cell_imbalance, max_cell=t.max_cell)
        return (fj, out) if flowja else out

    @property
    def heads(self) -> np.ndarray:
        x = np.zeros(self.nodes)
        rc = _lib.load().gbsln_get_heads(self._h, _lib.dptr(x))
        if rc < 0:
            raise _lib.GbimsError(rc, "get_heads")
        return x

    @heads.setter
    def heads(self, x: np.ndarray):
        x = _f(x)
        rc = _lib.load().gbsln_set_heads(self._h, _lib.dptr(x))
        if rc < 0:
            raise _lib.GbimsError(rc, "set_heads")

    def restart(self):
        """Heads back to IC STRT on the device (gbsln_restart)."""
        rc = _lib.load().gbsln_restart(self._h)
        if rc < 0:
            raise _lib.GbimsError(rc, "restart")

    def ims_handle(self) -> C.c_void_p:
        return C.c_void_p(_lib.load().gbsln_ims(self._h))

    def close(self):
        if self._h:
            _lib.load().gbsln_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
