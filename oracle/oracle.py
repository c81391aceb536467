"""ctypes wrapper of the CPU oracle (oracle/ims_oracle.c, oracle/gwf_oracle.c).

TEST INFRASTRUCTURE ONLY: this module is the checker.  It is imported by
tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline and
reference legs, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import math
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build() -> Path:
    srcs = [HERE / f for f in ("ims_oracle.c", "gwf_oracle.c", "ims_oracle.h", "gwf_oracle.h", "Makefile")]
    if not LIB.exists() or LIB.stat().st_mtime < max(s.stat().st_mtime for s in srcs):
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


class Settings(C.Structure):
    _fields_ = [("dvclose", C.c_double), ("rclose", C.c_double), ("icnvgopt", C.c_int),
                ("iter1", C.c_int), ("ilinmeth", C.c_int), ("iscl", C.c_int), ("iord", C.c_int),
                ("north", C.c_int), ("relax", C.c_double), ("level", C.c_int),
                ("droptol", C.c_double)]


class CnvgRecord(C.Structure):
    _fields_ = [("dvmax", C.c_double), ("rmax", C.c_double), ("l2norm", C.c_double),
                ("alpha", C.c_double), ("beta", C.c_double), ("rho", C.c_double),
                ("omega", C.c_double), ("locdv", C.c_int), ("locr", C.c_int)]


class Models(C.Structure):
    _fields_ = [("nmod", C.c_int), ("modstart", _ip), ("dvmax", _dp), ("rmax", _dp),
                ("locdv", _ip), ("locr", _ip), ("loc", _ip)]


class GwfModel(C.Structure):
    _fields_ = [("nlay", C.c_int), ("nrow", C.c_int), ("ncol", C.c_int), ("nodes", C.c_int),
                ("nja", C.c_int), ("njas", C.c_int),
                ("ia", _ip), ("ja", _ip), ("isym", _ip), ("jas", _ip), ("ihc", _ip),
                ("cl1", _dp), ("cl2", _dp), ("hwva", _dp),
                ("top", _dp), ("bot", _dp), ("area", _dp), ("k11", _dp), ("k33", _dp),
                ("icelltype", _ip), ("inewton", C.c_int), ("ivarcv", C.c_int),
                ("idewatcv", C.c_int), ("icellavg", C.c_int), ("satomega", C.c_double),
                ("inewtonur", C.c_int), ("ss", _dp), ("sy", _dp), ("iconvert", _ip),
                ("nwel", C.c_int), ("wel_node", _ip), ("wel_q", _dp),
                ("nrch", C.c_int), ("rch_node", _ip), ("rch_rate", _dp),
                ("nchd", C.c_int), ("chd_node", _ip), ("chd_head", _dp),
                ("ixt3d", C.c_int), ("nozee", C.c_int), ("nja_sln", C.c_int), ("ck", _dp),
                ("sia", _ip), ("sja", _ip), ("idxglo", _ip),
                ("xt_grid", C.c_int), ("xc", _dp), ("yc", _dp), ("anglex", _dp), ("hy", _dp)]


class Nonlinear(C.Structure):
    _fields_ = [("dvclose", C.c_double), ("mxiter", C.c_int), ("nonmeth", C.c_int),
                ("iallowptc", C.c_int), ("theta", C.c_double), ("akappa", C.c_double),
                ("gamma", C.c_double), ("amomentum", C.c_double), ("bigch", C.c_double),
                ("bigchold", C.c_double), ("relaxold", C.c_double),
                ("wsave", _dp), ("hchold", _dp), ("deold", _dp), ("dxold", _dp),
                ("numtrack", C.c_int), ("btol", C.c_double), ("breduc", C.c_double),
                ("res_lim", C.c_double), ("res_prev", C.c_double), ("res_new", C.c_double)]


class TimestepStats(C.Structure):
    _fields_ = [("outer", C.c_int), ("inner_total", C.c_int), ("converged", C.c_int),
                ("pivot_retries", C.c_int), ("last_dxmax", C.c_double), ("backtracks", C.c_int)]


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        lib.or_ims_create.restype = C.c_void_p
        lib.or_ims_create.argtypes = [C.POINTER(Settings), C.c_int, C.c_int, _ip, _ip]
        lib.or_ims_destroy.argtypes = [C.c_void_p]
        lib.or_ims_apply.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_int, C.c_int, _ip, _ip,
                                     C.POINTER(CnvgRecord), C.c_int]
        lib.or_ims_apc.restype = _dp
        lib.or_ims_apc.argtypes = [C.c_void_p]
        lib.or_ims_iapc.restype = _ip
        lib.or_ims_iapc.argtypes = [C.c_void_p]
        lib.or_ims_japc.restype = _ip
        lib.or_ims_japc.argtypes = [C.c_void_p]
        lib.or_ims_l2norm0.restype = C.c_double
        lib.or_ims_l2norm0.argtypes = [C.c_void_p]
        lib.or_ims_pivot_retries.argtypes = [C.c_void_p]
        lib.or_ims_njapc.argtypes = [C.c_void_p]
        lib.or_ims_ilut_ierr.argtypes = [C.c_void_p]
        lib.or_ilut_iwk.argtypes = [C.c_int, _ip, C.c_int]
        lib.or_genrcm.argtypes = [C.c_int, _ip, _ip, _ip]
        lib.or_genmd.argtypes = [C.c_int, _ip, _ip, _ip]
        lib.or_dperm.argtypes = [C.c_int, _dp, _ip, _ip, _dp, _ip, _ip, _ip]
        lib.or_pcu_ilut.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, _dp, _ip, _ip, _dp,
                                    _ip, _ip, C.c_int, _dp, _ip, _ip]
        lib.or_amux.argtypes = [C.c_int, _dp, _dp, _dp, _ip, _ip]
        lib.or_ims_set_models.argtypes = [C.c_void_p, C.c_void_p]
        lib.or_ilu0a.argtypes = [C.c_int, C.c_int, _dp, _ip, _ip, _dp, _dp]
        lib.or_amux_fma.argtypes = [C.c_int, _dp, _dp, _dp, _ip, _ip]
        lib.or_ilu0a_fma.argtypes = [C.c_int, _dp, _ip, _ip, _dp, _dp]
        lib.or_pccrs.argtypes = [C.c_int, C.c_int, _ip, _ip, _ip, _ip]
        lib.or_pcu.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, _dp, _ip, _ip, _dp, _ip, _ip, _ip, _dp]
        lib.or_dnrm2.restype = C.c_double
        lib.or_dnrm2.argtypes = [C.c_int, _dp]
        lib.or_ddot.restype = C.c_double
        lib.or_ddot.argtypes = [C.c_int, _dp, _dp]
        lib.or_epfact.restype = C.c_double
        lib.or_epfact.argtypes = [C.c_int, C.c_int]
        lib.or_is_close.argtypes = [C.c_double, C.c_double]
        lib.or_squadratic_sat.restype = C.c_double
        lib.or_squadratic_sat.argtypes = [C.c_double] * 4
        lib.or_squadratic_sat_derv.restype = C.c_double
        lib.or_squadratic_sat_derv.argtypes = [C.c_double] * 4
        lib.or_dis_sizes.argtypes = [C.c_int, C.c_int, C.c_int, _ip, _ip, _ip]
        lib.or_disv_connect.argtypes = [C.c_int, C.c_int, _dp, _dp, _ip, _ip, _dp, _dp, _dp, _dp,
                                        _ip, C.c_int, _ip, _ip, _ip, _ip, _ip, _dp, _dp, _dp, _dp]
        lib.or_dis_connect.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _ip, _ip, _ip,
                                       _ip, _ip, _dp, _dp, _dp]
        lib.or_xt3d_ck.argtypes = [C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, C.c_int, _dp]
        lib.or_xt3d_pattern.argtypes = [C.c_int, _ip, _ip, C.c_int, _ip, _ip, _ip]
        lib.or_xt3d_fc.argtypes = [C.POINTER(GwfModel), _ip, _dp, _dp, _dp, _dp, _dp]
        lib.or_xt3d_flowja.argtypes = [C.POINTER(GwfModel), _ip, _dp, _dp, _dp]
        lib.or_xt3d_fn.argtypes = [C.POINTER(GwfModel), _ip, _dp, _dp, _dp, _dp]
        lib.or_disu_connect.argtypes = [C.c_int, _ip, _ip, _ip, _dp, _dp, _dp, _ip, C.c_int, _ip,
                                        _ip, _ip, _ip, _ip, _ip, _dp, _dp, _dp, _dp]
        lib.or_npf_hy.argtypes = [C.POINTER(GwfModel), _dp, _dp, _dp, _dp, C.c_int, _dp]
        lib.or_disv_anglex.argtypes = [C.c_int, C.c_int, _dp, _dp, _ip, _ip, _ip, _ip, _ip, _ip,
                                       _ip, _dp]
        lib.or_npf_condsat.argtypes = [C.POINTER(GwfModel), _dp]
        lib.or_gwf_fc.argtypes = [C.POINTER(GwfModel), _ip, _dp, _dp, C.c_double, C.c_int, _dp, _dp, _dp, _dp]
        lib.or_sln_ls_fixups.argtypes = [C.c_int, _ip, _ip, _ip, C.c_int, _dp, _dp, _dp, _dp]
        lib.or_npf_cf.argtypes = [C.POINTER(GwfModel), _ip, _dp, _dp]
        lib.or_gwf_budget.argtypes = [C.POINTER(GwfModel), _ip, _dp, _dp, C.c_double, C.c_int, _dp,
                                      _dp, _dp, _dp]
        lib.or_gwf_timestep.argtypes = [C.POINTER(GwfModel), C.c_void_p, C.POINTER(Nonlinear), _dp, _ip,
                                        C.c_int, C.c_int, C.c_double, C.c_int, _dp, _dp,
                                        C.POINTER(TimestepStats)]
        _lib = lib
    return _lib


def dp(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous, (a.dtype, a.flags)
    return a.ctypes.data_as(_dp)


def ip(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous, (a.dtype, a.flags)
    return a.ctypes.data_as(_ip)


def settings(dvclose=1e-3, rclose=1e-1, icnvgopt=0, iter1=50, ilinmeth=1, iscl=0, iord=0,
             north=0, relax=0.0, level=0, droptol=0.0) -> Settings:
    return Settings(dvclose, rclose, icnvgopt, iter1, ilinmeth, iscl, iord, north, relax, level, droptol)


class Ims:
    """Oracle ImsLinearDataType (allocate / apply) for one matrix structure."""

    def __init__(self, s: Settings, ia: np.ndarray, ja: np.ndarray):
        self.lib = load()
        self.ia = np.ascontiguousarray(ia, np.int32)
        self.ja = np.ascontiguousarray(ja, np.int32)
        self.neq = self.ia.size - 1
        self.nja = self.ja.size
        self.s = s
        self.h = self.lib.or_ims_create(C.byref(s), self.neq, self.nja, ip(self.ia), ip(self.ja))

    def apply(self, amat, rhs, x, kstp=1, kiter=1, nrec=0):
        icnvg, in_iter = C.c_int(0), C.c_int(0)
        rec = (CnvgRecord * max(nrec, 1))()
        rc = self.lib.or_ims_apply(self.h, dp(amat), dp(rhs), dp(x), kstp, kiter, C.byref(icnvg),
                                   C.byref(in_iter), rec if nrec else None, nrec)
        if rc == -4:
            raise RuntimeError(f"oracle ilut failed: ierr {self.lib.or_ims_ilut_ierr(self.h)}")
        if rc != 0:
            raise RuntimeError(f"oracle apply failed: {rc}")
        recs = [{f: getattr(rec[i], f) for f, _ in CnvgRecord._fields_} for i in range(min(nrec, in_iter.value))]
        return icnvg.value, in_iter.value, recs

    def set_models(self, modstart, nrec):
        """Per-model records (CONVMODSTART, 0-based first rows ending at neq)
        for the next applies with nrec records; read them with model_records."""
        ms = np.ascontiguousarray(modstart, np.int32)
        nm = ms.size - 1
        self._mods = dict(ms=ms, dvmax=np.zeros(nrec * nm), rmax=np.zeros(nrec * nm),
                          locdv=np.zeros(nrec * nm, np.int32), locr=np.zeros(nrec * nm, np.int32),
                          loc=np.full(2 * nm, -1, np.int32), nm=nm)
        m = self._mods
        self._mstruct = Models(nm, ip(ms), dp(m["dvmax"]), dp(m["rmax"]), ip(m["locdv"]),
                               ip(m["locr"]), ip(m["loc"]))
        self.lib.or_ims_set_models(self.h, C.byref(self._mstruct))

    def model_records(self, nrec):
        m = self._mods
        nm = m["nm"]
        return {k: m[k][:nrec * nm].reshape(nrec, nm) for k in ("dvmax", "locdv", "rmax", "locr")}

    def apc(self) -> np.ndarray:
        n = self.lib.or_ims_njapc(self.h)
        return np.ctypeslib.as_array(self.lib.or_ims_apc(self.h), shape=(n,)).copy()

    def iapc(self) -> np.ndarray:
        return np.ctypeslib.as_array(self.lib.or_ims_iapc(self.h), shape=(self.neq + 1,)).copy()

    def japc(self) -> np.ndarray:
        n = self.lib.or_ims_njapc(self.h)
        return np.ctypeslib.as_array(self.lib.or_ims_japc(self.h), shape=(n,)).copy()

    def factor(self):
        """The preconditioner after the last apply as (iapc, japc, apc), cut
        to the storage in use (ILUT: positions up to iapc[neq])."""
        iapc = self.iapc()
        used = int(iapc[-1]) if self.lib.or_ims_ipc(self.h) >= 3 else self.nja
        return iapc, self.japc()[:used], self.apc()[:used]

    def l2norm0(self) -> float:
        return self.lib.or_ims_l2norm0(self.h)

    def pivot_retries(self) -> int:
        return self.lib.or_ims_pivot_retries(self.h)

    def __del__(self):
        try:
            self.lib.or_ims_destroy(self.h)
        except Exception:
            pass


def ilut(ia, ja, amat, level, droptol, relax=0.0):
    """ims_base_pcu with ILUT/MILUT (sparskit2/ilut.f90) on one matrix:
    returns (iapc, japc, apc, retries), storage cut to iapc[neq]."""
    lib = load()
    ia = np.ascontiguousarray(ia, np.int32)
    ja = np.ascontiguousarray(ja, np.int32)
    n = ia.size - 1
    iwk = lib.or_ilut_iwk(n, ip(ia), level)
    cap = max(iwk, n + 1)
    alu, japc = np.zeros(cap), np.zeros(cap, np.int32)
    iapc = np.zeros(n + 1, np.int32)
    w, jw, jr = np.zeros(n), np.zeros(n, np.int32), np.zeros(n, np.int32)
    rc = lib.or_pcu_ilut(n, level, droptol, relax, dp(np.ascontiguousarray(amat, float)), ip(ia),
                         ip(ja), dp(alu), ip(iapc), ip(japc), iwk, dp(w), ip(jw), ip(jr))
    if rc < 0:
        raise RuntimeError(f"oracle ilut failed: ierr {rc}")
    used = int(iapc[-1])
    return iapc, japc[:used], alu[:used], rc


def genrcm(ia, ja):
    """LORDER of REORDERING_METHOD RCM (rcm.f90 genrcm on the IMS pattern,
    0-based): lorder[i] is the i-th node of the RCM numbering."""
    lib = load()
    ia = np.ascontiguousarray(ia, np.int32)
    ja = np.ascontiguousarray(ja, np.int32)
    lorder = np.zeros(ia.size - 1, np.int32)
    lib.or_genrcm(ia.size - 1, ip(ia), ip(ja), ip(lorder))
    return lorder


def genmd(ia, ja):
    """LORDER of REORDERING_METHOD MD (ImsReordering.f90 odrv/md on the IMS
    pattern, 0-based): lorder[i] is the i-th eliminated node."""
    lib = load()
    ia = np.ascontiguousarray(ia, np.int32)
    ja = np.ascontiguousarray(ja, np.int32)
    lorder = np.zeros(ia.size - 1, np.int32)
    flag = lib.or_genmd(ia.size - 1, ip(ia), ip(ja), ip(lorder))
    if flag != 0:
        raise RuntimeError(f"oracle md failed: flag {flag}")
    return lorder


def dperm(ia, ja, a, perm):
    """sparsekit dperm (job 1): row j of A becomes row perm[j], columns
    relabelled by perm, entries kept in order."""
    lib = load()
    ia = np.ascontiguousarray(ia, np.int32)
    ja = np.ascontiguousarray(ja, np.int32)
    perm = np.ascontiguousarray(perm, np.int32)
    iao, jao, ao = np.zeros_like(ia), np.zeros_like(ja), np.zeros(ja.size)
    lib.or_dperm(ia.size - 1, dp(np.ascontiguousarray(a, float)), ip(ja), ip(ia), dp(ao), ip(jao),
                 ip(iao), ip(perm))
    return iao, jao, ao


def amux(ia, ja, a, x):
    lib = load()
    y = np.zeros(ia.size - 1)
    lib.or_amux(ia.size - 1, dp(x), dp(y), dp(a), ip(ja), ip(ia))
    return y


def amux_fma(ia, ja, a, x):
    lib = load()
    y = np.zeros(ia.size - 1)
    lib.or_amux_fma(ia.size - 1, dp(x), dp(y), dp(a), ip(ja), ip(ia))
    return y


def ilu0a(apc, iapc, japc, r, fma=False):
    lib = load()
    d = np.zeros(iapc.size - 1)
    if fma:
        lib.or_ilu0a_fma(iapc.size - 1, dp(apc), ip(iapc), ip(japc), dp(r), dp(d))
    else:
        lib.or_ilu0a(apc.size, iapc.size - 1, dp(apc), ip(iapc), ip(japc), dp(r), dp(d))
    return d


def dis_connect(nlay, nrow, ncol, delr, delc, top, bot) -> dict:
    lib = load()
    nodes, nja, njas = C.c_int(), C.c_int(), C.c_int()
    lib.or_dis_sizes(nlay, nrow, ncol, C.byref(nodes), C.byref(nja), C.byref(njas))
    n, nz, ns = nodes.value, nja.value, njas.value
    out = dict(ia=np.zeros(n + 1, np.int32), ja=np.zeros(nz, np.int32), isym=np.zeros(nz, np.int32),
               jas=np.zeros(nz, np.int32), ihc=np.zeros(ns, np.int32), cl1=np.zeros(ns),
               cl2=np.zeros(ns), hwva=np.zeros(ns))
    lib.or_dis_connect(nlay, nrow, ncol, dp(np.ascontiguousarray(delr, float)),
                       dp(np.ascontiguousarray(delc, float)), dp(np.ascontiguousarray(top, float)),
                       dp(np.ascontiguousarray(bot, float)), ip(out["ia"]), ip(out["ja"]),
                       ip(out["isym"]), ip(out["jas"]), ip(out["ihc"]), dp(out["cl1"]),
                       dp(out["cl2"]), dp(out["hwva"]))
    out.update(nodes=n, nja=nz, njas=ns)
    return out


def disv_connect(nlay, iavert, javert, vx, vy, xc, yc, top, bot, idomain=None) -> dict:
    """or_disv_connect: the connectivity of a DISV grid (closed vertex lists
    iavert/javert, 0-based; top/bot per user cell) reduced by IDOMAIN
    (> 0 active, 0 removed, < 0 vertical pass-through), with the cell
    areas."""
    lib = load()
    iavert = np.ascontiguousarray(iavert, np.int32)
    javert = np.ascontiguousarray(javert, np.int32)
    ncpl = iavert.size - 1
    red = None
    n = nlay * ncpl
    if idomain is not None:
        idomain = np.asarray(idomain)
        red = np.where(idomain < 0, -1, 0).astype(np.int32)
        act = idomain > 0
        red[act] = np.arange(1, int(act.sum()) + 1, dtype=np.int32)
        n = int(act.sum())
    cap = n * (3 + int(np.diff(iavert).max()))
    out = dict(ia=np.zeros(n + 1, np.int32), ja=np.zeros(cap, np.int32), isym=np.zeros(cap, np.int32),
               jas=np.zeros(cap, np.int32), ihc=np.zeros(cap, np.int32), cl1=np.zeros(cap),
               cl2=np.zeros(cap), hwva=np.zeros(cap), area=np.zeros(ncpl))
    f = lambda a: np.ascontiguousarray(a, np.float64)
    keep = [f(vx), f(vy), f(xc), f(yc), f(top), f(bot)]
    nja = lib.or_disv_connect(nlay, ncpl, dp(keep[0]), dp(keep[1]), ip(iavert), ip(javert),
                              dp(keep[2]), dp(keep[3]), dp(keep[4]), dp(keep[5]),
                              ip(red) if red is not None else None, cap,
                              ip(out["ia"]), ip(out["ja"]), ip(out["isym"]), ip(out["jas"]),
                              ip(out["ihc"]), dp(out["cl1"]), dp(out["cl2"]), dp(out["hwva"]),
                              dp(out["area"]))
    if nja < 0:
        raise RuntimeError("or_disv_connect: capacity exceeded")
    njas = (nja - n) // 2
    for k in ("ja", "isym", "jas"):
        out[k] = out[k][:nja].copy()
    for k in ("ihc", "cl1", "cl2", "hwva"):
        out[k] = out[k][:njas].copy()
    out.update(nodes=n, nja=nja, njas=njas)
    return out


DISU_ERRORS = {-1: "capacity exceeded", -2: "diagonal not first", -3: "row not ascending",
               -4: "no symmetric counterpart", -5: "IHC not symmetric",
               -6: "HWVA not symmetric", -7: "IHC outside 0..2", -8: "no active cell"}


def disu_connect(iac, ja, ihc, cl12, hwva, idomain=None, angldegx=None) -> dict:
    """or_disu_connect: the connectivity of a DISU grid from its input arrays
    (JA 1-based), reduced to the cells with IDOMAIN > 0, with anglex
    (radians, per connection n < m) when ANGLDEGX is given.  Raises
    ValueError with the failing check."""
    lib = load()
    iac = np.asarray(iac, np.int64)
    nu = iac.size
    iainp = np.zeros(nu + 1, np.int32)
    iainp[1:] = np.cumsum(iac)
    f = lambda a: np.ascontiguousarray(a, np.float64)
    jainp = np.ascontiguousarray(ja, np.int32)
    ihcinp = np.ascontiguousarray(ihc, np.int32)
    cl12inp, hwvainp = f(cl12), f(hwva)
    red = None
    if idomain is not None:
        keep = np.asarray(idomain) > 0
        red = np.full(nu, -1, np.int32)
        red[keep] = np.arange(int(keep.sum()), dtype=np.int32)
    cap = int(iainp[-1])
    n = C.c_int()
    out = dict(ia=np.zeros(nu + 1, np.int32), ja=np.zeros(cap, np.int32), isym=np.zeros(cap, np.int32),
               jas=np.zeros(cap, np.int32), ihc=np.zeros(cap, np.int32), cl1=np.zeros(cap),
               cl2=np.zeros(cap), hwva=np.zeros(cap), anglex=np.zeros(cap))
    ang = f(angldegx) if angldegx is not None else None
    nja = lib.or_disu_connect(nu, ip(iainp), ip(jainp), ip(ihcinp), dp(cl12inp), dp(hwvainp),
                              dp(ang) if ang is not None else None,
                              ip(red) if red is not None else None, cap, C.byref(n),
                              ip(out["ia"]), ip(out["ja"]), ip(out["isym"]), ip(out["jas"]),
                              ip(out["ihc"]), dp(out["cl1"]), dp(out["cl2"]), dp(out["hwva"]),
                              dp(out["anglex"]))
    if nja < 0:
        raise ValueError("or_disu_connect: " + DISU_ERRORS.get(nja, str(nja)))
    nodes = n.value
    njas = (nja - nodes) // 2
    out["ia"] = out["ia"][:nodes + 1].copy()
    for k in ("ja", "isym", "jas"):
        out[k] = out[k][:nja].copy()
    for k in ("ihc", "cl1", "cl2", "hwva", "anglex"):
        out[k] = out[k][:njas].copy()
    out.update(nodes=nodes, nja=nja, njas=njas)
    return out


class Gwf:
    """Oracle GWF model + NumericalSolution for one DIS model (a GwfDisModel),
    one DISV model (a DisvModel: connectivity from or_disv_connect) or one
    DISU model (a DisuModel: connectivity from or_disu_connect)."""

    def __init__(self, m, ims_settings: Settings, satomega=1.0e-6):
        self.lib = load()
        self.m = m
        if getattr(m, "disu", False):
            con = disu_connect(m.iac, m.ja, m.ihc_u, m.cl12, m.hwva_u, m.idomain,
                               getattr(m, "angldegx", None))
            area = m.area
        elif getattr(m, "disv", False):
            iav, jav = m.vertex_lists
            con = disv_connect(m.nlay, iav, jav, m.vertices[:, 0], m.vertices[:, 1], m.xc, m.yc,
                               m.user_top, m.botm, getattr(m, "idomain", None))
            area = np.tile(con["area"], m.nlay)[m.nodeuser]
        else:
            con = dis_connect(m.nlay, m.nrow, m.ncol, m.delr, m.delc, m.cell_top, m.cell_bot)
            area = m.area
        self.con = con
        keep = {}

        def d(a):
            a = np.ascontiguousarray(a, np.float64)
            keep[id(a)] = a
            return dp(a)

        def i(a):
            a = np.ascontiguousarray(a, np.int32)
            keep[id(a)] = a
            return ip(a)

        n = m.nodes
        ss = m.ss if m.ss is not None else np.zeros(n)
        sy = m.sy if m.sy is not None else np.zeros(n)
        self.model = GwfModel(
            m.nlay, m.nrow, m.ncol, n, con["nja"], con["njas"],
            i(con["ia"]), i(con["ja"]), i(con["isym"]), i(con["jas"]), i(con["ihc"]),
            d(con["cl1"]), d(con["cl2"]), d(con["hwva"]),
            d(m.cell_top), d(m.cell_bot), d(area), d(m.k11), d(m.k33), i(m.icelltype),
            int(m.inewton), int(getattr(m, "ivarcv", 0)), int(getattr(m, "idewatcv", 0)),
            int(getattr(m, "icellavg", 0)), satomega, int(getattr(m, "inewtonur", 0)),
            d(ss), d(sy), i(m.icelltype),
            int(m.wel_node.size), i(m.wel_node), d(m.wel_q),
            int(m.rch_node.size), i(m.rch_node), d(m.rch_rate),
            int(m.chd_node.size), i(m.chd_node), d(m.chd_head))
        self.mcon = con
        general = getattr(m, "disv", False) or getattr(m, "disu", False)
        dpio180 = math.atan(1.0) / 45.0
        rad = lambda a: (None if a is None else np.asarray(a, float) * dpio180)
        if general and (int(getattr(m, "ixt3d", 0)) or getattr(m, "k22", None) is not None
                        or getattr(m, "angle2", None) is not None):
            # the connection geometry: DISV, the shared edges' normal angles
            # (cprops); DISU, ANGLDEGX
            if getattr(m, "disv", False):
                iav, jav = m.vertex_lists
                ax = np.zeros(con["njas"])
                self.lib.or_disv_anglex(m.nodes, len(m.icvert), d(m.vertices[:, 0]),
                                        d(m.vertices[:, 1]), i(iav), i(jav), i(m.nodeuser),
                                        i(con["ia"]), i(con["ja"]), i(con["jas"]), i(con["ihc"]),
                                        dp(ax))
                xcn, ycn = m.xcn, m.ycn
                self.model.xt_grid = 1
            else:
                ax = con["anglex"]
                xcn, ycn = m.xc, m.yc
                self.model.xt_grid = 2
            self.model.xc, self.model.yc, self.model.anglex = d(xcn), d(ycn), d(ax)
            con = dict(con, anglex=ax)
        if not int(getattr(m, "ixt3d", 0)) and (getattr(m, "k22", None) is not None
                                                or getattr(m, "angle2", None) is not None):
            # hy_eff per connection (K22 and the angles, standard formulation)
            hy = np.zeros(2 * con["njas"])
            opt = lambda a: d(a) if a is not None else None
            self.lib.or_npf_hy(C.byref(self.model), opt(getattr(m, "k22", None)),
                               opt(rad(getattr(m, "angle1", None))), opt(rad(getattr(m, "angle2", None))),
                               opt(rad(getattr(m, "angle3", None))), int(getattr(m, "iavgkeff", 0)),
                               dp(hy))
            self.model.hy = d(hy)
            con = dict(con, hy=hy)
        if int(getattr(m, "ixt3d", 0)):
            # XT3D on a DIS grid: the tensor per cell and the wider pattern
            nozee = m.angle2 is None
            radz = lambda a: (np.zeros(n) if a is None else np.asarray(a, float) * dpio180)
            k22 = m.k11 if m.k22 is None else m.k22
            ck = np.zeros(9 * n)
            self.lib.or_xt3d_ck(n, d(m.k11), d(k22), d(m.k33), d(radz(m.angle1)), d(radz(m.angle2)),
                                d(radz(m.angle3)), int(nozee), dp(ck))
            ixt3d = int(m.ixt3d)
            if ixt3d == 2:
                # XT3D RHS: the model's own pattern
                sia = np.ascontiguousarray(con["ia"], np.int32)
                sja = np.ascontiguousarray(con["ja"], np.int32)
                idxglo = np.arange(con["nja"], dtype=np.int32)
                nja_sln = int(con["nja"])
            else:
                cap = int(np.diff(con["ia"])[con["ja"]].sum()) + n
                sia = np.zeros(n + 1, np.int32)
                sja = np.zeros(cap, np.int32)
                idxglo = np.zeros(con["nja"], np.int32)
                nja_sln = self.lib.or_xt3d_pattern(n, i(con["ia"]), i(con["ja"]), cap, ip(sia),
                                                   ip(sja), ip(idxglo))
                if nja_sln < 0:
                    raise RuntimeError("or_xt3d_pattern: capacity exceeded")
                sja = sja[:nja_sln].copy()
            self.model.ixt3d, self.model.nozee, self.model.nja_sln = ixt3d, int(nozee), nja_sln
            self.model.ck, self.model.sia, self.model.sja, self.model.idxglo = d(ck), i(sia), i(sja), i(idxglo)
            con = dict(con, ia=sia, ja=sja, nja=nja_sln, idxglo=idxglo, ck=ck)
        self.con = con
        self._keep = keep
        self.condsat = np.zeros(con["njas"])
        self.lib.or_npf_condsat(C.byref(self.model), dp(self.condsat))
        self.ibound = np.ascontiguousarray(m.ibound, np.int32)
        self.ims = Ims(ims_settings, con["ia"], con["ja"])
        self.x = np.ascontiguousarray(m.strt, np.float64).copy()
        self.xold = self.x.copy()
        self._nlv = [np.zeros(n) for _ in range(4)]

    def assemble(self, hnew, hold=None, delt=0.0, transient=False):
        """gwf_fc into a zeroed amat/rhs (before the sln_ls fix-ups)."""
        n, nja = self.m.nodes, self.con["nja"]
        amat = np.zeros(nja)
        rhs = np.zeros(n)
        sat = np.ones(n)  # npf_ar's initial saturation; npf_cf updates convertible cells
        hnew = np.ascontiguousarray(hnew, np.float64)
        hold = np.ascontiguousarray(hnew if hold is None else hold, np.float64)
        self.lib.or_gwf_fc(C.byref(self.model), ip(self.ibound), dp(self.condsat), dp(sat), delt,
                           int(transient), dp(hold), dp(hnew), dp(amat), dp(rhs))
        return amat, rhs

    def fixups(self, amat, rhs, x, isymmetric=True):
        xtemp = np.zeros_like(x)
        self.lib.or_sln_ls_fixups(x.size, ip(self.con["ia"]), ip(self.con["ja"]), ip(self.ibound),
                                  int(isymmetric), dp(amat), dp(rhs), dp(x), dp(xtemp))
        return amat, rhs

    def sat(self, hnew):
        """npf_cf: cell saturation at the given heads."""
        s = np.ones(self.m.nodes)
        h = np.ascontiguousarray(hnew, np.float64)
        self.lib.or_npf_cf(C.byref(self.model), ip(self.ibound), dp(h), dp(s))
        return s

    def budget(self, hnew, hold=None, delt=0.0, transient=False, sat=None):
        """gwf_cq + gwf_bd (or_gwf_budget): FLOW-JA-FACE and the model budget
        (entries STO-SS, STO-SY, CHD, WEL, RCH; totals and percent difference
        summed in entry order, Budget.f90:250-266).  sat defaults to npf_cf at
        hnew."""
        hnew = np.ascontiguousarray(hnew, np.float64)
        hold = np.ascontiguousarray(hnew if hold is None else hold, np.float64)
        sat = self.sat(hnew) if sat is None else np.ascontiguousarray(sat, np.float64)
        flowja = np.zeros(self.mcon["nja"])
        terms = np.zeros(10)
        self.lib.or_gwf_budget(C.byref(self.model), ip(self.ibound), dp(self.condsat), dp(sat), delt,
                               int(transient), dp(hold), dp(hnew), dp(flowja), dp(terms))
        rin, rout = terms[0::2].copy(), terms[1::2].copy()
        tin = tout = 0.0
        for k in range(5):
            tin += rin[k]
            tout += rout[k]
        avg = (tin + tout) / 2.0
        pd = 100.0 * (tin - tout) / avg if avg != 0.0 else 0.0
        act = self.ibound > 0
        diag = flowja[self.mcon["ia"][:-1]]
        imb = np.abs(np.where(act, diag, 0.0))
        return flowja, dict(rate_in=rin, rate_out=rout, total_in=tin, total_out=tout,
                            percent_discrepancy=pd, max_cell_imbalance=float(imb.max()),
                            max_cell=int(imb.argmax()) if imb.max() > 0 else -1)

    def timestep(self, kper=1, kstp=1, delt=1.0, transient=False, dvclose=1e-3, mxiter=25,
                 nonmeth=0, theta=1.0, akappa=0.0, gamma=1.0, amomentum=0.0, iallowptc=1,
                 numtrack=0, btol=0.0, breduc=0.0, res_lim=0.0):
        w = self._nlv
        nl = Nonlinear(dvclose, mxiter, nonmeth, iallowptc, theta, akappa, gamma, amomentum,
                       0.0, 0.0, 0.0, dp(w[0]), dp(w[1]), dp(w[2]), dp(w[3]),
                       numtrack, btol, breduc, res_lim, 0.0, 0.0)
        st = TimestepStats()
        rc = self.lib.or_gwf_timestep(C.byref(self.model), self.ims.h, C.byref(nl), dp(self.condsat),
                                      ip(self.ibound), kper, kstp, delt, int(transient), dp(self.x),
                                      dp(self.xold), C.byref(st))
        if rc != 0:
            raise RuntimeError(f"oracle timestep failed: {rc}")
        return {f: getattr(st, f) for f, _ in TimestepStats._fields_}
