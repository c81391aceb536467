"""Batched ensembles: many independent GWF DIS models solved together by one
batched IMS (gbims_batch_* C ABI).

MODFLOW 6 solves ensemble members one simulation at a time.  Here the
members' systems are concatenated into one block-diagonal system; every
kernel of the PCG iteration runs once for all members, each member keeps its
own Krylov scalars and closure test (its own ImsLinearBase.f90:30-240
iteration), and a member that has converged drops out while the others go on.

`make_ensemble` builds the seeded 256-member workload (nx, ny ~ U{50..450},
nlay ~ U{1..5}, sigma_lnK ~ U(0.5, 2), per-member west/east CHD heads);
`assemble_member` fills a member's system with the GPU NPF kernels
(gbnpf_fill) and the sln_ls fix-ups; `EnsembleLinear` is the batched
counterpart of ImsLinear.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .dis import GwfDisModel, _faces_chd, lognormal_field
from .ims import ApplyResult, ImsLinearSettings, _summary
from .solution import sln_ls_fixups


def make_ensemble(count: int = 256, seed: int = 0, scale: float = 1.0) -> list[GwfDisModel]:
    """Member i is drawn from numpy.random.default_rng(seed + i): confined
    steady state, 10 m layers, delr = delc = 10 m, Kh lognormal with its own
    sigma (10-cell correlation), Kv = 0.1 Kh, CHD heads U(10, 20) m on the
    west face and U(0, 10) m on the east face.  `scale` < 1 shrinks nrow and
    ncol for CPU-sized test ensembles."""
    members = []
    for i in range(count):
        rng = np.random.default_rng(seed + i)
        nrow, ncol = (max(3, int(round(int(v) * scale))) for v in rng.integers(50, 451, size=2))
        nlay = int(rng.integers(1, 6))
        sigma = float(rng.uniform(0.5, 2.0))
        hw, he = float(rng.uniform(10.0, 20.0)), float(rng.uniform(0.0, 10.0))
        nrc = nrow * ncol
        top = np.full(nrc, 10.0 * nlay)
        botm = np.repeat(10.0 * nlay - 10.0 * np.arange(1, nlay + 1), nrc)
        corr = max(1.0, 10.0 * scale) if scale < 1 else 10.0
        kh = np.concatenate([lognormal_field(rng, (nrow, ncol), sigma, corr).ravel()
                             for _ in range(nlay)])
        m = GwfDisModel(nlay, nrow, ncol, np.full(ncol, 10.0), np.full(nrow, 10.0), top, botm,
                        kh, 0.1 * kh, np.zeros(nlay * nrc, np.int32),
                        np.full(nlay * nrc, 0.5 * (hw + he)), name=f"c4-{seed + i}")
        m.chd_node, m.chd_head = _faces_chd(nlay, nrow, ncol, hw, he)
        members.append(m)
    return members


def initial_heads(m: GwfDisModel) -> np.ndarray:
    x = m.strt.copy()
    x[m.chd_node] = m.chd_head
    return x


def assemble_member(m: GwfDisModel):
    """The member's linear system as sln_ls hands it to IMS: the NPF fill
    (npf_fc on the device, gbnpf_fill) at the initial heads, then the sln_ls
    fix-ups (CHD rows, symmetric form for CG).  Returns (con, amat, rhs, x0);
    CHD and NPF are the only packages of an ensemble member."""
    import torch

    lib = _lib.load()
    con = m.connections()
    ip = lambda a: np.ascontiguousarray(a, dtype=np.int32).ctypes.data_as(C.POINTER(C.c_int))
    dp = lambda a: np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.POINTER(C.c_double))
    opt = _lib.GbnpfOptions(0, 0, 0, 0, 1.0e-6, 0)
    h = C.c_void_p()
    top, bot = m.cell_top, m.cell_bot
    rc = lib.gbnpf_create(C.byref(opt), m.nodes, con["nja"], con["njas"], ip(con["ia"]),
                          ip(con["ja"]), ip(con["jas"]), ip(con["isym"]), ip(con["ihc"]),
                          dp(con["cl1"]), dp(con["cl2"]), dp(con["hwva"]), dp(top), dp(bot),
                          dp(m.k11), dp(m.k33), ip(m.icelltype), C.byref(h))
    if rc != 0:
        raise _lib.GbimsError(rc, "gbnpf_create failed")
    try:
        x0 = initial_heads(m)
        dev = torch.device("cuda")
        d_amat = torch.zeros(con["nja"], dtype=torch.float64, device=dev)
        d_rhs = torch.zeros(m.nodes, dtype=torch.float64, device=dev)
        d_ib = torch.from_numpy(m.ibound).to(dev)
        d_h = torch.from_numpy(x0).to(dev)
        torch.cuda.synchronize()
        rc = lib.gbnpf_fill(h, d_ib.data_ptr(), d_h.data_ptr(), d_amat.data_ptr(), d_rhs.data_ptr())
        if rc != 0:
            raise _lib.GbimsError(rc, "gbnpf_fill failed")
        amat, rhs = d_amat.cpu().numpy(), d_rhs.cpu().numpy()
    finally:
        lib.gbnpf_destroy(h)
    amat, rhs = sln_ls_fixups(con["ia"], con["ja"], m.ibound, amat, rhs, x0, isymmetric=True)
    return con, amat, rhs, x0


def concat_systems(cons, amats=None, rhss=None, xs=None):
    """Block-diagonal concatenation: member row offsets (nm + 1) and the
    0-based global CSR (ia, ja), plus the concatenated values if given."""
    mrow = np.zeros(len(cons) + 1, np.int64)
    for i, c in enumerate(cons):
        mrow[i + 1] = mrow[i] + c["nodes"]
    nz = np.cumsum([0] + [c["nja"] for c in cons])
    ia = np.concatenate([c["ia"][:-1] + nz[i] for i, c in enumerate(cons)] + [[nz[-1]]])
    ja = np.concatenate([c["ja"] + mrow[i] for i, c in enumerate(cons)])
    out = [mrow.astype(np.int32), ia.astype(np.int32), ja.astype(np.int32)]
    for vals in (amats, rhss, xs):
        if vals is not None:
            out.append(np.concatenate(vals))
    return tuple(out)


class EnsembleLinear:
    """The batched counterpart of ImsLinear: one handle for all members,
    one apply solving every member to its own closure."""

    def __init__(self, settings: ImsLinearSettings):
        self.settings = settings
        self._lib = _lib.load()
        self._h = C.c_void_p()
        self.nm = 0

    def allocate(self, member_rows: np.ndarray, ia: np.ndarray, ja: np.ndarray,
                 shapes=None) -> "EnsembleLinear":
        """shapes: optional (nlay, nrow, ncol) per member (full DIS grids),
        which selects the batched wavefront preconditioner."""
        mr = np.ascontiguousarray(member_rows, np.int32)
        ia = np.ascontiguousarray(ia, np.int32)
        ja = np.ascontiguousarray(ja, np.int32)
        sh = None if shapes is None else np.ascontiguousarray(np.asarray(shapes).reshape(-1), np.int32)
        s = self.settings.to_c(0)
        rc = self._lib.gbims_batch_create(C.byref(s), mr.size - 1, _lib.iptr(mr), int(mr[-1]),
                                          ja.size, _lib.iptr(ia), _lib.iptr(ja),
                                          None if sh is None else _lib.iptr(sh), C.byref(self._h))
        if rc < 0:
            msg = self._lib.gbims_last_error(self._h).decode() if self._h else ""
            raise _lib.GbimsError(rc, msg)
        self.nm = mr.size - 1
        return self

    def apply(self, amat: np.ndarray, rhs: np.ndarray, x: np.ndarray, kstp: int = 1,
              kiter: int = 1) -> list[ApplyResult]:
        """Solves every member; x (all members) is overwritten."""
        icnvg = np.zeros(self.nm, np.int32)
        it = np.zeros(self.nm, np.int32)
        sums = (_lib.GbimsSummary * self.nm)()
        rc = self._lib.gbims_batch_apply(self._h, _lib.dptr(amat), _lib.dptr(rhs), _lib.dptr(x),
                                         kstp, kiter, _lib.iptr(icnvg), _lib.iptr(it), sums)
        if rc < 0:
            raise _lib.GbimsError(rc, self._lib.gbims_last_error(self._h).decode())
        return [ApplyResult(int(icnvg[m]), int(it[m]), rc, _summary(sums[m])) for m in range(self.nm)]

    def apply_device(self, d_amat: int, d_rhs: int, d_x: int, kstp: int = 1,
                     kiter: int = 1) -> list[ApplyResult]:
        icnvg = np.zeros(self.nm, np.int32)
        it = np.zeros(self.nm, np.int32)
        sums = (_lib.GbimsSummary * self.nm)()
        rc = self._lib.gbims_batch_apply_device(self._h, C.c_void_p(d_amat), C.c_void_p(d_rhs),
                                                C.c_void_p(d_x), kstp, kiter, _lib.iptr(icnvg),
                                                _lib.iptr(it), sums)
        if rc < 0:
            raise _lib.GbimsError(rc, self._lib.gbims_last_error(self._h).decode())
        return [ApplyResult(int(icnvg[m]), int(it[m]), rc, _summary(sums[m])) for m in range(self.nm)]

    def close(self):
        if self._h:
            self._lib.gbims_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
