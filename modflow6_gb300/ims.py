"""Host mirror of the MODFLOW 6 IMS linear-solver interface over libgbims.

`ImsLinearSettings` carries the IMS LINEAR block options with the meaning of
src/Solution/LinearMethods/ImsLinearSettings.f90 (presets :74-116), and
`ImsLinear` mirrors ImsLinearDataType (ImsLinear.f90:22-102):
`imslinear_allocate` (:111-339) and `imslinear_apply` (:617-750).  Both
delegate to the C ABI in include/gbims.h; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib

CG_METHOD = 1
# `structure` value that keeps the level-scheduled sweeps on a DIS pattern
GENERAL = (-1, 0, 0)
BCGS_METHOD = 2

EXIT_REASONS = {0: "none", 1: "closure", 2: "stagnation", 3: "itmax", 4: "exact", 5: "zero rho"}


@dataclass
class ImsLinearSettings:
    """IMS LINEAR options (defaults: COMPLEXITY SIMPLE, ImsLinearSettings.f90:79-89)."""

    dvclose: float = 1.0e-3      # INNER_DVCLOSE
    rclose: float = 1.0e-1       # INNER_RCLOSE
    icnvgopt: int = 0            # RCLOSE option (0 inf-norm, 1 strict, 2 L2, 3 rel. L2, 4 L2 + rel.)
    iter1: int = 50              # INNER_MAXIMUM
    ilinmeth: int = CG_METHOD    # LINEAR_ACCELERATION
    iscl: int = 0                # SCALING_METHOD
    iord: int = 0                # REORDERING_METHOD
    north: int = 0               # NUMBER_ORTHOGONALIZATIONS
    relax: float = 0.0           # RELAXATION_FACTOR (MILU0 when > 0)
    level: int = 0               # PRECONDITIONER_LEVELS
    droptol: float = 0.0         # PRECONDITIONER_DROP_TOLERANCE
    precision: int = _lib.GBIMS_FP64
    # (nlay, nrow, ncol) of a DIS grid for the wavefront sweeps; (0, 0, 0):
    # found from the pattern; GENERAL: the level-scheduled sweeps always
    structure: tuple = field(default=(0, 0, 0))

    @classmethod
    def preset_config(cls, complexity: str, **overrides) -> "ImsLinearSettings":
        """COMPLEXITY presets of ImsLinearSettings.f90:74-116."""
        c = complexity.upper()
        if c == "SIMPLE":
            s = cls(iter1=50, ilinmeth=1, dvclose=1e-3, rclose=1e-1)
        elif c == "MODERATE":
            s = cls(iter1=100, ilinmeth=2, dvclose=1e-2, rclose=1e-1, relax=0.97)
        elif c == "COMPLEX":
            s = cls(iter1=500, ilinmeth=2, dvclose=1e-1, rclose=1e-1, level=5, droptol=1e-4, north=2)
        else:
            raise ValueError(f"unknown COMPLEXITY {complexity!r}")
        for k, v in overrides.items():
            setattr(s, k, v)
        return s

    @property
    def ipc(self) -> int:
        """Preconditioner choice of ImsLinear.f90:178-185."""
        ipc = 3 if (self.level > 0 or self.droptol > 0.0) else 1
        return ipc + 1 if self.relax > 0.0 else ipc

    def to_c(self, index_base: int = 0) -> _lib.GbimsSettings:
        nl, nr, nc = self.structure
        return _lib.GbimsSettings(
            self.dvclose, self.rclose, self.icnvgopt, self.iter1, self.ilinmeth, self.iscl,
            self.iord, self.north, self.relax, self.level, self.droptol, self.precision,
            index_base, nl, nr, nc)


@dataclass
class ApplyResult:
    icnvg: int
    in_iter: int
    status: int
    summary: dict


class ImsLinear:
    """GB300 IMS linear accelerator with the ImsLinearDataType contract.

    `imslinear_allocate` builds IAPC/JAPC, the level schedule and the device
    layouts once per matrix structure.  `imslinear_apply` takes the solution's
    AMAT, RHS and X (X is the initial guess and is overwritten with the
    solution) and returns ICNVG and IN_ITER.
    """

    def __init__(self, settings: ImsLinearSettings):
        self.settings = settings
        self._h = C.c_void_p()
        self.neq = 0
        self.nja = 0

    # -- ImsLinear.f90:111-339
    def imslinear_allocate(self, neq: int, ia: np.ndarray, ja: np.ndarray, index_base: int = 0):
        lib = _lib.load()
        ia = np.ascontiguousarray(ia, dtype=np.int32)
        ja = np.ascontiguousarray(ja, dtype=np.int32)
        self.neq, self.nja = int(neq), int(ja.size)
        cs = self.settings.to_c(index_base)
        rc = lib.gbims_create(C.byref(cs), self.neq, self.nja, _lib.iptr(ia), _lib.iptr(ja),
                              C.byref(self._h))
        if rc < 0:
            msg = lib.gbims_last_error(self._h).decode() if self._h else ""
            lib.gbims_destroy(self._h)
            self._h = C.c_void_p()
            raise _lib.GbimsError(rc, msg or lib.gbims_status_string(rc).decode())
        return self

    # -- ImsLinear.f90:617-750
    def imslinear_apply(self, amat: np.ndarray, rhs: np.ndarray, x: np.ndarray, kstp: int = 1,
                        kiter: int = 1) -> ApplyResult:
        lib = _lib.load()
        if not self._h:
            raise _lib.GbimsError(_lib.GBIMS_ERR_STATE, "imslinear_allocate was not called")
        icnvg, in_iter = C.c_int(0), C.c_int(0)
        sm = _lib.GbimsSummary()
        rc = lib.gbims_apply(self._h, _lib.dptr(amat), _lib.dptr(rhs), _lib.dptr(x), kstp, kiter,
                             C.byref(icnvg), C.byref(in_iter), C.byref(sm))
        if rc < 0:
            raise _lib.GbimsError(rc, lib.gbims_last_error(self._h).decode())
        return ApplyResult(icnvg.value, in_iter.value, rc, _summary(sm))

    def set_dis_nodes(self, nodeuser: np.ndarray):
        """gbims_set_dis_nodes: the handle's pattern is the DIS grid of the
        settings' shape with IDOMAIN cells removed, `nodeuser` the user cell
        of each node (DisType%nodeuser): the ILU0 sweeps then run as
        wavefront sweeps on the full grid.  Before the first apply."""
        lib = _lib.load()
        nu = np.ascontiguousarray(nodeuser, dtype=np.int32)
        if nu.size != self.neq:
            raise _lib.GbimsError(_lib.GBIMS_ERR_ARG, "nodeuser needs one entry per node")
        rc = lib.gbims_set_dis_nodes(self._h, _lib.iptr(nu))
        if rc < 0:
            raise _lib.GbimsError(rc, lib.gbims_last_error(self._h).decode())
        return self

    def set_inner_records(self, nconv: int, convmodstart=None, index_base: int = 0):
        """Keep up to `nconv` per-inner-iteration records per apply
        (imslinear_ap's NCONV; 0 switches them off).  `convmodstart`: the
        first row of each model and neq (CONVMODSTART), default one model."""
        lib = _lib.load()
        ms = np.ascontiguousarray([index_base, self.neq + index_base] if convmodstart is None
                                  else convmodstart, dtype=np.int32)
        self._rec_nmod = int(ms.size - 1) if nconv > 0 else 0
        self._rec_cap = int(nconv)
        rc = lib.gbims_set_inner_records(self._h, int(nconv), self._rec_nmod or 1, _lib.iptr(ms))
        if rc < 0:
            raise _lib.GbimsError(rc, lib.gbims_last_error(self._h).decode())

    def inner_records(self) -> dict:
        """The last apply's records: itinner, alpha, omega (CACCEL), and per
        model (shape [nrec, convnmod]) dvmax, locdv, rmax, locr."""
        lib = _lib.load()
        cap, nm = getattr(self, "_rec_cap", 0), max(getattr(self, "_rec_nmod", 0), 1)
        it = np.zeros(max(cap, 1), np.int32)
        al, om = np.zeros(max(cap, 1)), np.zeros(max(cap, 1))
        ldv, lr = np.zeros(max(cap, 1) * nm, np.int32), np.zeros(max(cap, 1) * nm, np.int32)
        dv, rm = np.zeros(max(cap, 1) * nm), np.zeros(max(cap, 1) * nm)
        nrec = C.c_int(0)
        rc = lib.gbims_get_inner_records(self._h, cap, C.byref(nrec), _lib.iptr(it), _lib.dptr(al),
                                         _lib.dptr(om), _lib.iptr(ldv), _lib.dptr(dv),
                                         _lib.iptr(lr), _lib.dptr(rm))
        if rc < 0:
            raise _lib.GbimsError(rc, lib.gbims_last_error(self._h).decode())
        k = nrec.value
        return dict(itinner=it[:k], alpha=al[:k], omega=om[:k], locdv=ldv[:k * nm].reshape(k, nm),
                    dvmax=dv[:k * nm].reshape(k, nm), locr=lr[:k * nm].reshape(k, nm),
                    rmax=rm[:k * nm].reshape(k, nm))

    def get_factor(self):
        """The preconditioner of the last factor or apply as (iapc, japc, apc),
        0-based: row i's L entries at [iapc[i], japc[i]), its U entries at
        [japc[i], iapc[i+1]), apc[:neq] the inverse pivots (ILU0's APC, or
        ILUT's MSR storage with its row pointers in iapc)."""
        lib = _lib.load()
        njapc = C.c_int(0)
        rc = lib.gbims_get_factor(self._h, None, None, None, 0, C.byref(njapc))
        if rc < 0:
            raise _lib.GbimsError(rc, lib.gbims_last_error(self._h).decode())
        iapc = np.zeros(self.neq + 1, np.int32)
        japc = np.zeros(njapc.value, np.int32)
        apc = np.zeros(njapc.value)
        rc = lib.gbims_get_factor(self._h, _lib.iptr(iapc), _lib.iptr(japc), _lib.dptr(apc),
                                  njapc.value, C.byref(njapc))
        if rc < 0:
            raise _lib.GbimsError(rc, lib.gbims_last_error(self._h).decode())
        return iapc, japc, apc

    def apply_device(self, d_amat: int, d_rhs: int, d_x: int, kstp: int = 1,
                     kiter: int = 1) -> ApplyResult:
        """imslinear_apply on device pointers (e.g. torch tensors' data_ptr())."""
        lib = _lib.load()
        icnvg, in_iter = C.c_int(0), C.c_int(0)
        sm = _lib.GbimsSummary()
        rc = lib.gbims_apply_device(self._h, C.c_void_p(d_amat), C.c_void_p(d_rhs),
                                    C.c_void_p(d_x), kstp, kiter, C.byref(icnvg),
                                    C.byref(in_iter), C.byref(sm))
        if rc < 0:
            raise _lib.GbimsError(rc, lib.gbims_last_error(self._h).decode())
        return ApplyResult(icnvg.value, in_iter.value, rc, _summary(sm))

    def imslinear_da(self):
        if self._h:
            _lib.load().gbims_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.imslinear_da()
        except Exception:
            pass


def _summary(sm: _lib.GbimsSummary) -> dict:
    d = {name: getattr(sm, name) for name, _ in sm._fields_}
    d["exit"] = EXIT_REASONS.get(sm.exit_reason, "?")
    return d
