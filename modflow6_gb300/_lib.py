"""ctypes bindings of libgbims.so (the C ABI declared in include/gbims.h).

The library is loaded from the package directory.  There is no fallback: if
the shared library is missing, every entry point raises, so a GPU run can
never silently compute on the CPU.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libgbims.so"

GBIMS_OK = 0
GBIMS_WARN_PIVOT = 1
GBIMS_WARN_FALLBACK = 2
GBIMS_ERR_ARG = -1
GBIMS_ERR_CUDA = -2
GBIMS_ERR_UNSUPPORTED = -3
GBIMS_ERR_NONFINITE = -4
GBIMS_ERR_NOMEM = -5
GBIMS_ERR_STATE = -6
GBIMS_FP64 = 0
GBIMS_MIXED = 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class GbimsSettings(C.Structure):
    _fields_ = [
        ("dvclose", C.c_double), ("rclose", C.c_double), ("icnvgopt", C.c_int),
        ("iter1", C.c_int), ("ilinmeth", C.c_int), ("iscl", C.c_int), ("iord", C.c_int),
        ("north", C.c_int), ("relax", C.c_double), ("level", C.c_int),
        ("droptol", C.c_double), ("precision", C.c_int), ("index_base", C.c_int),
        ("nlay", C.c_int), ("nrow", C.c_int), ("ncol", C.c_int),
    ]


class GbimsSummary(C.Structure):
    _fields_ = [
        ("iter_cnt", C.c_int), ("icnvg", C.c_int), ("pivot_retries", C.c_int),
        ("exit_reason", C.c_int), ("dvmax", C.c_double), ("locdv", C.c_int),
        ("rmax", C.c_double), ("locr", C.c_int), ("l2norm0", C.c_double),
        ("l2norm", C.c_double), ("solve_ms", C.c_double), ("refinements", C.c_int),
        ("structured", C.c_int),
    ]


class GbimsKernelTimes(C.Structure):
    _fields_ = [("spmv_ms", C.c_double), ("precond_ms", C.c_double), ("dot_ms", C.c_double),
                ("update_ms", C.c_double), ("spmv_bytes", C.c_double), ("precond_bytes", C.c_double)]


class GbnpfOptions(C.Structure):
    _fields_ = [
        ("inewton", C.c_int), ("ivarcv", C.c_int), ("idewatcv", C.c_int),
        ("icellavg", C.c_int), ("satomega", C.c_double), ("index_base", C.c_int),
        ("inewtonur", C.c_int),
    ]


class GbslnModel(C.Structure):
    _fields_ = [
        ("nlay", C.c_int), ("nrow", C.c_int), ("ncol", C.c_int),
        ("delr", _dp), ("delc", _dp), ("top", _dp), ("botm", _dp),
        ("k11", _dp), ("k33", _dp), ("icelltype", _ip), ("ss", _dp), ("sy", _dp),
        ("nchd", C.c_int), ("chd_node", _ip), ("chd_head", _dp),
        ("nwel", C.c_int), ("wel_node", _ip), ("wel_q", _dp),
        ("nrch", C.c_int), ("rch_node", _ip), ("rch_rate", _dp),
    ]


class GbslnGrid(C.Structure):
    _fields_ = [
        ("nodes", C.c_int), ("nja", C.c_int), ("ia", _ip), ("ja", _ip), ("ihc", _ip),
        ("cl1", _dp), ("cl2", _dp), ("hwva", _dp), ("top", _dp), ("bot", _dp), ("area", _dp),
    ]


class GbslnKTensor(C.Structure):
    _fields_ = [("k22", _dp), ("angle1", _dp), ("angle2", _dp), ("angle3", _dp), ("xt3d", C.c_int),
                ("iavgkeff", C.c_int)]


class GbslnGeometry(C.Structure):
    _fields_ = [("xc", _dp), ("yc", _dp), ("anglex", _dp), ("centre_vertical", C.c_int)]


class GbslnNonlinear(C.Structure):
    _fields_ = [
        ("dvclose", C.c_double), ("mxiter", C.c_int), ("nonmeth", C.c_int),
        ("theta", C.c_double), ("akappa", C.c_double), ("gamma", C.c_double),
        ("amomentum", C.c_double), ("iallowptc", C.c_int), ("numtrack", C.c_int),
        ("btol", C.c_double), ("breduc", C.c_double), ("res_lim", C.c_double),
    ]


class GbslnStats(C.Structure):
    _fields_ = [
        ("outer", C.c_int), ("inner_total", C.c_int), ("converged", C.c_int),
        ("pivot_retries", C.c_int), ("dxmax", C.c_double), ("fill_ms", C.c_double),
        ("solve_ms", C.c_double), ("total_ms", C.c_double), ("backtracks", C.c_int),
        ("guess_alpha", C.c_double), ("prev_alpha", C.c_double),
    ]


class GbmpnnScaling(C.Structure):
    _fields_ = [("head_ref", C.c_double), ("head_scale", C.c_double), ("dh_soft", C.c_double),
                ("dh_scale", C.c_double), ("unit_max", C.c_double)]


class GbimsTuning(C.Structure):
    _fields_ = [
        ("sweep_config", C.c_int), ("sweep_chunk", C.c_int), ("sweep_ring", C.c_int),
        ("sweep_prefetch", C.c_int), ("sweep_occupancy", C.c_int), ("reduction_blocks", C.c_int),
        ("level_mode", C.c_int), ("level_ms", C.c_double * 2), ("ncandidates", C.c_int),
        ("candidate_ms", C.c_double * 16), ("precond_ms", C.c_double), ("vector_ms", C.c_double),
        ("sweep_config_backward", C.c_int),
    ]


class GbslnBudgetTable(C.Structure):
    _fields_ = [
        ("rate_in", C.c_double * 5), ("rate_out", C.c_double * 5), ("total_in", C.c_double),
        ("total_out", C.c_double), ("percent_discrepancy", C.c_double),
        ("max_cell_imbalance", C.c_double), ("max_cell", C.c_int),
    ]


# name -> (restype, argtypes)
_SIGS = {
    "gbims_create": (C.c_int, [C.POINTER(GbimsSettings), C.c_int, C.c_int, _ip, _ip, C.POINTER(C.c_void_p)]),
    "gbims_apply": (C.c_int, [C.c_void_p, _dp, _dp, _dp, C.c_int, C.c_int, _ip, _ip, C.POINTER(GbimsSummary)]),
    "gbims_apply_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, _ip, _ip, C.POINTER(GbimsSummary)]),
    "gbims_destroy": (C.c_int, [C.c_void_p]),
    "gbims_batch_create": (C.c_int, [C.POINTER(GbimsSettings), C.c_int, _ip, C.c_int, C.c_int, _ip,
                                     _ip, _ip, C.POINTER(C.c_void_p)]),
    "gbims_batch_apply": (C.c_int, [C.c_void_p, _dp, _dp, _dp, C.c_int, C.c_int, _ip, _ip,
                                    C.POINTER(GbimsSummary)]),
    "gbims_batch_apply_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                           C.c_int, _ip, _ip, C.POINTER(GbimsSummary)]),
    "gbims_time_kernels": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "gbims_factor": (C.c_int, [C.c_void_p, _dp, _ip]),
    "gbims_get_apc": (C.c_int, [C.c_void_p, _dp]),
    "gbims_get_factor": (C.c_int, [C.c_void_p, _ip, _ip, _dp, C.c_int, _ip]),
    "gbims_set_inner_records": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _ip]),
    "gbims_get_inner_records": (C.c_int, [C.c_void_p, C.c_int, _ip, _ip, _dp, _dp, _ip, _dp, _ip,
                                          _dp]),
    "gbims_calc_order": (C.c_int, [C.c_int, C.c_int, C.c_int, _ip, _ip, C.c_int, _ip, _ip]),
    "gbims_matvec": (C.c_int, [C.c_void_p, _dp, _dp]),
    "gbims_precondition": (C.c_int, [C.c_void_p, _dp, _dp]),
    "gbims_kernel_launches": (C.c_longlong, [C.c_void_p]),
    "gbims_last_error": (C.c_char_p, [C.c_void_p]),
    "gbims_status_string": (C.c_char_p, [C.c_int]),
    "gbims_residual_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                         C.POINTER(C.c_double), C.POINTER(C.c_double),
                                         C.POINTER(C.c_int)]),
    "gbnpf_create": (C.c_int, [C.POINTER(GbnpfOptions), C.c_int, C.c_int, C.c_int, _ip, _ip, _ip, _ip, _ip,
                               _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip, C.POINTER(C.c_void_p)]),
    "gbnpf_fill": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gbnpf_get_condsat": (C.c_int, [C.c_void_p, _dp]),
    "gbnpf_destroy": (C.c_int, [C.c_void_p]),
    "gbsln_create": (C.c_int, [C.POINTER(GbslnModel), C.POINTER(GbnpfOptions), C.POINTER(GbimsSettings),
                               C.POINTER(GbslnNonlinear), _dp, C.POINTER(C.c_void_p)]),
    "gbsln_create_tensor": (C.c_int, [C.POINTER(GbslnModel), C.POINTER(GbslnKTensor), C.POINTER(GbnpfOptions),
                                    C.POINTER(GbimsSettings), C.POINTER(GbslnNonlinear), _dp,
                                    C.POINTER(C.c_void_p)]),
    "gbsln_budget_cells": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp, _dp]),
    "gbsln_create_grid_tensor": (C.c_int, [C.POINTER(GbslnGrid), C.POINTER(GbslnModel), C.POINTER(GbslnKTensor),
                                         C.POINTER(GbslnGeometry), C.POINTER(GbnpfOptions),
                                         C.POINTER(GbimsSettings), C.POINTER(GbslnNonlinear), _dp,
                                         C.POINTER(C.c_void_p)]),
    "gbsln_create_grid": (C.c_int, [C.POINTER(GbslnGrid), C.POINTER(GbslnModel), C.POINTER(GbnpfOptions),
                                    C.POINTER(GbimsSettings), C.POINTER(GbslnNonlinear), _dp,
                                    C.POINTER(C.c_void_p)]),
    "gbsln_timestep": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double, C.POINTER(GbslnStats)]),
    "gbsln_timestep_guess": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_void_p,
                                       C.POINTER(GbslnStats)]),
    "gbsln_formulate": (C.c_int, [C.c_void_p, C.c_double, _dp, _dp, _dp]),
    "gbsln_last_error": (C.c_char_p, [C.c_void_p]),
    "gbsln_restart": (C.c_int, [C.c_void_p]),
    "gbsln_budget": (C.c_int, [C.c_void_p, _dp, C.POINTER(GbslnBudgetTable)]),
    "gbims_autotune": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(GbimsTuning)]),
    "gbims_set_dis_nodes": (C.c_int, [C.c_void_p, _ip]),
    "gbims_set_tuning": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "gbsln_get_heads": (C.c_int, [C.c_void_p, _dp]),
    "gbsln_set_heads": (C.c_int, [C.c_void_p, _dp]),
    "gbsln_ims": (C.c_void_p, [C.c_void_p]),
    "gbsln_destroy": (C.c_int, [C.c_void_p]),
    "gbmpnn_param_count": (C.c_longlong, []),
    "gbmpnn_create": (C.c_int, [C.c_int, C.c_int, _ip, _ip, C.c_ulonglong, C.POINTER(C.c_void_p)]),
    "gbmpnn_set_graph": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gbmpnn_set_loss": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(GbmpnnScaling), C.c_float]),
    "gbmpnn_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "gbsln_warm_guess": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(GbmpnnScaling),
                                   C.c_int, C.c_void_p, C.POINTER(C.c_float)]),
    "gbsln_timestep_warm": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_void_p, C.c_int,
                                      C.POINTER(GbslnStats)]),
    "gbmpnn_gradients": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float,
                                   C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "gbmpnn_train_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float,
                                    C.c_float, C.POINTER(C.c_float)]),
    "gbmpnn_get_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "gbmpnn_set_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "gbmpnn_last_error": (C.c_char_p, [C.c_void_p]),
    "gbmpnn_destroy": (C.c_int, [C.c_void_p]),
}

EXPORTED = tuple(_SIGS)

_lib = None


def load() -> C.CDLL:
    """Loads libgbims.so from the package directory (raises if absent)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with modflow6_gb300.build.build() "
                "(the GB300 library has no CPU fallback)")
        lib = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class GbimsError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"status {status}: {msg}")
        self.status = status


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)
