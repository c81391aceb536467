"""gbims_residual_noalloc, the entry point that allocates nothing, against the
handle-based entry points on the same system: its residual vector against
b - gbims_matvec(x), its L2 norm against gbims_apply's L2NORM0, and its
signed max|r| against the residual's own maximum -- bit for bit, on two
calls in a row (the static scratch carries nothing from one call to the
next) -- and the device's free memory unchanged across the second call.
Collected last so it also runs after every other GPU test.
"""
import ctypes as C

import numpy as np
import pytest

from modflow6_gb300 import _lib
from test_gpu_ims import c1_system, gpu_ims

pytestmark = pytest.mark.gpu

MAX_ROWS = 608 * 256


def _noalloc(lib, n, nja, dev, base):
    l2, rmax, locr = C.c_double(), C.c_double(-1.0), C.c_int(-7)
    rc = lib.gbims_residual_noalloc(n, nja, dev["ia"].data_ptr(), dev["ja"].data_ptr(),
                                    dev["amat"].data_ptr(), dev["x"].data_ptr(),
                                    dev["rhs"].data_ptr(), dev["resid"].data_ptr(), base, None,
                                    C.byref(l2), C.byref(rmax), C.byref(locr))
    return rc, l2.value, rmax.value, locr.value


@pytest.mark.parametrize("base", [0, 1])
def test_residual_noalloc_matches_handle_entry_points(gblib, base):
    torch = pytest.importorskip("torch")
    con, amat, rhs, x0 = c1_system()
    n, nja = con["nodes"], con["nja"]
    # the handle-based entry points on the same inputs
    ims = gpu_ims(con, dvclose=1e-8, rclose=1e-6, iter1=500)
    res = ims.imslinear_apply(amat.copy(), rhs.copy(), x0.copy())
    l2_ref = res.summary["l2norm0"]
    y = np.zeros(n)
    assert gblib.gbims_matvec(ims._h, _lib.dptr(x0), _lib.dptr(y)) == 0
    r_ref = rhs - y
    loc_ref = int(np.argmax(np.abs(r_ref)))
    dev = {"ia": torch.from_numpy(con["ia"].astype(np.int32) + base).cuda(),
           "ja": torch.from_numpy(con["ja"].astype(np.int32) + base).cuda(),
           "amat": torch.from_numpy(amat).cuda(), "x": torch.from_numpy(x0).cuda(),
           "rhs": torch.from_numpy(rhs).cuda(),
           "resid": torch.full((n,), np.nan, dtype=torch.float64, device="cuda")}
    torch.cuda.synchronize()
    for call in range(2):
        dev["resid"].fill_(np.nan)
        torch.cuda.synchronize()
        # the first call looks up the static array and loads the kernels; from
        # the second on, the device's free memory must not move
        free_before = torch.cuda.mem_get_info()[0]
        rc, l2, rmax, locr = _noalloc(gblib, n, nja, dev, base)
        free_after = torch.cuda.mem_get_info()[0]
        assert rc == _lib.GBIMS_OK
        if call > 0:
            assert free_after == free_before
        np.testing.assert_array_equal(dev["resid"].cpu().numpy(), r_ref)
        assert l2 == l2_ref
        assert locr == loc_ref and rmax == r_ref[loc_ref]


def test_residual_noalloc_rejects_oversize(gblib):
    torch = pytest.importorskip("torch")
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = buf.data_ptr()
    l2, rmax, locr = C.c_double(), C.c_double(), C.c_int()
    for n in (0, MAX_ROWS + 1):
        rc = gblib.gbims_residual_noalloc(n, 7 * max(n, 1), p, p, p, p, p, p, 0, None,
                                          C.byref(l2), C.byref(rmax), C.byref(locr))
        assert rc == _lib.GBIMS_ERR_ARG
