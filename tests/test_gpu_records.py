"""Per-inner-iteration convergence records through the C ABI
(gbims_set_inner_records / gbims_get_inner_records) against the oracle's
ConvergenceSummary rows: ITINNER, the CACCEL values (alpha; BiCGSTAB alpha
and omega) and, per model, the signed largest head change and residual with
their rows (ImsLinearBase.f90:141-197, :431-493).  The level-scheduled FP64
path sums its dot products in another order than ddot, so values agree to
rounding and the rows exactly over the first iterations."""
import numpy as np
import pytest

from modflow6_gb300 import _lib
from test_gpu_ims import c1_system, gpu_ims, oracle_solve  # noqa: F401
import oracle

pytestmark = pytest.mark.gpu

TOL = dict(dvclose=1e-8, rclose=1e-6, iter1=400)


@pytest.mark.parametrize("ilinmeth", [1, 2])
@pytest.mark.parametrize("modstart", [[0, 10000], [0, 2500, 6100, 10000]])
def test_inner_records_match_oracle(gblib, ilinmeth, modstart):
    con, amat, rhs, x0 = c1_system()
    ims = gpu_ims(con, ilinmeth=ilinmeth, **TOL)
    ims.set_inner_records(500, modstart)
    res = ims.imslinear_apply(amat.copy(), rhs.copy(), x0.copy())
    rec = ims.inner_records()
    assert res.icnvg == 1 and rec["itinner"].size == res.in_iter
    np.testing.assert_array_equal(rec["itinner"], np.arange(1, res.in_iter + 1))
    o = oracle.Ims(oracle.settings(ilinmeth=ilinmeth, **TOL), con["ia"], con["ja"])
    o.set_models(modstart, 500)
    icnvg, it, orec = o.apply(amat.copy(), rhs.copy(), x0.copy(), nrec=500)
    om = o.model_records(it)
    k = min(10, it, res.in_iter)
    al = np.array([r["alpha"] for r in orec[:k]])
    np.testing.assert_allclose(rec["alpha"][:k], al, rtol=1e-9)
    if ilinmeth == 2:
        omg = np.array([r["omega"] for r in orec[:k]])
        np.testing.assert_allclose(rec["omega"][:k], omg, rtol=1e-9)
    else:
        assert np.all(rec["omega"] == 0.0)
    for key in ("locdv", "locr"):
        np.testing.assert_array_equal(rec[key][:k], om[key][:k])
    for key in ("dvmax", "rmax"):
        scale = np.abs(om[key][:k]).max(axis=1, keepdims=True)
        assert np.all(np.abs(rec[key][:k] - om[key][:k]) <= 1e-8 * scale)
    # the last record's overall maxima are the apply's summary
    s = res.summary
    im = int(np.argmax(np.abs(rec["dvmax"][-1])))
    assert rec["dvmax"][-1, im] == s["dvmax"] and rec["locdv"][-1, im] == s["locdv"]
    im = int(np.argmax(np.abs(rec["rmax"][-1])))
    assert rec["rmax"][-1, im] == s["rmax"] and rec["locr"][-1, im] == s["locr"]
    # every model's rows lie in the model
    ms = np.array(modstart)
    for key in ("locdv", "locr"):
        lo = rec[key]
        assert np.all((lo >= ms[:-1]) & (lo < ms[1:]))


def test_inner_records_capacity_base_and_off(gblib):
    """At most nconv records; rows in the handle's index base (1-based for a
    Fortran caller); nconv 0 switches them off; bad CONVMODSTART is refused."""
    con, amat, rhs, x0 = c1_system()
    ims = gpu_ims(con, **TOL)
    ims.set_inner_records(5)
    r = ims.imslinear_apply(amat.copy(), rhs.copy(), x0.copy())
    rec = ims.inner_records()
    assert r.in_iter > 5 and rec["itinner"].size == 5
    lib = _lib.load()
    for bad in ([1, 10000], [0, 9999], [0, 5000, 5000, 10000]):
        ms = np.array(bad, np.int32)
        assert lib.gbims_set_inner_records(ims._h, 10, ms.size - 1, _lib.iptr(ms)) == _lib.GBIMS_ERR_ARG
    ims.set_inner_records(0)
    ims.imslinear_apply(amat.copy(), rhs.copy(), x0.copy())
    assert ims.inner_records()["itinner"].size == 0
    # a 1-based caller gets 1-based rows
    ia1, ja1 = con["ia"] + 1, con["ja"] + 1
    from modflow6_gb300.ims import GENERAL, ImsLinear, ImsLinearSettings
    f = ImsLinear(ImsLinearSettings(structure=GENERAL, **TOL)).imslinear_allocate(
        con["nodes"], ia1, ja1, index_base=1)
    f.set_inner_records(500, [1, 5001, 10001], index_base=1)
    f.imslinear_apply(amat.copy(), rhs.copy(), x0.copy())
    g = gpu_ims(con, **TOL)
    g.set_inner_records(500, [0, 5000, 10000])
    g.imslinear_apply(amat.copy(), rhs.copy(), x0.copy())
    r1, r0 = f.inner_records(), g.inner_records()
    np.testing.assert_array_equal(r1["locdv"], r0["locdv"] + 1)
    np.testing.assert_array_equal(r1["dvmax"], r0["dvmax"])


def test_inner_records_refused_for_mixed(gblib):
    con, amat, rhs, x0 = c1_system()
    ims = gpu_ims(con, precision=_lib.GBIMS_MIXED, **TOL)
    with pytest.raises(_lib.GbimsError):
        ims.set_inner_records(10)
