"""Pins the CPU oracle to the known answers held by the reference's own tests.

* autotest/test_gwf_chd01.py:13-127: 1x1x100 confined column, CHD 1.0 and 0.0
  at the ends, CG, inner/outer dvclose 1e-6, rclose 1e-6; answer
  np.linspace(1, 0, 100) (:126-127).
* autotest/test_gwf_newton01.py:8-103: 2x3x3 convertible Newton model, CHD 7
  in layer 2, recharge 1 on layer 1; answers H1 = 8.0 at (0,1,1) and
  H2 = 7.0 at (1,1,1) (:95-103).  The reference runs COMPLEXITY COMPLEX
  (BiCGSTAB + ILUT, backtracking); the case is run both that way and with
  PRECONDITIONER_LEVELS 0 / DROP_TOLERANCE 0 (BiCGSTAB + ILU0), which must
  reach the same heads.
* autotest/test_gwf_newton_under_relaxation.py:8-35, 106-119 (case nr_ur01):
  51x51x1 convertible model over the bumpy bottom of
  autotest/data/ex-gwf-bump/bottom.txt, NEWTON UNDER_RELAXATION, BiCGSTAB,
  CHD 7.5 / 2.5 on the first and last columns.  Its answer is a head file
  that MODFLOW 6 wrote, autotest/data/ex-gwf-bump/results.hds.cmp, compared
  with np.allclose; both arrays are in tests/golden/ex_gwf_bump.npz
  (tests/golden/make_bump_fixture.py).
"""
from pathlib import Path

import numpy as np
import pytest

import oracle
from modflow6_gb300.dis import GwfDisModel

GOLDEN = Path(__file__).resolve().parent / "golden"


def chd01_model():
    nlay, nrow, ncol = 1, 1, 100
    m = GwfDisModel(nlay, nrow, ncol, np.ones(ncol), np.ones(nrow), np.ones(ncol), np.zeros(ncol),
                    np.ones(ncol), np.ones(ncol), np.zeros(ncol, np.int32), np.ones(ncol))
    m.chd_node = np.array([0, 99], np.int32)
    m.chd_head = np.array([1.0, 0.0])
    return m


def newton01_model():
    nlay, nrow, ncol = 2, 3, 3
    nrc = nrow * ncol
    m = GwfDisModel(nlay, nrow, ncol, np.ones(ncol), np.ones(nrow), np.full(nrc, 20.0),
                    np.concatenate([np.full(nrc, 10.0), np.zeros(nrc)]), np.full(2 * nrc, 10.0),
                    np.full(2 * nrc, 10.0), np.ones(2 * nrc, np.int32), np.full(2 * nrc, 7.0),
                    inewton=1)
    m.chd_node = np.arange(nrc, 2 * nrc, dtype=np.int32)
    m.chd_head = np.full(nrc, 7.0)
    m.rch_node = np.arange(nrc, dtype=np.int32)
    m.rch_rate = np.ones(nrc)
    return m


def test_chd01_linspace():
    m = chd01_model()
    s = oracle.settings(dvclose=1e-6, rclose=1e-6, iter1=300, ilinmeth=1)
    g = oracle.Gwf(m, s)
    st = g.timestep(kper=1, kstp=1, delt=5.0, transient=False, dvclose=1e-6, mxiter=100)
    assert st["converged"] == 1
    np.testing.assert_allclose(g.x, np.linspace(1, 0, 100), rtol=1e-5, atol=1e-8)


@pytest.mark.parametrize("ilinmeth", [1, 2])
def test_chd01_both_accelerators(ilinmeth):
    m = chd01_model()
    s = oracle.settings(dvclose=1e-9, rclose=1e-9, iter1=300, ilinmeth=ilinmeth)
    g = oracle.Gwf(m, s)
    st = g.timestep(kper=1, kstp=1, delt=5.0, dvclose=1e-9, mxiter=100)
    assert st["converged"] == 1
    np.testing.assert_allclose(g.x, np.linspace(1, 0, 100), atol=1e-7)


def test_newton01_h1_h2():
    m = newton01_model()
    # COMPLEX preset (ImsLinearSettings.f90:100-111, sln_setouter :2657-2669)
    # with ILU0 in place of ILUT and the test's dvclose 1e-9.
    s = oracle.settings(dvclose=1e-9, rclose=0.1, iter1=500, ilinmeth=2, north=2)
    g = oracle.Gwf(m, s)
    st = g.timestep(kper=1, kstp=1, delt=1.0, transient=False, dvclose=1e-9, mxiter=100,
                    nonmeth=3, theta=0.8, akappa=1e-4, gamma=0.0, amomentum=0.0)
    assert st["converged"] == 1
    h1 = g.x[0 * 9 + 1 * 3 + 1]
    h2 = g.x[1 * 9 + 1 * 3 + 1]
    assert np.isclose(h1, 8.0), h1
    assert np.isclose(h2, 7.0), h2


def test_newton01_h1_h2_complex_preset():
    """The reference's own configuration: COMPLEXITY COMPLEX as a whole
    (ImsLinearSettings.f90:100-111 -- BiCGSTAB, ILUT with PRECONDITIONER_LEVELS
    5 and DROP_TOLERANCE 1e-4, NORTH 2; sln_setouter
    NumericalSolution.f90:2657-2669 -- DBD under-relaxation and backtracking)
    with the test's INNER/OUTER_DVCLOSE 1e-9."""
    m = newton01_model()
    s = oracle.settings(dvclose=1e-9, rclose=0.1, iter1=500, ilinmeth=2, north=2, level=5,
                        droptol=1e-4)
    g = oracle.Gwf(m, s)
    st = g.timestep(kper=1, kstp=1, delt=1.0, transient=False, dvclose=1e-9, mxiter=100,
                    nonmeth=3, theta=0.8, akappa=1e-4, gamma=0.0, amomentum=0.0,
                    numtrack=20, btol=1.05, breduc=0.1, res_lim=0.002)
    assert st["converged"] == 1
    assert g.ims.lib.or_ims_ipc(g.ims.h) == 3
    h1 = g.x[0 * 9 + 1 * 3 + 1]
    h2 = g.x[1 * 9 + 1 * 3 + 1]
    assert np.isclose(h1, 8.0), h1
    assert np.isclose(h2, 7.0), h2


# autotest/test_gwf_newton_under_relaxation.py:8-35 (nr_ur01): TDIS defaults
# (one steady period of one step), IMS COMPLEXITY SIMPLE (ImsLinearSettings.f90:
# 81-90, sln_setouter NumericalSolution.f90:2630-2641) with BICGSTAB,
# OUTER_MAXIMUM 75, OUTER_DVCLOSE 1e-8, INNER_MAXIMUM 100, INNER_DVCLOSE 1e-9,
# INNER_RCLOSE 1e-3 and NO_PTC ALL (NumericalSolution.f90:640-653).
BUMP_IMS = dict(dvclose=1e-9, rclose=1e-3, iter1=100, ilinmeth=2)
BUMP_OUTER = dict(dvclose=1e-8, mxiter=75, nonmeth=0, iallowptc=0)


def bump_model():
    f = np.load(GOLDEN / "ex_gwf_bump.npz")
    nrow = ncol = 51
    n = nrow * ncol
    delr = np.full(ncol, 100.0 / ncol)
    delc = np.full(nrow, 100.0 / nrow)
    m = GwfDisModel(1, nrow, ncol, delr, delc, np.full(n, 25.0), f["bottom"].ravel().copy(),
                    np.ones(n), np.ones(n), np.ones(n, np.int32), np.full(n, 7.5),
                    inewton=1, inewtonur=1, name="ex-gwf-bump")
    m.chd_node = np.concatenate([np.arange(nrow) * ncol, np.arange(nrow) * ncol + ncol - 1]).astype(np.int32)
    m.chd_head = np.concatenate([np.full(nrow, 7.5), np.full(nrow, 2.5)])
    return m, f["heads"].ravel()


def test_newton_under_relaxation_bump_matches_mf6_heads():
    """The oracle against heads written by MODFLOW 6 itself, with the
    reference test's own check (np.allclose)."""
    m, mf6_heads = bump_model()
    g = oracle.Gwf(m, oracle.settings(**BUMP_IMS))
    st = g.timestep(kper=1, kstp=1, delt=1.0, transient=False, **BUMP_OUTER)
    assert st["converged"] == 1
    assert np.allclose(mf6_heads, g.x)
    # closer than np.allclose asks: a few OUTER_DVCLOSE
    assert np.max(np.abs(g.x - mf6_heads)) <= 5e-8
    # the dry cells of the bump sit on their bottom, as in the file
    dry = mf6_heads - m.botm < 1e-6
    assert dry.sum() > 100 and np.all(g.x[dry] - m.botm[dry] < 1e-6)


def test_bump_needs_newton_under_relaxation():
    """Without NEWTON UNDER_RELAXATION (gwf_nur runs only with it,
    gwf.f90:717) the same model does not close in 75 outer iterations, so
    the option is what the known answer depends on."""
    m, mf6_heads = bump_model()
    m.inewtonur = 0
    g = oracle.Gwf(m, oracle.settings(**BUMP_IMS))
    st = g.timestep(kper=1, kstp=1, delt=1.0, transient=False, **BUMP_OUTER)
    assert st["converged"] == 0
    assert not np.allclose(mf6_heads, g.x)
