"""REORDERING_METHOD RCM and MD on the CPU: the library's numberings
(gbims_calc_order, host code) against the oracle's restatements of genrcm
(rcm/rcm.f90) and of the Yale minimum-degree ordering (ImsReordering.f90),
and the oracle's reordered IMS solves against natural order -- the property
the reference's own test checks (autotest/test_gwf_ims_rcm_reorder.py: the
same budgets with and without RCM, ILUT level 10, drop tolerance 1e-6).
The reference commits no orderings, so the numberings are pinned by the two
restatements agreeing and by what the orderings are for (RCM's bandwidth,
MD's fill).
"""
import shutil

import numpy as np
import pytest

import oracle
from modflow6_gb300.dis import GwfDisModel, make_config


def lib_or_skip():
    from modflow6_gb300 import _lib
    if not _lib.LIB_PATH.exists():
        if shutil.which("nvcc") is None:
            pytest.skip("library not built and nvcc not available")
        from modflow6_gb300 import build
        build.build()
    return _lib


def pattern(name, scale=1.0, seed=0):
    g = oracle.Gwf(make_config(name, seed=seed, scale=scale), oracle.settings())
    return g.con["ia"], g.con["ja"]


def grid_pattern(nlay, nrow, ncol):
    con = oracle.dis_connect(nlay, nrow, ncol, np.ones(ncol), np.ones(nrow), np.zeros(nrow * ncol),
                             -np.arange(1, nlay + 1, dtype=float).repeat(nrow * ncol))
    return con["ia"], con["ja"]


def disconnected_pattern():
    """Two grids side by side (the second numbered first in part) and three
    isolated nodes: several components, each numbered on its own."""
    ia1, ja1 = grid_pattern(1, 4, 7)
    ia2, ja2 = grid_pattern(2, 3, 3)
    n1, n2 = ia1.size - 1, ia2.size - 1
    rows = [list(ja2[ia2[r]:ia2[r + 1]] + 2) for r in range(n2)]
    rows = [[0], [1]] + rows + [list(ja1[ia1[r]:ia1[r + 1]] + 2 + n2) for r in range(n1)] + [[2 + n1 + n2]]
    ia = np.cumsum([0] + [len(r) for r in rows]).astype(np.int32)
    ja = np.concatenate([np.array(r, np.int32) for r in rows])
    return ia, ja


def lib_order(_lib, ia, ja, base=0):
    n = ia.size - 1
    lo, io = np.zeros(n, np.int32), np.zeros(n, np.int32)
    iab = np.ascontiguousarray(ia + base, np.int32)  # kept alive across the call
    jab = np.ascontiguousarray(ja + base, np.int32)
    rc = _lib.load().gbims_calc_order(1, n, int(ia[-1]), _lib.iptr(iab), _lib.iptr(jab), base,
                                      _lib.iptr(lo), _lib.iptr(io))
    assert rc == 0
    return lo - base, io - base


CASES = {
    "c1": lambda: pattern("c1"),
    "c2-small": lambda: pattern("c2", 0.05, 3),
    "c3-small": lambda: pattern("c3", 0.04, 1),
    "rcm-autotest-grid": lambda: grid_pattern(2, 5, 30),
    "disconnected": disconnected_pattern,
}


@pytest.mark.parametrize("name", list(CASES))
def test_library_rcm_matches_oracle(name):
    _lib = lib_or_skip()
    ia, ja = CASES[name]()
    lo_ref = oracle.genrcm(ia, ja)
    assert np.array_equal(np.sort(lo_ref), np.arange(ia.size - 1))
    lo, io = lib_order(_lib, ia, ja)
    np.testing.assert_array_equal(lo, lo_ref)
    np.testing.assert_array_equal(io[lo], np.arange(ia.size - 1))
    lo1, _ = lib_order(_lib, ia, ja, base=1)  # Fortran indexing gives the same numbering
    np.testing.assert_array_equal(lo1, lo_ref)


def test_rcm_numbering_reduces_the_profile():
    """The RCM list itself is a bandwidth-reducing numbering of the
    2 x 5 x 30 grid (natural bandwidth 150 -> RCM's at most 10)."""
    ia, ja = grid_pattern(2, 5, 30)
    lo = oracle.genrcm(ia, ja)
    pos = np.empty_like(lo)
    pos[lo] = np.arange(lo.size)
    rows = np.repeat(np.arange(ia.size - 1), np.diff(ia))
    assert np.max(np.abs(rows - ja)) == 150
    assert np.max(np.abs(pos[rows] - pos[ja])) <= 10


def test_reordered_solve_matches_natural_order():
    """The reference's reorder test in the oracle: ILUT level 10, drop
    tolerance 1e-6, inner closure 1e-12 -- the heads with and without RCM."""
    nlay, nrow, ncol = 2, 5, 30
    m = GwfDisModel(nlay, nrow, ncol, np.full(ncol, 100.0), np.full(nrow, 100.0),
                    np.zeros(nrow * ncol), np.concatenate([np.full(nrow * ncol, -10.0),
                                                           np.full(nrow * ncol, -20.0)]),
                    np.ones(nlay * nrow * ncol), np.ones(nlay * nrow * ncol),
                    np.zeros(nlay * nrow * ncol, np.int32), np.zeros(nlay * nrow * ncol))
    m.chd_node = np.array([r * ncol for r in range(nrow)] + [r * ncol + ncol - 1 for r in range(nrow)],
                          np.int32)
    m.chd_head = np.array([10.0] * nrow + [5.0] * nrow)
    heads = []
    for iord in (0, 1):
        s = oracle.settings(dvclose=1e-12, rclose=1e-6, iter1=100, ilinmeth=2, iord=iord, level=10,
                            droptol=1e-6)
        g = oracle.Gwf(m, s)
        st = g.timestep(kper=1, kstp=1, delt=1.0, transient=False, dvclose=1e-9, mxiter=100)
        assert st["converged"] == 1
        heads.append(g.x.copy())
    assert np.max(np.abs(heads[0] - heads[1])) <= 1e-9


# -- REORDERING_METHOD MD (ImsReordering.f90: the Yale minimum-degree ordering)

def lib_md_order(_lib, ia, ja):
    n = ia.size - 1
    lo, io = np.zeros(n, np.int32), np.zeros(n, np.int32)
    iab = np.ascontiguousarray(ia, np.int32)
    jab = np.ascontiguousarray(ja, np.int32)
    rc = _lib.load().gbims_calc_order(2, n, int(ia[-1]), _lib.iptr(iab), _lib.iptr(jab), 0,
                                      _lib.iptr(lo), _lib.iptr(io))
    assert rc == 0
    return lo, io


@pytest.mark.parametrize("name", list(CASES))
def test_library_md_matches_oracle(name):
    _lib = lib_or_skip()
    ia, ja = CASES[name]()
    lo_ref = oracle.genmd(ia, ja)
    assert np.array_equal(np.sort(lo_ref), np.arange(ia.size - 1))
    lo, io = lib_md_order(_lib, ia, ja)
    np.testing.assert_array_equal(lo, lo_ref)
    np.testing.assert_array_equal(io[lo], np.arange(ia.size - 1))


def test_md_numbering_cuts_the_fill():
    """Eliminating in the MD list's order fills far less than the natural
    order (symbolic LU of the 2 x 5 x 30 grid and of c1)."""
    scipy_linalg = pytest.importorskip("scipy.sparse.linalg")
    import scipy.sparse as sp
    for ia, ja in (grid_pattern(2, 5, 30), pattern("c1")):
        n = ia.size - 1
        A = sp.csr_matrix((np.ones(ja.size), ja, ia), shape=(n, n)) + 10.0 * sp.eye(n)
        lo = oracle.genmd(ia, ja)

        def fill(M):
            f = scipy_linalg.splu(M.tocsc(), permc_spec="NATURAL", diag_pivot_thresh=0.0,
                                  options=dict(SymmetricMode=True))
            return f.L.nnz + f.U.nnz
        assert fill(A[lo][:, lo]) < 0.25 * fill(A)


def test_md_reordered_solve_matches_natural_order():
    """As the reference's reorder test, with MD: ILUT level 10 / 1e-6, the
    heads with and without the ordering agree."""
    from test_gpu_ims import c1_system  # the oracle-assembled c1 system (no GPU involved)
    con, amat, rhs, x0 = c1_system(isym=False)
    xs = []
    for iord in (0, 2):
        s = oracle.settings(dvclose=1e-10, rclose=1e-8, iter1=2000, ilinmeth=2, iord=iord,
                            level=10, droptol=1e-6)
        ims = oracle.Ims(s, con["ia"], con["ja"])
        x = x0.copy()
        icnvg, it, _ = ims.apply(amat.copy(), rhs.copy(), x)
        assert icnvg == 1
        xs.append(x)
    assert np.max(np.abs(xs[0] - xs[1])) <= 1e-7


def test_calc_order_rejects_bad_arguments():
    _lib = lib_or_skip()
    lib = _lib.load()
    ia, ja = grid_pattern(1, 3, 3)
    n = ia.size - 1
    lo, io = np.zeros(n, np.int32), np.zeros(n, np.int32)

    def call(iord, ia_, ja_, nja=None, base=0):
        iab = np.ascontiguousarray(ia_, np.int32)
        jab = np.ascontiguousarray(ja_, np.int32)
        return lib.gbims_calc_order(iord, n, int(ia_[-1]) - base if nja is None else nja,
                                    _lib.iptr(iab), _lib.iptr(jab), base, _lib.iptr(lo),
                                    _lib.iptr(io))

    assert call(1, ia, ja) == 0 and call(2, ia, ja) == 0
    assert call(3, ia, ja) == _lib.GBIMS_ERR_ARG                     # no such ordering
    bad = ja.copy()
    bad[3] = n                                                         # column out of range
    assert call(1, ia, bad) == _lib.GBIMS_ERR_ARG
    assert call(1, ia, ja, nja=int(ia[-1]) - 1) == _lib.GBIMS_ERR_ARG  # ia inconsistent with nja
    assert call(1, ia + 1, ja + 1, base=1) == 0                         # 1-based input
    assert call(1, ia + 2, ja + 2, base=2) == _lib.GBIMS_ERR_ARG        # index_base neither 0 nor 1
