"""The oracle's ILUT restatement (sparskit2/ilut.f90 as vendored in MODFLOW 6)
against what the routine documents, on the CPU.  The reference's tests pin
it through newton01 under the COMPLEX preset
(tests/test_oracle_known_answers.py); these check the documented behaviour
directly:

* with nothing dropped (lfil >= the fill, droptol 0) the factor is the exact
  LU, so one application solves A z = b;
* each row keeps at most lfil L entries and lfil - 1 U entries (the copy
  loop of ilut.f90:380-385 stores ilen - 1 U entries), L columns below the
  row, U columns above it, both in the storage that lusol reads;
* every kept multiplier exceeds DROP_TOLERANCE and every kept U entry
  exceeds DROP_TOLERANCE x the row's mean |a| (ilut.f90:268, 363);
* the pivot guard retries with the delta sequence of ims_base_pcu.
"""
import numpy as np
import pytest

import oracle
from test_rcm_order import grid_pattern


def grid_system(nlay, nrow, ncol, seed=0):
    ia, ja = grid_pattern(nlay, nrow, ncol)
    rng = np.random.default_rng(seed)
    n = ia.size - 1
    a = np.zeros(ja.size)
    for r in range(n):
        off = [k for k in range(ia[r], ia[r + 1]) if ja[k] != r]
        a[off] = -(0.5 + rng.random(len(off)))
        a[ia[r]] = -a[off].sum() + (1.0 if r % 7 == 0 else 0.01)
    return ia, ja, a


def dense(ia, ja, a):
    n = ia.size - 1
    A = np.zeros((n, n))
    for r in range(n):
        A[r, ja[ia[r]:ia[r + 1]]] = a[ia[r]:ia[r + 1]]
    return A


def test_no_dropping_gives_the_exact_lu():
    ia, ja, a = grid_system(2, 6, 7)
    n = ia.size - 1
    iapc, japc, apc, retries = oracle.ilut(ia, ja, a, n, 0.0)
    assert retries == 0
    b = np.random.default_rng(1).standard_normal(n)
    z = oracle.ilu0a(apc, iapc, japc, b)
    A = dense(ia, ja, a)
    assert np.linalg.norm(A @ z - b) <= 1e-12 * np.linalg.norm(b) * np.linalg.cond(A)


@pytest.mark.parametrize("lfil,droptol", [(1, 0.0), (3, 1e-3), (5, 1e-4), (8, 1e-2), (0, 1e-3)])
def test_caps_structure_and_thresholds(lfil, droptol):
    ia, ja, a = grid_system(3, 8, 9, seed=lfil)
    n = ia.size - 1
    iapc, japc, apc, _ = oracle.ilut(ia, ja, a, lfil, droptol)
    assert iapc[0] == n + 1
    assert np.all(np.diff(iapc) >= 0)
    for r in range(n):
        lo, mid, hi = iapc[r], japc[r], iapc[r + 1]
        assert lo <= mid <= hi
        assert mid - lo <= lfil and hi - mid <= max(lfil - 1, 0)
        assert np.all(japc[lo:mid] < r) and np.all(japc[mid:hi] > r)
        assert len(set(japc[lo:hi])) == hi - lo
        assert np.all(np.abs(apc[lo:mid]) > droptol)
        tnorm = np.abs(a[ia[r]:ia[r + 1]]).sum() / (ia[r + 1] - ia[r])
        assert np.all(np.abs(apc[mid:hi]) > droptol * tnorm)
        assert apc[r] != 0.0 and np.isfinite(apc[r])


def test_kept_u_entries_are_the_largest():
    """qsplit keeps the lfil - 1 largest U candidates of a row: with lfil = 2
    every row keeps its single largest candidate.  On a tridiagonal matrix
    with no fill, each row's only U candidate is its upper neighbour."""
    n = 9
    rows = [[r] + [c for c in (r - 1, r + 1) if 0 <= c < n] for r in range(n)]
    ia = np.cumsum([0] + [len(x) for x in rows]).astype(np.int32)
    ja = np.concatenate([np.array(x, np.int32) for x in rows])
    a = np.where(np.repeat(np.arange(n), np.diff(ia)) == ja, 4.0, -1.0)
    iapc, japc, apc, _ = oracle.ilut(ia, ja, a, 2, 0.0)
    for r in range(n - 1):
        assert list(japc[japc[r]:iapc[r + 1]]) == [r + 1]
        np.testing.assert_equal(apc[japc[r]:iapc[r + 1]], [-1.0])


def test_pivot_guard_retries_with_the_pcu_sequence():
    # [[1,1,0],[1,1,1],[0,1,3]]: row 1 eliminates to a zero pivot at delta 0;
    # the first retry (delta 1e-3) scales row 0's pivot and succeeds
    ia = np.array([0, 2, 5, 7], np.int32)
    ja = np.array([0, 1, 1, 0, 2, 2, 1], np.int32)
    a = np.array([1.0, 1.0, 1.0, 1.0, 1.0, 3.0, 1.0])
    iapc, japc, apc, retries = oracle.ilut(ia, ja, a, 2, 0.0)
    assert retries == 1
    np.testing.assert_equal(apc[0], 1.0 / (1.001 * 1.0))
