"""The oracle's cell-by-cell flows and model budget (gwf_cq / gwf_bd
restated in oracle/gwf_oracle.c) on cases with a known answer: the
chd01 autotest (autotest/test_gwf_chd01.py: 100 cells between CHD 1 and 0,
K = 1, unit faces) carries 1/99 through every face, and the budget of a
converged steady solve closes."""
import numpy as np

import oracle
from modflow6_gb300.dis import make_config
from test_oracle_known_answers import chd01_model


def test_chd01_budget_known_answer():
    m = chd01_model()
    g = oracle.Gwf(m, oracle.settings(dvclose=1e-10, rclose=1e-10, iter1=300, ilinmeth=1))
    st = g.timestep(kper=1, kstp=1, delt=1.0, dvclose=1e-10, mxiter=20)
    assert st["converged"] == 1
    fj, b = g.budget(g.x)
    ia, ja, isym = g.con["ia"], g.con["ja"], g.con["isym"]
    off = np.ones(fj.size, bool)
    off[ia[:-1]] = False
    # FLOW-JA-FACE is antisymmetric: q(n->m) = -q(m->n)
    np.testing.assert_array_equal(fj[off], -fj[isym[off]])
    # every face carries K A dh/dx = 1/99 from column 1 toward column 100
    rows = np.repeat(np.arange(m.nodes), np.diff(ia))
    east = off & (ja > rows)
    np.testing.assert_allclose(-fj[east], 1.0 / 99.0, rtol=1e-8)
    assert np.isclose(b["rate_in"][2], 1.0 / 99.0, rtol=1e-8)
    assert np.isclose(b["rate_out"][2], 1.0 / 99.0, rtol=1e-8)
    assert abs(b["percent_discrepancy"]) < 1e-6
    # the interior cells balance: their FLOW-JA-FACE diagonal is their net flow
    assert b["max_cell_imbalance"] < 1e-9


def test_c1_budget_closes():
    """C1 (recharge over the grid, CHD on two sides): recharge in equals CHD
    out less CHD in, to the closure of the solve."""
    m = make_config("c1", seed=0)
    g = oracle.Gwf(m, oracle.settings(dvclose=1e-8, rclose=1e-6, iter1=1000))
    st = g.timestep(kper=1, kstp=1, delt=1.0, dvclose=1e-8, mxiter=10)
    assert st["converged"] == 1
    _, b = g.budget(g.x)
    rch_in = b["rate_in"][4]
    assert np.isclose(rch_in, 1e-4 * 100.0 * (m.nodes - m.chd_node.size), rtol=1e-12)
    assert np.isclose(b["rate_out"][2] - b["rate_in"][2], rch_in, rtol=1e-6)
    assert abs(b["percent_discrepancy"]) < 1e-5
