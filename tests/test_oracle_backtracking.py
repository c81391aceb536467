"""The oracle's sln_backtracking (NumericalSolution.f90:2680-2838): on a
transient Newton case whose residual rises between outer iterations it cuts
steps by BREDUC and still reaches the outer closure; with
BACKTRACKING_NUMBER 0 it never does, and on a case whose residual falls
monotonically (autotest newton01) the options change nothing."""
import numpy as np

import oracle
from modflow6_gb300.dis import make_config
from test_oracle_known_answers import newton01_model

COMPLEX_BT = dict(numtrack=20, btol=1.05, breduc=0.1, res_lim=0.002)


def run_c3(bt):
    m = make_config("c3", seed=1, scale=0.04)
    m.wel_q = m.wel_q * 0.2
    g = oracle.Gwf(m, oracle.settings(dvclose=1e-6, rclose=1e-3, iter1=500, ilinmeth=2))
    delt, out = 10.0, []
    for kstp in range(1, 4):
        out.append(g.timestep(kper=1, kstp=kstp, delt=delt, transient=True, dvclose=1e-5,
                              mxiter=100, nonmeth=3, theta=0.8, akappa=1e-4, gamma=0.0, **bt))
        delt *= 1.2
    return out, g.x.copy()


def test_backtracking_cuts_steps_and_converges():
    st, x = run_c3(COMPLEX_BT)
    assert all(s["converged"] == 1 for s in st)
    assert sum(s["backtracks"] for s in st) > 0
    st0, x0 = run_c3(dict(numtrack=0, btol=0.0, breduc=0.0, res_lim=0.0))
    assert all(s["converged"] == 1 for s in st0)
    assert sum(s["backtracks"] for s in st0) == 0
    # both paths reach the same closure
    assert np.max(np.abs(x - x0)) <= 1e-3


def test_backtracking_inert_on_monotone_case():
    res = []
    for bt in (dict(numtrack=0), COMPLEX_BT):
        m = newton01_model()
        g = oracle.Gwf(m, oracle.settings(dvclose=1e-9, rclose=0.1, iter1=500, ilinmeth=2, north=2))
        st = g.timestep(kper=1, kstp=1, delt=1.0, dvclose=1e-9, mxiter=100, nonmeth=3, theta=0.8,
                        akappa=1e-4, gamma=0.0, **bt)
        res.append((st, g.x.copy()))
    assert res[1][0]["backtracks"] == 0
    assert res[0][0]["outer"] == res[1][0]["outer"]
    np.testing.assert_array_equal(res[0][1], res[1][1])
    assert np.isclose(res[1][1][4], 8.0) and np.isclose(res[1][1][13], 7.0)
