"""The oracle's per-inner-iteration records with several models (CONVNMOD,
CONVMODSTART; ImsLinearBase.f90:141-197 for PCG, :431-493 for BiCGSTAB):
the largest head change and residual of each model, and their rows, are
consistent with the whole system's (the model holding the overall maximum
reports it), and a single model reproduces the overall values."""
import numpy as np
import pytest

import oracle
from modflow6_gb300.dis import make_config


def c1_system():
    m = make_config("c1", seed=0)
    g = oracle.Gwf(m, oracle.settings())
    x0 = g.x.copy()
    x0[m.chd_node] = m.chd_head
    amat, rhs = g.assemble(x0)
    amat, rhs = g.fixups(amat, rhs, x0, isymmetric=True)
    return g.con, amat, rhs, x0


@pytest.mark.parametrize("ilinmeth", [1, 2])
@pytest.mark.parametrize("modstart", [[0, 10000], [0, 2500, 6100, 10000]])
def test_model_records_consistent(ilinmeth, modstart):
    con, amat, rhs, x0 = c1_system()
    ims = oracle.Ims(oracle.settings(dvclose=1e-8, rclose=1e-6, iter1=400, ilinmeth=ilinmeth),
                     con["ia"], con["ja"])
    nrec = 400
    ims.set_models(modstart, nrec)
    icnvg, it, recs = ims.apply(amat.copy(), rhs.copy(), x0.copy(), nrec=nrec)
    assert icnvg == 1 and len(recs) == it
    mr = ims.model_records(it)
    ms = np.array(modstart)
    for k, r in enumerate(recs):
        for key, lkey, g, gl in (("dvmax", "locdv", r["dvmax"], r["locdv"]),
                                 ("rmax", "locr", r["rmax"], r["locr"])):
            v, loc = mr[key][k], mr[lkey][k]
            # each model's row lies in the model
            for im in range(ms.size - 1):
                assert ms[im] <= loc[im] < ms[im + 1]
            # the model holding the overall maximum reports it
            im = int(np.searchsorted(ms, gl, side="right") - 1)
            assert v[im] == g and loc[im] == gl
            assert np.all(np.abs(v) <= abs(g))
