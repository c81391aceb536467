"""The precomputed sln_ls loose ends (LsFixups) equal the per-call restatement
(sln_ls_fixups) and the oracle's (NumericalSolution.f90:2434-2478) bit for
bit, with CHD rows, tiny diagonals and both symmetric and nonsymmetric
accelerators."""
import numpy as np
import pytest

import oracle
from modflow6_gb300.dis import make_config
from modflow6_gb300.solution import LsFixups, sln_ls_fixups


@pytest.mark.parametrize("name,scale", [("c1", 1.0), ("c2", 0.03), ("c3", 0.04)])
@pytest.mark.parametrize("isym", [True, False])
def test_fixups_agree(name, scale, isym):
    m = make_config(name, seed=5, scale=scale)
    if m.chd_node.size == 0:
        m.chd_node = np.array([0, 7, m.nodes - 1], np.int32)
        m.chd_head = np.array([3.0, 2.0, 1.0])
    g = oracle.Gwf(m, oracle.settings())
    rng = np.random.default_rng(1)
    x = m.strt + rng.uniform(-1, 1, m.nodes)
    x[m.chd_node] = m.chd_head
    amat, rhs = g.assemble(x)
    # a few active rows with a vanishing diagonal
    act = np.flatnonzero(m.ibound > 0)[:5]
    amat[g.con["ia"][act]] = 1e-17
    a1, r1 = sln_ls_fixups(g.con["ia"], g.con["ja"], m.ibound, amat, rhs, x, isymmetric=isym)
    fx = LsFixups(g.con["ia"], g.con["ja"], m.ibound, isymmetric=isym)
    a2, r2 = fx.apply(amat.copy(), rhs.copy(), x)
    np.testing.assert_array_equal(a1, a2)
    np.testing.assert_array_equal(r1, r2)
    a3, r3 = g.fixups(amat.copy(), rhs.copy(), x.copy(), isymmetric=isym)
    np.testing.assert_array_equal(a2, a3)
    np.testing.assert_array_equal(r2, r3)
