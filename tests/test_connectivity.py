"""The vectorised DIS connectivity of the product equals the oracle's loop
restatement of Connections.f90:463-698 (disconnections) + fillisym/filljas."""
import numpy as np
import pytest

import oracle
from modflow6_gb300.dis import dis_connections, make_config


@pytest.mark.parametrize("shape", [(1, 1, 7), (1, 5, 1), (3, 1, 1), (2, 3, 4), (3, 7, 5), (1, 2, 2)])
def test_dis_connections_match_oracle(shape):
    nlay, nrow, ncol = shape
    rng = np.random.default_rng(1)
    delr = rng.uniform(1, 3, ncol)
    delc = rng.uniform(1, 3, nrow)
    nrc = nrow * ncol
    top = np.full(nrc, 10.0)
    botm = np.concatenate([np.full(nrc, 10.0 - 2.0 * (k + 1)) - rng.uniform(0, 0.5, nrc) for k in range(nlay)])
    cell_top = np.concatenate([top, botm[:-nrc]]) if nlay > 1 else top
    a = dis_connections(nlay, nrow, ncol, delr, delc, cell_top, botm)
    b = oracle.dis_connect(nlay, nrow, ncol, delr, delc, cell_top, botm)
    for key in ("ia", "ja", "isym", "jas", "ihc"):
        np.testing.assert_array_equal(a[key], b[key], err_msg=key)
    for key in ("cl1", "cl2", "hwva"):
        np.testing.assert_array_equal(a[key], b[key], err_msg=key)
    assert a["nja"] == b["nja"] and a["njas"] == b["njas"]


def test_config_c1_shapes():
    m = make_config("c1", seed=0)
    con = m.connections()
    assert m.nodes == 10_000 and con["nja"] == 49_600 and con["njas"] == 19_800


def test_config_c2_small_shapes():
    m = make_config("c2", seed=0, scale=0.02)
    con = m.connections()
    assert con["nja"] == m.nodes + 2 * con["njas"]
    assert np.all(m.wel_q < -50) and np.all(m.wel_q > -500)
