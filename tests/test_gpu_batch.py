"""Batched ensembles (gbims_batch_*) against the oracle, member by member.

Each member of a small seeded ensemble is solved alone by the oracle's IMS;
the batch solves all of them at once.  Every member must reach its own
closure with PCG parity (heads within 0.1 x INNER_DVCLOSE, inner-iteration
counts within 2 or 10 %), and the GPU NPF fill of a member must equal the
oracle's assembly bit for bit.
"""
import numpy as np
import pytest

import oracle
from modflow6_gb300 import _lib
from modflow6_gb300.ensemble import (EnsembleLinear, assemble_member, concat_systems,
                                     initial_heads, make_ensemble)
from modflow6_gb300.ims import ImsLinearSettings
from test_gpu_ims import assert_closure_parity, iters_close, tight_solution

pytestmark = pytest.mark.gpu

TOL = dict(dvclose=1e-8, rclose=1e-6, iter1=1000)


def oracle_member(m):
    g = oracle.Gwf(m, oracle.settings())
    x0 = initial_heads(m)
    amat, rhs = g.assemble(x0)
    amat, rhs = g.fixups(amat, rhs, x0, isymmetric=True)
    return g.con, amat, rhs, x0


def test_member_assembly_matches_oracle(gblib):
    for m in make_ensemble(3, seed=21, scale=0.08):
        con, amat, rhs, x0 = assemble_member(m)
        _, ao, ro, _ = oracle_member(m)
        np.testing.assert_array_equal(amat, ao)
        np.testing.assert_array_equal(rhs, ro)


@pytest.mark.parametrize("wavefront", [False, True], ids=["levels", "wavefront"])
@pytest.mark.parametrize("count,seed,scale", [(1, 5, 0.1), (7, 11, 0.1), (24, 40, 0.05)])
def test_batch_members_match_oracle(gblib, count, seed, scale, wavefront):
    members = make_ensemble(count, seed=seed, scale=scale)
    systems = [oracle_member(m) for m in members]
    cons = [s[0] for s in systems]
    mrow, ia, ja, amat, rhs, x = concat_systems(cons, [s[1] for s in systems],
                                                [s[2] for s in systems], [s[3] for s in systems])
    shapes = [(m.nlay, m.nrow, m.ncol) for m in members] if wavefront else None
    ens = EnsembleLinear(ImsLinearSettings(**TOL)).allocate(mrow, ia, ja, shapes)
    res = ens.apply(amat.copy(), rhs.copy(), x)
    assert len(res) == count
    for i, (con, am, rh, x0) in enumerate(systems):
        o = oracle.Ims(oracle.settings(**TOL), con["ia"], con["ja"])
        xo = x0.copy()
        icnvg_o, it_o, _ = o.apply(am.copy(), rh.copy(), xo)
        xm = x[mrow[i]:mrow[i + 1]]
        assert res[i].icnvg == icnvg_o == 1, (i, res[i])
        assert res[i].summary["structured"] == int(wavefront)
        assert iters_close(res[i].in_iter, it_o), (i, res[i].in_iter, it_o)
        if not wavefront and np.max(np.abs(xm - xo)) <= 0.1 * TOL["dvclose"]:
            continue  # the reference's sweep order: the PCG iterates agree
        # The batch sums each member's dot products chunk by chunk, another
        # order than the single-model reductions; on the stiffer members
        # (sigma_lnK up to 2) that moves the iterates by more than
        # 0.1 x INNER_DVCLOSE.  The result must then be as accurate as the
        # oracle's own, measured against a tightly converged solution.
        x_star = tight_solution(con, am, rh, x0, 1)
        assert_closure_parity(xm, xo, x_star, TOL["dvclose"], False)
    ens.close()


def test_batch_rejects_coupled_members(gblib):
    # two 2-row "members" whose rows reference each other
    ia = np.array([0, 2, 4, 6, 8], np.int32)
    ja = np.array([0, 2, 1, 0, 2, 1, 3, 2], np.int32)
    with pytest.raises(_lib.GbimsError) as e:
        EnsembleLinear(ImsLinearSettings(**TOL)).allocate(np.array([0, 2, 4], np.int32), ia, ja)
    assert e.value.status == _lib.GBIMS_ERR_ARG


@pytest.mark.parametrize("wavefront", [False, True], ids=["levels", "wavefront"])
def test_batch_mixed_members_reach_closure(gblib, wavefront):
    """The batched mixed form (FP32 matrix, factors and inner vectors, FP64
    refinement per member): every member reaches its own FP64 closure,
    its FP64 true residual meets INNER_RCLOSE, and its heads are as accurate
    as the FP64 single solve's (5x the oracle's error plus INNER_DVCLOSE,
    against a tightly converged solution); members refine independently."""
    members = make_ensemble(7, seed=11, scale=0.1)
    systems = [oracle_member(m) for m in members]
    cons = [s[0] for s in systems]
    mrow, ia, ja, amat, rhs, x = concat_systems(cons, [s[1] for s in systems],
                                                [s[2] for s in systems], [s[3] for s in systems])
    shapes = [(m.nlay, m.nrow, m.ncol) for m in members] if wavefront else None
    ens = EnsembleLinear(ImsLinearSettings(precision=_lib.GBIMS_MIXED, **TOL)).allocate(
        mrow, ia, ja, shapes)
    res = ens.apply(amat.copy(), rhs.copy(), x)
    refinements = []
    for i, (con, am, rh, x0) in enumerate(systems):
        o = oracle.Ims(oracle.settings(**TOL), con["ia"], con["ja"])
        xo = x0.copy()
        icnvg_o, it_o, _ = o.apply(am.copy(), rh.copy(), xo)
        xm = x[mrow[i]:mrow[i + 1]]
        assert res[i].icnvg == 1, (i, res[i])
        resid = rh - oracle.amux(con["ia"], con["ja"], am, xm)
        assert np.max(np.abs(resid)) <= TOL["rclose"] * 1.0001, i
        x_star = tight_solution(con, am, rh, x0, 1)
        assert_closure_parity(xm, xo, x_star, TOL["dvclose"], False)
        refinements.append(res[i].summary["refinements"])
    assert max(refinements) >= 1
    ens.close()
