"""Structured 7-point wavefront sweeps (DIS grids) against the oracle.

The sweeps sum each cell's terms in another order than ilu0a (the lane's own
line first), the backward sweep uses inverse-pivot-scaled upper factors, and
the FP64 form computes in df64 (pairs of floats, about 48 significant bits)
when the factor lies in the float exponent range: all equal to ilu0a in exact
arithmetic, so the preconditioner output is compared at 1e-12 relative to its
scale, and solves at closure (heads within 0.1 x INNER_DVCLOSE of the
oracle's IMS solve).
"""
import os
import numpy as np
import pytest

import oracle
from modflow6_gb300 import _lib
from modflow6_gb300.dis import GwfDisModel, lognormal_field, make_config
from modflow6_gb300.ims import ImsLinear, ImsLinearSettings
from test_gpu_ims import assert_closure_parity

pytestmark = pytest.mark.gpu


def dis_system(nlay, nrow, ncol, seed=0, isym=True):
    rng = np.random.default_rng(seed)
    nrc = nrow * ncol
    n = nlay * nrc
    k = np.exp(rng.normal(0.0, 1.0, n))
    m = GwfDisModel(nlay, nrow, ncol, np.full(ncol, 10.0), np.full(nrow, 10.0),
                    np.full(nrc, 10.0 * nlay), np.repeat(10.0 * (nlay - 1 - np.arange(nlay)), nrc),
                    k, 0.1 * k, np.zeros(n, np.int32), np.full(n, 5.0))
    m.chd_node = np.array([0], np.int32)
    m.chd_head = np.array([1.0])
    m.wel_node = np.array([n - 1], np.int32)
    m.wel_q = np.array([-3.0])
    g = oracle.Gwf(m, oracle.settings())
    x0 = g.x.copy()
    x0[m.chd_node] = m.chd_head
    amat, rhs = g.assemble(x0)
    amat, rhs = g.fixups(amat, rhs, x0, isymmetric=isym)
    return m, g.con, amat, rhs, x0


SHAPES = [(1, 1, 7), (3, 1, 1), (1, 5, 1), (2, 3, 4), (1, 33, 5), (2, 65, 3), (3, 40, 41), (10, 70, 64)]


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_structured_precondition_matches_oracle(gblib, shape):
    m, con, amat, rhs, x0 = dis_system(*shape)
    ims = ImsLinear(ImsLinearSettings(structure=shape)).imslinear_allocate(m.nodes, con["ia"], con["ja"])
    assert gblib.gbims_factor(ims._h, _lib.dptr(amat), None) == 0
    v = np.random.default_rng(5).standard_normal(m.nodes)
    z = np.zeros_like(v)
    assert gblib.gbims_precondition(ims._h, _lib.dptr(v), _lib.dptr(z)) == 0
    o = oracle.Ims(oracle.settings(), con["ia"], con["ja"])
    o.apply(amat.copy(), rhs.copy(), x0.copy())
    zo = oracle.ilu0a(o.apc(), o.iapc(), o.japc(), v, fma=True)
    scale = np.max(np.abs(zo))
    assert np.max(np.abs(z - zo)) <= 1e-12 * scale


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_structured_matvec_bitexact(gblib, shape):
    """The index-free product of a full DIS grid sums every CSR row in JA
    order with FMA, exactly like amux."""
    m, con, amat, rhs, x0 = dis_system(*shape)
    ims = ImsLinear(ImsLinearSettings(structure=shape)).imslinear_allocate(m.nodes, con["ia"], con["ja"])
    assert gblib.gbims_factor(ims._h, _lib.dptr(amat), None) == 0
    v = np.random.default_rng(6).standard_normal(m.nodes)
    y = np.zeros_like(v)
    assert gblib.gbims_matvec(ims._h, _lib.dptr(v), _lib.dptr(y)) == 0
    np.testing.assert_array_equal(y, oracle.amux_fma(con["ia"], con["ja"], amat, v))


@pytest.mark.parametrize("ilinmeth", [1, 2])
@pytest.mark.parametrize("precision", [_lib.GBIMS_FP64, _lib.GBIMS_MIXED])
def test_structured_solve_c2_small(gblib, ilinmeth, precision):
    m = make_config("c2", seed=4, scale=0.06)
    g = oracle.Gwf(m, oracle.settings())
    x0 = g.x.copy()
    x0[m.chd_node] = m.chd_head
    amat, rhs = g.assemble(x0)
    amat, rhs = g.fixups(amat, rhs, x0, isymmetric=(ilinmeth == 1))
    tol = dict(dvclose=1e-8, rclose=1e-4, iter1=2000)
    o = oracle.Ims(oracle.settings(ilinmeth=ilinmeth, **tol), g.con["ia"], g.con["ja"])
    xo = x0.copy()
    icnvg_o, it_o, _ = o.apply(amat.copy(), rhs.copy(), xo)
    s = ImsLinearSettings(ilinmeth=ilinmeth, precision=precision,
                          structure=(m.nlay, m.nrow, m.ncol), **tol)
    ims = ImsLinear(s).imslinear_allocate(m.nodes, g.con["ia"], g.con["ja"])
    x = x0.copy()
    r = ims.imslinear_apply(amat.copy(), rhs.copy(), x)
    assert r.summary["structured"] == 1
    assert r.icnvg == 1 and icnvg_o == 1
    # the structured backward sweep rounds differently from ilu0a, so even
    # PCG stops an iteration or so apart: compare accuracy, not iterates
    ts = oracle.settings(ilinmeth=ilinmeth, dvclose=1e-13, rclose=1e-11, iter1=20000)
    x_star = x0.copy()
    oracle.Ims(ts, g.con["ia"], g.con["ja"]).apply(amat.copy(), rhs.copy(), x_star)
    assert_closure_parity(x, xo, x_star, tol["dvclose"], False)
    if precision == _lib.GBIMS_FP64:
        assert abs(r.in_iter - it_o) <= max(2, int(0.05 * it_o)), (r.in_iter, it_o)


@pytest.mark.parametrize("precision", [_lib.GBIMS_FP64, _lib.GBIMS_MIXED])
@pytest.mark.parametrize("shape", [(2, 65, 3), (3, 40, 41), (4, 97, 150), (2, 256, 40)], ids=lambda s: "x".join(map(str, s)) if isinstance(s, tuple) else str(s))
def test_every_sweep_tiling_gives_the_same_result(gblib, shape, precision):
    """The wavefront tilings (chunk, ring depth, prefetch depth, CTAs per
    SM) the autotuner chooses among compute every cell in the same order:
    the preconditioner output is bit for bit the same under each."""
    import ctypes as C
    m, con, amat, rhs, x0 = dis_system(*shape)
    ims = ImsLinear(ImsLinearSettings(structure=shape, precision=precision)).imslinear_allocate(
        m.nodes, con["ia"], con["ja"])
    assert gblib.gbims_factor(ims._h, _lib.dptr(amat), None) == 0
    v = np.random.default_rng(9).standard_normal(m.nodes)
    ref = None
    t = _lib.GbimsTuning()
    assert gblib.gbims_autotune(ims._h, 2, C.byref(t)) == 0, gblib.gbims_last_error(ims._h)
    assert t.ncandidates >= 2 and 0 <= t.sweep_config < t.ncandidates
    assert all(t.candidate_ms[i] > 0.0 for i in range(t.ncandidates))
    assert 0 <= t.sweep_config_backward < t.ncandidates
    # the chosen pair (each sweep's fastest tiling) timed again: about the
    # best candidate's time or below
    assert t.reduction_blocks > 0 and 0.0 < t.precond_ms <= 1.5 * min(t.candidate_ms[:t.ncandidates])
    for cfg in range(t.ncandidates):
        assert gblib.gbims_set_tuning(ims._h, cfg, 0, -1) == 0
        z = np.zeros_like(v)
        assert gblib.gbims_precondition(ims._h, _lib.dptr(v), _lib.dptr(z)) == 0
        if ref is None:
            ref = z
        else:
            np.testing.assert_array_equal(z, ref)


def test_autotuned_solve_reaches_the_same_closure(gblib):
    import ctypes as C
    shape = (3, 40, 41)
    m, con, amat, rhs, x0 = dis_system(*shape)
    tol = dict(dvclose=1e-9, rclose=1e-7, iter1=2000)
    ims = ImsLinear(ImsLinearSettings(structure=shape, **tol)).imslinear_allocate(m.nodes, con["ia"], con["ja"])
    x1 = x0.copy()
    r1 = ims.imslinear_apply(amat.copy(), rhs.copy(), x1)
    t = _lib.GbimsTuning()
    assert gblib.gbims_autotune(ims._h, 3, C.byref(t)) == 0, gblib.gbims_last_error(ims._h)
    x2 = x0.copy()
    r2 = ims.imslinear_apply(amat.copy(), rhs.copy(), x2)
    assert r1.icnvg == 1 and r2.icnvg == 1
    assert abs(r1.in_iter - r2.in_iter) <= 2
    assert np.max(np.abs(x1 - x2)) <= 0.1 * tol["dvclose"]


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_dis_shape_found_from_the_pattern(gblib, shape):
    """A caller that passes only IA/JA (as imslinear_ar does) reaches the
    wavefront sweeps: the shape is found from the pattern, and the
    preconditioner equals, bit for bit, the one built with the shape given
    (a grid with a dimension of one has the pattern of a smaller-rank grid,
    which sweeps the same cells in the same order)."""
    m, con, amat, rhs, x0 = dis_system(*shape)
    v = np.random.default_rng(6).standard_normal(m.nodes)
    out = []
    for st in (shape, (0, 0, 0)):
        ims = ImsLinear(ImsLinearSettings(structure=st)).imslinear_allocate(m.nodes, con["ia"], con["ja"])
        assert gblib.gbims_factor(ims._h, _lib.dptr(amat), None) == 0
        z = np.zeros_like(v)
        assert gblib.gbims_precondition(ims._h, _lib.dptr(v), _lib.dptr(z)) == 0
        r = ims.imslinear_apply(amat.copy(), rhs.copy(), x0.copy())
        assert r.summary["structured"] == (1 if m.nodes > 1 else 0)
        out.append(z)
    np.testing.assert_array_equal(out[0], out[1])


def test_reduced_pattern_keeps_the_level_sweeps(gblib):
    """A pattern that is not a full DIS grid (one cell cut out, as IDOMAIN
    does) keeps the level-scheduled sweeps; so does structure GENERAL on a
    full grid."""
    from modflow6_gb300.ims import GENERAL
    m, con, amat, rhs, x0 = dis_system(2, 9, 8)
    ia, ja = con["ia"], con["ja"]
    cut = 37
    keep = np.ones(m.nodes, bool)
    keep[cut] = False
    new = np.cumsum(keep) - 1
    rows = []
    for r in np.flatnonzero(keep):
        cols = [new[c] for c in ja[ia[r]:ia[r + 1]] if keep[c]]
        rows.append(cols)
    ia2 = np.concatenate([[0], np.cumsum([len(c) for c in rows])]).astype(np.int32)
    ja2 = np.concatenate(rows).astype(np.int32)
    n2 = keep.sum()
    a2 = np.zeros(ja2.size)
    for r in range(n2):
        a2[ia2[r]] = 6.0
        a2[ia2[r] + 1:ia2[r + 1]] = -1.0
    ims = ImsLinear(ImsLinearSettings(structure=(0, 0, 0))).imslinear_allocate(int(n2), ia2, ja2)
    res = ims.imslinear_apply(a2, np.ones(n2), np.zeros(n2))
    assert res.summary["structured"] == 0
    ims = ImsLinear(ImsLinearSettings(structure=GENERAL)).imslinear_allocate(m.nodes, ia, ja)
    res = ims.imslinear_apply(amat.copy(), rhs.copy(), x0.copy())
    assert res.summary["structured"] == 0


def _precondition(gblib, shape, amat, con, v, native):
    """The wavefront preconditioner applied to v, with df64 or native FP64
    sweeps (GBIMS_SWEEP_NATIVE is read when the handle is created)."""
    old = os.environ.get("GBIMS_SWEEP_NATIVE")
    os.environ["GBIMS_SWEEP_NATIVE"] = "1" if native else "0"
    try:
        ims = ImsLinear(ImsLinearSettings(structure=shape)).imslinear_allocate(
            con["nodes"], con["ia"], con["ja"])
    finally:
        if old is None:
            del os.environ["GBIMS_SWEEP_NATIVE"]
        else:
            os.environ["GBIMS_SWEEP_NATIVE"] = old
    assert gblib.gbims_factor(ims._h, _lib.dptr(amat), None) == 0
    z = np.zeros_like(v)
    assert gblib.gbims_precondition(ims._h, _lib.dptr(v), _lib.dptr(z)) == 0
    return z


@pytest.mark.parametrize("shape", [(1, 33, 5), (3, 40, 41), (10, 70, 64)], ids=lambda s: "x".join(map(str, s)))
def test_df64_and_native_fp64_sweeps_agree(gblib, shape):
    """The df64 sweeps and the native FP64 sweeps give the same
    preconditioner to 1e-12 of its scale, and both meet ilu0a there."""
    m, con, amat, rhs, x0 = dis_system(*shape)
    v = np.random.default_rng(11).standard_normal(m.nodes)
    zd = _precondition(gblib, shape, amat, con, v, native=False)
    zn = _precondition(gblib, shape, amat, con, v, native=True)
    o = oracle.Ims(oracle.settings(), con["ia"], con["ja"])
    o.apply(amat.copy(), rhs.copy(), x0.copy())
    zo = oracle.ilu0a(o.apc(), o.iapc(), o.japc(), v, fma=True)
    scale = np.max(np.abs(zo))
    assert np.max(np.abs(zd - zn)) <= 1e-12 * scale
    assert np.max(np.abs(zd - zo)) <= 1e-12 * scale
    assert np.max(np.abs(zn - zo)) <= 1e-12 * scale


@pytest.mark.parametrize("factor", [1e-40, 1e40])
def test_out_of_float_range_factor_keeps_native_sweeps(gblib, factor):
    """A system scaled so that its factor leaves the float exponent range
    (inverse pivots near 1e40 or 1e-40) is swept in native FP64 and still
    matches ilu0a; the residual scale that comes with it is tiny or huge."""
    shape = (3, 40, 41)
    m, con, amat, rhs, x0 = dis_system(*shape)
    a = amat * factor
    v = np.random.default_rng(12).standard_normal(m.nodes) * factor
    z = _precondition(gblib, shape, a, con, v, native=False)
    o = oracle.Ims(oracle.settings(), con["ia"], con["ja"])
    o.apply(a.copy(), rhs.copy() * factor, x0.copy())
    zo = oracle.ilu0a(o.apc(), o.iapc(), o.japc(), v, fma=True)
    assert np.max(np.abs(z - zo)) <= 1e-12 * np.max(np.abs(zo))


def test_df64_right_hand_side_extremes(gblib):
    """df64 sweeps on right-hand sides that span many decades (1e-20 to 1e20
    in one vector) stay within 1e-12 of ilu0a, relative to the result's
    scale."""
    shape = (2, 33, 40)
    m, con, amat, rhs, x0 = dis_system(*shape)
    rng = np.random.default_rng(13)
    v = rng.standard_normal(m.nodes) * 10.0 ** rng.uniform(-20, 20, m.nodes)
    z = _precondition(gblib, shape, amat, con, v, native=False)
    o = oracle.Ims(oracle.settings(), con["ia"], con["ja"])
    o.apply(amat.copy(), rhs.copy(), x0.copy())
    zo = oracle.ilu0a(o.apc(), o.iapc(), o.japc(), v, fma=True)
    assert np.max(np.abs(z - zo)) <= 1e-12 * np.max(np.abs(zo))


def reduced_system(nlay, nrow, ncol, frac, seed=3):
    """The DIS system of dis_system with a seeded fraction of its cells
    removed as IDOMAIN does (rows and columns dropped, the kept cells
    renumbered in user order; the CHD cell 0 is kept): (nodeuser, ia, ja,
    amat, rhs, x0)."""
    m, con, amat, rhs, x0 = dis_system(nlay, nrow, ncol)
    ia, ja = con["ia"], con["ja"]
    keep = np.random.default_rng(seed).uniform(size=m.nodes) >= frac
    keep[0] = True
    new = np.cumsum(keep) - 1
    rows, vals = [], []
    for r in np.flatnonzero(keep):
        sel = [q for q in range(ia[r], ia[r + 1]) if keep[ja[q]]]
        rows.append([new[ja[q]] for q in sel])
        vals.append([amat[q] for q in sel])
    ia2 = np.concatenate([[0], np.cumsum([len(c) for c in rows])]).astype(np.int32)
    ja2 = np.concatenate(rows).astype(np.int32)
    a2 = np.concatenate(vals)
    nodeuser = np.flatnonzero(keep).astype(np.int32)
    return nodeuser, ia2, ja2, a2, rhs[keep].copy(), x0[keep].copy()


@pytest.mark.parametrize("precision", [_lib.GBIMS_FP64, _lib.GBIMS_MIXED])
@pytest.mark.parametrize("shape,frac", [((2, 40, 37), 0.1), ((3, 70, 64), 0.3), ((1, 33, 9), 0.5)],
                         ids=["2x40x37", "3x70x64", "1x33x9"])
def test_idomain_grid_sweeps_on_the_full_grid(gblib, shape, frac, precision):
    """An IDOMAIN-reduced DIS grid with its node map runs the wavefront
    sweeps on the full grid (inactive cells decoupled): the preconditioner
    matches the oracle's ilu0a of the reduced matrix (FP64: 1e-12 of its
    scale; FP32: 1e-5), and the same handle solves to the oracle's closure."""
    nodeuser, ia, ja, amat, rhs, x0 = reduced_system(*shape, frac)
    n = ia.size - 1
    ims = ImsLinear(ImsLinearSettings(structure=shape, precision=precision)).imslinear_allocate(
        n, ia, ja)
    ims.set_dis_nodes(nodeuser)
    assert gblib.gbims_factor(ims._h, _lib.dptr(amat), None) == 0
    v = np.random.default_rng(5).standard_normal(n)
    z = np.zeros_like(v)
    assert gblib.gbims_precondition(ims._h, _lib.dptr(v), _lib.dptr(z)) == 0
    o = oracle.Ims(oracle.settings(), ia, ja)
    o.apply(amat.copy(), rhs.copy(), x0.copy())
    zo = oracle.ilu0a(o.apc(), o.iapc(), o.japc(), v, fma=True)
    scale = np.max(np.abs(zo))
    tol = 1e-12 if precision == _lib.GBIMS_FP64 else 1e-5
    assert np.max(np.abs(z - zo)) <= tol * scale, np.max(np.abs(z - zo)) / scale
    tol_s = dict(dvclose=1e-9, rclose=1e-7, iter1=2000)
    ob = oracle.Ims(oracle.settings(**tol_s), ia, ja)
    xo = x0.copy()
    ob.apply(amat.copy(), rhs.copy(), xo)
    ims2 = ImsLinear(ImsLinearSettings(structure=shape, precision=precision, **tol_s)).imslinear_allocate(
        n, ia, ja)
    ims2.set_dis_nodes(nodeuser)
    x2 = x0.copy()
    r2 = ims2.imslinear_apply(amat.copy(), rhs.copy(), x2)
    assert r2.summary["structured"] == 1 and r2.icnvg == 1
    bar = 1e-6 if precision == _lib.GBIMS_FP64 else 1e-4
    assert np.max(np.abs(x2 - xo)) <= bar * max(1.0, np.max(np.abs(xo))), np.max(np.abs(x2 - xo))


def test_idomain_node_map_is_checked(gblib):
    """A node map that does not describe the pattern, or that comes after the
    first factorisation, is refused; the handle keeps its level sweeps."""
    nodeuser, ia, ja, amat, rhs, x0 = reduced_system(2, 20, 11, 0.2)
    n = ia.size - 1
    ims = ImsLinear(ImsLinearSettings(structure=(2, 20, 11))).imslinear_allocate(n, ia, ja)
    bad = nodeuser.copy()
    bad[3] += 1 if bad[4] > bad[3] + 1 else 0
    bad[-1] = 2 * 20 * 11 + 5  # outside the grid
    with pytest.raises(_lib.GbimsError):
        ims.set_dis_nodes(bad)
    assert gblib.gbims_factor(ims._h, _lib.dptr(amat), None) == 0
    with pytest.raises(_lib.GbimsError):
        ims.set_dis_nodes(nodeuser)
    res = ims.imslinear_apply(amat.copy(), rhs.copy(), x0.copy())
    assert res.summary["structured"] == 0
