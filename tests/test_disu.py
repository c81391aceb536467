"""DISU (unstructured) grids: the library's connectivity
(modflow6_gb300.disu) equals the oracle's restatement of disuconnections /
con_finalize / fillisym / filljas (Connections.f90:160-316, 801-928,
1205-1268) array for array, on full, reduced (IDOMAIN) and vertically
staggered grids; a DIS grid written as DISU gives the DIS connectivity; the
input checks of disu_ck and con_finalize reject what the reference rejects;
the staggered conductance (GwfConductanceUtils.f90:375-393) is checked by
hand; and on the GPU the fill is bit-exact and the device-resident time step
matches the oracle's on DISU and DISV grids."""
import ctypes as C

import numpy as np
import pytest

import oracle
from modflow6_gb300.dis import dis_connections
from modflow6_gb300.disu import (DisuError, DisuModel, dis_as_disu, disu_check, disu_connections,
                                 make_disu_model, refined_grid)

KEYS = ("ia", "ja", "isym", "jas", "ihc", "cl1", "cl2", "hwva")


@pytest.mark.parametrize("stagger", [0.0, 3.0])
@pytest.mark.parametrize("holes", [0, 0.2])
def test_connectivity_matches_oracle(stagger, holes):
    g = refined_grid(3, 8, 10, 50.0, (2, 5, 3, 6), stagger=stagger, seed=1)
    idom = None
    if holes:
        idom = (np.random.default_rng(0).random(g["iac"].size) > holes).astype(int)
    c = disu_connections(g["iac"], g["ja"], g["ihc"], g["cl12"], g["hwva"], idom)
    o = oracle.disu_connect(g["iac"], g["ja"], g["ihc"], g["cl12"], g["hwva"], idom)
    assert c["nodes"] == o["nodes"] and c["nja"] == o["nja"] and c["njas"] == o["njas"]
    for k in KEYS:
        np.testing.assert_array_equal(c[k], o[k], err_msg=k)
    if stagger:
        assert (c["ihc"] == 2).sum() > 0
    # a refined cell beside a coarse one: the coarse cell has two neighbours
    # across that face, so some rows have more than four horizontal entries
    assert (np.diff(c["ia"]) - 1).max() >= 6


def test_dis_written_as_disu_equals_dis():
    nl, nr, nc = 3, 4, 5
    delr, delc = np.linspace(10, 20, nc), np.linspace(5, 9, nr)
    top = np.full(nr * nc, 30.0)
    botm = np.concatenate([np.full(nr * nc, 20.0), np.full(nr * nc, 9.0), np.zeros(nr * nc)])
    u = dis_as_disu(nl, nr, nc, delr, delc, top, botm)
    c = disu_connections(u["iac"], u["ja"], u["ihc"], u["cl12"], u["hwva"])
    d = dis_connections(nl, nr, nc, delr, delc, u["top"], u["bot"])
    for k in KEYS:
        np.testing.assert_array_equal(c[k], d[k], err_msg=k)


def test_reduced_dis_as_disu_is_the_dis_submatrix():
    """IDOMAIN 0 cells removed: the rows and columns of the kept cells of the
    full DIS connectivity, renumbered, with the kept connections' IHC, CL1,
    CL2 and HWVA."""
    nl, nr, nc = 2, 5, 6
    delr, delc = np.full(nc, 10.0), np.full(nr, 8.0)
    top = np.full(nr * nc, 20.0)
    botm = np.concatenate([np.full(nr * nc, 10.0), np.zeros(nr * nc)])
    u = dis_as_disu(nl, nr, nc, delr, delc, top, botm)
    n = u["iac"].size
    idom = np.ones(n, int)
    idom[[3, 7, 8, 14, 33, 40]] = 0
    c = disu_connections(u["iac"], u["ja"], u["ihc"], u["cl12"], u["hwva"], idom)
    d = dis_connections(nl, nr, nc, delr, delc, u["top"], u["bot"])
    red = np.full(n, -1)
    red[idom > 0] = np.arange((idom > 0).sum())
    rown = np.repeat(np.arange(n), np.diff(d["ia"]))
    keep = (idom[rown] > 0) & (idom[d["ja"]] > 0)
    np.testing.assert_array_equal(c["ja"], red[d["ja"][keep]])
    np.testing.assert_array_equal(c["nodeuser"], np.flatnonzero(idom > 0))
    up = keep & (d["ja"] > rown)
    for k in ("ihc", "cl1", "cl2", "hwva"):
        np.testing.assert_array_equal(c[k], d[k][d["jas"][up]], err_msg=k)


def _tiny():
    """Three cells in a row, 1-based JA with each diagonal written negative
    (as DISU files often do)."""
    return dict(iac=[2, 3, 2], ja=[-1, 2, -2, 1, 3, -3, 2], ihc=[1, 1, 1, 1, 1, 1, 1],
                cl12=[0, 5.0, 0, 5.0, 5.0, 0, 5.0], hwva=[0, 10.0, 0, 10.0, 10.0, 0, 10.0],
                top=[10.0] * 3, bot=[0.0] * 3, area=[100.0] * 3)


def _both(t, **over):
    """The library's checks and the oracle's, on input t with changes."""
    t = {**t, **over}
    err = None
    try:
        ja = disu_check(t["top"], t["bot"], t["area"], t["iac"], t["ja"], t["ihc"])
        disu_connections(t["iac"], ja, t["ihc"], t["cl12"], t["hwva"])
    except DisuError as e:
        err = e
    oerr = None
    try:
        oracle.disu_connect(t["iac"], t["ja"], t["ihc"], t["cl12"], t["hwva"])
    except ValueError as e:
        oerr = e
    return err, oerr


def test_checks_accept_and_reject_like_the_reference():
    t = _tiny()
    err, oerr = _both(t)
    assert err is None and oerr is None
    c = disu_connections(t["iac"], t["ja"], t["ihc"], t["cl12"], t["hwva"])
    np.testing.assert_array_equal(c["ja"], [0, 1, 1, 0, 2, 2, 1])
    np.testing.assert_array_equal(c["cl1"], [5.0, 5.0])
    # the diagonal not first
    err, oerr = _both(t, ja=[2, 1, -2, 1, 3, -3, 2])
    assert err and "first connection" in str(err) and oerr and "diagonal" in str(oerr)
    # a row not ascending
    err, oerr = _both(t, iac=[3, 2, 2], ja=[1, 3, 2, 2, 1, 3, 1], ihc=[1] * 7,
                      cl12=[0, 5, 5, 0, 5, 0, 5.0], hwva=[0, 10, 10, 0, 10, 0, 10.0])
    assert err and "not sorted" in str(err) and oerr and "ascending" in str(oerr)
    # a connection without its counterpart (1-2 given only in row 1)
    err, oerr = _both(t, iac=[2, 2, 2], ja=[1, 2, 2, 3, 3, 2], ihc=[1] * 6,
                      cl12=[0, 5, 0, 5, 0, 5.0], hwva=[0, 10, 0, 10, 0, 10.0])
    assert err and "symmetric counterpart" in str(err) and oerr and "counterpart" in str(oerr)
    # HWVA not symmetric
    err, oerr = _both(t, hwva=[0, 10.0, 0, 11.0, 10.0, 0, 10.0])
    assert err and "HWVA" in str(err) and oerr and "HWVA" in str(oerr)
    # IHC not symmetric, and IHC out of range
    err, oerr = _both(t, ihc=[1, 1, 1, 2, 1, 1, 1])
    assert err and "IHC" in str(err) and oerr and "IHC" in str(oerr)
    err, oerr = _both(t, ihc=[1, 3, 1, 3, 1, 1, 1])
    assert err and "IHC must be" in str(err) and oerr and "0..2" in str(oerr)
    # disu_ck: thickness, area, a cell below whose top is above the bottom of
    # the cell above, IDOMAIN values
    with pytest.raises(DisuError, match="THICKNESS"):
        disu_check([10, 0, 10], [0, 0, 0], [1, 1, 1], t["iac"], t["ja"], t["ihc"])
    with pytest.raises(DisuError, match="area"):
        disu_check([10] * 3, [0] * 3, [1, 0, 1], t["iac"], t["ja"], t["ihc"])
    with pytest.raises(DisuError, match="Top elevation"):
        disu_check([10, 12, 10], [5, 0, 0], [1] * 3, t["iac"], t["ja"], [1, 0, 0, 0, 1, 1, 1])
    disu_check([10, 5.5, 10], [5, 0, 0], [1] * 3, t["iac"], t["ja"], [1, 0, 0, 0, 1, 1, 1],
               voffsettol=0.5)
    with pytest.raises(DisuError, match="idomain"):
        disu_check(t["top"], t["bot"], t["area"], t["iac"], t["ja"], t["ihc"], idomain=[1, 2, 1])


def test_staggered_conductance_by_hand():
    """Two convertible cells side by side, vertically offset (IHC 2): the
    conductance the oracle assembles is the harmonic mean over the wetted
    parts of the cells that lie within their vertical overlap
    (staggered_thkfrac), not over the cells' own wetted thicknesses."""
    top, bot = np.array([10.0, 8.0]), np.array([0.0, -3.0])
    k = np.array([2.0, 5.0])
    m = DisuModel(top, bot, np.array([100.0, 100.0]), [2, 2], [1, 2, 2, 1], [1, 2, 1, 2],
                  [0, 5.0, 0, 4.0], [0, 10.0, 0, 10.0], k, k, np.array([1, 1], np.int32),
                  np.array([6.0, 6.0]))
    assert m.connections()["ihc"].tolist() == [2]
    g = oracle.Gwf(m, oracle.settings())
    h = np.array([6.0, 5.0])
    amat, _ = g.assemble(h)
    sat = (h - bot) / (top - bot)
    sill_top, sill_bot = min(top), max(bot)
    t = [max(min(bot[i] + sat[i] * (top[i] - bot[i]), sill_top) - sill_bot, 0.0) for i in (0, 1)]

    def hmean(t):  # condmean, harmonic mean of the transmissivities
        t1, t2 = k[0] * t[0], k[1] * t[1]
        return 10.0 * t1 * t2 / (t1 * 4.0 + t2 * 5.0)

    assert amat[1] == pytest.approx(hmean(t), rel=1e-14)
    # IHC 1 on the same cells uses the cells' own wetted thicknesses
    m1 = DisuModel(top, bot, np.array([100.0, 100.0]), [2, 2], [1, 2, 2, 1], [1, 1, 1, 1],
                   [0, 5.0, 0, 4.0], [0, 10.0, 0, 10.0], k, k, np.array([1, 1], np.int32),
                   np.array([6.0, 6.0]))
    a1, _ = oracle.Gwf(m1, oracle.settings()).assemble(h)
    assert a1[1] == pytest.approx(hmean(sat * (top - bot)), rel=1e-14)
    assert a1[1] != pytest.approx(amat[1], rel=1e-3)


def test_oracle_solves_a_disu_model():
    m = make_disu_model(2, 12, 16, seed=4, stagger=2.0, idomain_holes=6)
    g = oracle.Gwf(m, oracle.settings(dvclose=1e-8, rclose=1e-6, iter1=2000, ilinmeth=1))
    st = g.timestep(kper=1, kstp=1, delt=1.0, transient=False, dvclose=1e-8, mxiter=20)
    assert st["converged"] == 1
    amat, rhs = g.assemble(g.x)
    r = rhs - oracle.amux(g.con["ia"], g.con["ja"], amat, g.x)
    assert np.max(np.abs(r[m.ibound > 0])) < 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("newton,stagger", [(False, 0.0), (False, 2.5), (True, 2.5)])
def test_gpu_fill_on_disu_bitexact(gblib, newton, stagger):
    """The device fill (NPF fc/fn, STO fc/fn, WEL, RCH) of a DISU model on
    the general connectivity entry point, bit for bit against the oracle's,
    with heads across the cell bottoms so that the staggered thicknesses
    and the Newton overlap terms are exercised."""
    from modflow6_gb300.ims import ImsLinearSettings
    from modflow6_gb300.solution import GwfSolution, Nonlinear
    m = make_disu_model(3, 10, 14, seed=5, stagger=stagger, transient=True, newton=newton,
                        idomain_holes=4)
    g = oracle.Gwf(m, oracle.settings())
    sol = GwfSolution(m, ImsLinearSettings(), Nonlinear())
    rng = np.random.default_rng(6)
    h = m.strt + rng.uniform(-22.0, 3.0, m.nodes)
    hold = m.strt + rng.uniform(-3.0, 3.0, m.nodes)
    sol.heads = h
    amat, rhs = sol.formulate(delt=2.5, hold=hold)
    ao, ro = g.assemble(h, hold=hold, delt=2.5, transient=True)
    np.testing.assert_array_equal(amat, ao)
    np.testing.assert_array_equal(rhs, ro)


@pytest.mark.gpu
@pytest.mark.parametrize("grid", ["disu", "disu_staggered_newton", "disv"])
def test_gpu_timestep_on_general_grid_matches_oracle(gblib, grid):
    """One steady time step to closure on the device (gbsln_create_grid:
    SELL-32 product, level-scheduled ILU0) against the oracle's outer loop:
    the same number of outer iterations (within one) and heads within 0.1 x
    OUTER_DVCLOSE (2e-6 m for the Newton case, whose under-relaxation walks
    the ibotnode chain)."""
    from modflow6_gb300.disv import make_disv_model
    from modflow6_gb300.ims import ImsLinearSettings
    from modflow6_gb300.solution import GwfSolution, Nonlinear
    if grid == "disv":
        m = make_disv_model(3, 20, 14, seed=8)
    elif grid == "disu":
        m = make_disu_model(2, 12, 16, seed=8, idomain_holes=5)
    else:
        # wells at 0.3x, so that Newton converges with two cells below their
        # bottoms but above the model bottom (the ibotnode cell's)
        m = make_disu_model(3, 12, 16, seed=8, stagger=2.0, newton=True)
        m.inewtonur = 1
        m.wel_q = 0.3 * m.wel_q
    tol = dict(dvclose=1e-9, rclose=1e-7, iter1=2000, ilinmeth=2 if m.inewton else 1)
    g = oracle.Gwf(m, oracle.settings(**tol))
    so = g.timestep(kper=1, kstp=1, delt=1.0, dvclose=1e-7, mxiter=50)
    sol = GwfSolution(m, ImsLinearSettings(**tol), Nonlinear(dvclose=1e-7, mxiter=50))
    sg = sol.timestep(1, 1, 1.0)
    assert so["converged"] == 1 and sg["converged"] == 1
    assert abs(sg["outer"] - so["outer"]) <= 1, (sg["outer"], so["outer"])
    lim = 2e-6 if m.inewton else 1e-8
    assert np.max(np.abs(sol.heads - g.x)) <= lim


@pytest.mark.gpu
def test_gpu_create_grid_rejects_bad_connectivity(gblib):
    """gbsln_create_grid makes con_finalize's checks before any device
    work: a row without its diagonal first, an unsorted row, and a
    connection without its counterpart each return GBIMS_ERR_ARG with the
    reason."""
    from modflow6_gb300 import _lib
    from modflow6_gb300.ims import ImsLinearSettings
    from modflow6_gb300.solution import Nonlinear
    lib = _lib.load()
    f = lambda a: np.ascontiguousarray(a, np.float64)
    i = lambda a: np.ascontiguousarray(a, np.int32)
    cases = [([0, 2, 5, 7], [1, 0, 1, 0, 2, 2, 1], "diagonal"),
             ([0, 2, 5, 7], [0, 1, 1, 2, 0, 2, 1], "sorted"),
             ([0, 2, 4, 6], [0, 1, 1, 2, 2, 1], "counterpart")]
    for ia, ja, why in cases:
        keep = dict(ia=i(ia), ja=i(ja), ihc=i([1, 1]), c=f([5.0, 5.0]), top=f([10.0] * 3),
                    bot=f([0.0] * 3), area=f([100.0] * 3), k=f([1.0] * 3), ict=i([0] * 3),
                    z=i([0]), zd=f([0.0]), strt=f([5.0] * 3), d0=f([0.0]))
        grid = _lib.GbslnGrid(3, len(ja), _lib.iptr(keep["ia"]), _lib.iptr(keep["ja"]),
                              _lib.iptr(keep["ihc"]), _lib.dptr(keep["c"]), _lib.dptr(keep["c"]),
                              _lib.dptr(keep["c"]), _lib.dptr(keep["top"]), _lib.dptr(keep["bot"]),
                              _lib.dptr(keep["area"]))
        d0 = _lib.dptr(keep["d0"])
        cm = _lib.GbslnModel(0, 0, 0, d0, d0, d0, d0, _lib.dptr(keep["k"]), _lib.dptr(keep["k"]),
                             _lib.iptr(keep["ict"]), None, None, 0, _lib.iptr(keep["z"]),
                             _lib.dptr(keep["zd"]), 0, _lib.iptr(keep["z"]), _lib.dptr(keep["zd"]),
                             0, _lib.iptr(keep["z"]), _lib.dptr(keep["zd"]))
        npf = _lib.GbnpfOptions(0, 0, 0, 0, 1.0e-6, 0, 0)
        cs = ImsLinearSettings().to_c(0)
        nl = Nonlinear()
        cnl = _lib.GbslnNonlinear(nl.dvclose, nl.mxiter, nl.nonmeth, nl.theta, nl.akappa, nl.gamma,
                                  nl.amomentum, nl.iallowptc, nl.numtrack, nl.btol, nl.breduc,
                                  nl.res_lim)
        h = C.c_void_p()
        rc = lib.gbsln_create_grid(C.byref(grid), C.byref(cm), C.byref(npf), C.byref(cs),
                                   C.byref(cnl), _lib.dptr(keep["strt"]), C.byref(h))
        msg = lib.gbsln_last_error(h).decode()
        lib.gbsln_destroy(h)
        assert rc == _lib.GBIMS_ERR_ARG and why in msg, (rc, msg)
