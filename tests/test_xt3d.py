"""XT3D (Xt3dInterface.f90, Xt3dAlgorithm.f90): the full conductivity
tensor on the neighbours-of-neighbours stencil, on DIS grids.

The oracle's restatement is pinned by the property XT3D exists for (and
which the reference's own XT3D tests check against analytical answers):
uniform flow through a rotated anisotropic medium, here with specified heads
on two faces and no flow through the others, is reproduced exactly, where
the standard two-point conductances miss it by decimetres.  The library's
pattern equals the oracle's; on the GPU the fill is bit-exact against the
oracle (permanently confined cells with their precomputed terms, convertible
cells, Newton, transient) and the device-resident time step reproduces the
analytical field."""
import math

import numpy as np
import pytest

import oracle
from modflow6_gb300.dis import GwfDisModel
from modflow6_gb300.xt3d import xt3d_pattern


def ktensor(k11, k22, k33, a1, a2, a3):
    d = math.pi / 180.0
    s1, c1, s2, c2, s3, c3 = (math.sin(a1 * d), math.cos(a1 * d), math.sin(a2 * d),
                              math.cos(a2 * d), math.sin(a3 * d), math.cos(a3 * d))
    r = np.array([[c1 * c2, c1 * s2 * s3 - s1 * c3, -c1 * s2 * c3 - s1 * s3],
                  [s1 * c2, s1 * s2 * s3 + c1 * c3, -s1 * s2 * c3 + c1 * s3],
                  [s2, -c2 * s3, c2 * c3]])
    return r @ np.diag([k11, k22, k33]) @ r.T


def aniso_model(nlay, nrow, ncol, angles, three_d, seed=0, xt3d=True, icelltype=0):
    """Uniform flow h = 100 + a x + b y + c z through K = R diag(5, 1, 0.5)
    R^T on a seeded non-uniform DIS grid: CHD on the first and last columns,
    no flow elsewhere, so b and c make (K grad h) normal to the other faces
    zero.  Returns the model and the analytical heads."""
    rng = np.random.default_rng(seed)
    delr, delc = rng.uniform(8, 12, ncol), rng.uniform(8, 12, nrow)
    nrc = nrow * ncol
    top = np.full(nrc, 10.0 * nlay)
    botm = np.concatenate([np.full(nrc, 10.0 * (nlay - 1 - k)) for k in range(nlay)])
    n = nlay * nrc
    x = np.concatenate([[0], np.cumsum(delr)])
    y = np.concatenate([[0], np.cumsum(delc)])
    xc, yc = 0.5 * (x[1:] + x[:-1]), -0.5 * (y[1:] + y[:-1])
    X = np.tile(np.add.outer(np.zeros(nrow), xc).ravel(), nlay)
    Y = np.tile(np.add.outer(yc, np.zeros(ncol)).ravel(), nlay)
    ct = np.concatenate([top, botm[:-nrc]])
    Z = botm + 0.5 * (ct - botm)
    K = ktensor(5.0, 1.0, 0.5, *angles)
    a = 0.03
    if three_d:
        b, c = np.linalg.solve(K[1:, 1:], -a * K[1:, 0])
    else:
        b, c = -a * K[1, 0] / K[1, 1], 0.0
    h = 100.0 + a * X + b * Y + c * Z
    m = GwfDisModel(nlay, nrow, ncol, delr, delc, top, botm, np.full(n, 5.0), np.full(n, 0.5),
                    np.full(n, icelltype, np.int32), h.copy())
    m.ixt3d = 1 if xt3d else 0
    m.k22 = np.full(n, 1.0)
    m.angle1 = np.full(n, angles[0])
    if three_d:
        m.angle2, m.angle3 = np.full(n, angles[1]), np.full(n, angles[2])
    j = np.arange(n) % ncol
    bnd = (j == 0) | (j == ncol - 1)
    m.chd_node = np.flatnonzero(bnd).astype(np.int32)
    m.chd_head = h[bnd]
    m.strt = np.where(bnd, h, 100.0)
    return m, h


CASES = [(1, 9, 11, (30.0, 0.0, 0.0), False), (4, 7, 9, (30.0, 20.0, 10.0), True)]


@pytest.mark.parametrize("case", CASES, ids=["2d", "3d"])
def test_oracle_reproduces_uniform_anisotropic_flow(case):
    tol = dict(dvclose=1e-12, rclose=1e-10, iter1=4000, ilinmeth=2)
    m, h = aniso_model(*case)
    g = oracle.Gwf(m, oracle.settings(**tol))
    st = g.timestep(kper=1, kstp=1, delt=1.0, dvclose=1e-11, mxiter=20)
    assert st["converged"] == 1
    assert np.abs(g.x - h).max() < 1e-9
    ms, _ = aniso_model(*case, xt3d=False)
    gs = oracle.Gwf(ms, oracle.settings(**tol))
    gs.timestep(kper=1, kstp=1, delt=1.0, dvclose=1e-11, mxiter=20)
    assert np.abs(gs.x - h).max() > 0.1


def test_pattern_matches_oracle():
    m, _ = aniso_model(3, 6, 7, (30.0, 20.0, 10.0), True)
    g = oracle.Gwf(m, oracle.settings())
    con = g.mcon
    sia, sja, idxglo = xt3d_pattern(con["ia"], con["ja"])
    np.testing.assert_array_equal(sia, g.con["ia"])
    np.testing.assert_array_equal(sja, g.con["ja"])
    np.testing.assert_array_equal(idxglo, g.con["idxglo"])
    # a cell of the middle layer of three: itself, 6 neighbours and the 16
    # cells two steps away (18 less the two two layers up and down)
    assert np.diff(sia).max() == 23


@pytest.mark.parametrize("case", CASES, ids=["2d", "3d"])
def test_oracle_rows_conserve(case):
    """Every XT3D term moves flow between two cells: without storage or
    boundaries each row of the conductance matrix sums to zero."""
    m, h = aniso_model(*case, icelltype=1)
    m.chd_node = np.zeros(0, np.int32)
    m.chd_head = np.zeros(0)
    g = oracle.Gwf(m, oracle.settings())
    hh = h - 3.0 * np.random.default_rng(1).random(h.size)
    amat, _ = g.assemble(hh)
    ia = g.con["ia"]
    rs = np.add.reduceat(amat, ia[:-1])
    assert np.abs(rs).max() <= 1e-12 * np.abs(amat).max()


def test_oracle_confined_terms_precomputed_equal_direct():
    """Confined cells take the terms made once with saturated areas (amatpc,
    amatpcx); convertible cells with heads above their tops take the same
    terms in the per-call loop: the matrices agree to rounding."""
    case = CASES[1]
    mc, h = aniso_model(*case, icelltype=0)
    mv, _ = aniso_model(*case, icelltype=1)
    a1, _ = oracle.Gwf(mc, oracle.settings()).assemble(h + 100.0)
    a2, _ = oracle.Gwf(mv, oracle.settings()).assemble(h + 100.0)
    np.testing.assert_allclose(a1, a2, rtol=1e-12, atol=1e-12 * np.abs(a1).max())


def test_oracle_isotropic_equals_standard():
    """Isotropic K on a DIS grid: XT3D's terms on the 7-point positions are
    the standard conductances, and the extended positions are zero."""
    m, h = aniso_model(3, 6, 7, (0.0, 0.0, 0.0), False)
    m.k22 = m.k11.copy()
    m.k33 = m.k11.copy()
    g = oracle.Gwf(m, oracle.settings())
    ax, _ = g.assemble(h)
    m.ixt3d = 0
    gs = oracle.Gwf(m, oracle.settings())
    a0, _ = gs.assemble(h)
    idx = g.con["idxglo"]
    np.testing.assert_allclose(ax[idx], a0, rtol=1e-13, atol=1e-13 * np.abs(a0).max())
    ext = np.ones(ax.size, bool)
    ext[idx] = False
    assert np.abs(ax[ext]).max() <= 1e-13 * np.abs(a0).max()


def _gpu_pair(m):
    from modflow6_gb300.ims import ImsLinearSettings
    from modflow6_gb300.solution import GwfSolution, Nonlinear
    g = oracle.Gwf(m, oracle.settings())
    sol = GwfSolution(m, ImsLinearSettings(), Nonlinear())
    return g, sol


@pytest.mark.gpu
@pytest.mark.parametrize("icelltype,newton,transient", [(0, 0, 0), (1, 0, 1), (1, 1, 1), (0, 1, 0)],
                         ids=["confined", "convertible", "newton", "confined-newton"])
@pytest.mark.parametrize("case", CASES, ids=["2d", "3d"])
def test_gpu_xt3d_fill_bitexact(gblib, case, icelltype, newton, transient):
    """The device fill with XT3D against the oracle's, bit for bit: the
    permanently confined terms (made once on the device), the per-call
    terms at heads across the cell bottoms, the Newton terms and storage."""
    m, h = aniso_model(*case, icelltype=icelltype)
    m.inewton = newton
    if transient:
        m.ss, m.sy = np.full(m.nodes, 1e-5), np.full(m.nodes, 0.15)
    g, sol = _gpu_pair(m)
    rng = np.random.default_rng(3)
    hh = h + rng.uniform(-14.0, 2.0, m.nodes)
    hold = h + rng.uniform(-1.0, 1.0, m.nodes)
    sol.heads = hh
    delt = 2.5 if transient else 0.0
    amat, rhs = sol.formulate(delt=delt, hold=hold if transient else None)
    ao, ro = g.assemble(hh, hold=hold, delt=delt, transient=bool(transient))
    assert amat.size == ao.size == g.con["nja"]
    np.testing.assert_array_equal(amat, ao)
    np.testing.assert_array_equal(rhs, ro)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=["2d", "3d"])
def test_gpu_xt3d_timestep_reproduces_uniform_flow(gblib, case):
    """The device-resident time step with XT3D reaches the analytical heads
    of uniform flow through the rotated anisotropic medium, and the
    oracle's heads."""
    from modflow6_gb300.ims import ImsLinearSettings
    from modflow6_gb300.solution import GwfSolution, Nonlinear
    tol = dict(dvclose=1e-12, rclose=1e-10, iter1=4000, ilinmeth=2)
    m, h = aniso_model(*case)
    g = oracle.Gwf(m, oracle.settings(**tol))
    so = g.timestep(kper=1, kstp=1, delt=1.0, dvclose=1e-11, mxiter=20)
    sol = GwfSolution(m, ImsLinearSettings(**tol), Nonlinear(dvclose=1e-11, mxiter=20))
    sg = sol.timestep(1, 1, 1.0)
    assert sg["converged"] == 1 and so["converged"] == 1
    assert np.abs(sol.heads - h).max() < 1e-9
    assert np.abs(sol.heads - g.x).max() < 1e-9


@pytest.mark.gpu
def test_gpu_xt3d_newton_timestep_matches_oracle(gblib):
    """A convertible Newton model with XT3D, pumping from the top layer:
    the device time step against the oracle's, heads within 1e-6 m."""
    from modflow6_gb300.ims import ImsLinearSettings
    from modflow6_gb300.solution import GwfSolution, Nonlinear
    m, h = aniso_model(3, 8, 10, (25.0, 15.0, 5.0), True, icelltype=1)
    m.inewton = 1
    m.wel_node = np.array([m.nrow * m.ncol // 2 + 3], np.int32)
    m.wel_q = np.array([-2.0])
    tol = dict(dvclose=1e-10, rclose=1e-8, iter1=4000, ilinmeth=2)
    g = oracle.Gwf(m, oracle.settings(**tol))
    so = g.timestep(kper=1, kstp=1, delt=1.0, dvclose=1e-9, mxiter=50)
    sol = GwfSolution(m, ImsLinearSettings(**tol), Nonlinear(dvclose=1e-9, mxiter=50))
    sg = sol.timestep(1, 1, 1.0)
    assert so["converged"] == 1 and sg["converged"] == 1
    assert abs(sg["outer"] - so["outer"]) <= 1
    assert np.abs(sol.heads - g.x).max() < 1e-6


# ---- DISV and DISU grids ---------------------------------------------------

def _general_linear(m, xt3d=True, icelltype=0, angle=30.0):
    """XT3D on a DISV or DISU model: K = R diag(5, 1, 0.5) R^T rotated by
    ANGLE1 in the plane, CHD on the cells of the grid's outer ring with
    h = 100 + 0.03 x - 0.02 y, which is then the exact solution (no flux
    through the top and bottom: the tensor has no vertical coupling)."""
    n = m.nodes
    con = m.connections()
    m.k11, m.k33 = np.full(n, 5.0), np.full(n, 0.5)
    m.k22 = np.full(n, 1.0)
    m.angle1 = np.full(n, angle)
    m.angle2 = m.angle3 = None
    m.icelltype = np.full(n, icelltype, np.int32)
    m.ixt3d = 1 if xt3d else 0
    if getattr(m, "disu", False):
        x, y = m.xc, m.yc
        full = 4
    else:
        x, y = m.xcn, m.ycn
        full = 6
    h = 100.0 + 0.03 * x - 0.02 * y
    rown = np.repeat(np.arange(n), np.diff(con["ia"]))
    off = con["ja"] != rown
    hz = off & (con["ihc"][np.maximum(con["jas"], 0)] != 0)
    hdeg = np.bincount(rown[hz], minlength=n)
    bnd = hdeg < full
    m.chd_node = np.flatnonzero(bnd).astype(np.int32)
    m.chd_head = h[bnd]
    m.wel_node = np.zeros(0, np.int32)
    m.wel_q = np.zeros(0)
    m.rch_node = np.zeros(0, np.int32)
    m.rch_rate = np.zeros(0)
    m.strt = np.where(bnd, h, 100.0)
    return m, h


def _disv():
    from modflow6_gb300.disv import make_disv_model
    return make_disv_model(3, 14, 10, seed=3)


def _disu():
    from modflow6_gb300.disu import make_disu_model
    return make_disu_model(2, 12, 15, seed=3)


GENERAL = [("disv", _disv), ("disu", _disu)]


def test_anglex_matches_oracle():
    from modflow6_gb300.disu import refined_grid
    m = _disv()
    con = m.connections()
    iav, jav = m.vertex_lists
    ax = np.zeros(con["njas"])
    lib = oracle.load()
    keep = [np.ascontiguousarray(a, np.float64) for a in (m.vertices[:, 0], m.vertices[:, 1])]
    ints = [np.ascontiguousarray(a, np.int32) for a in (iav, jav, m.nodeuser, con["ia"], con["ja"],
                                                        con["jas"], con["ihc"])]
    lib.or_disv_anglex(m.nodes, len(m.icvert), oracle.dp(keep[0]), oracle.dp(keep[1]),
                       *[oracle.ip(a) for a in ints], oracle.dp(ax))
    np.testing.assert_array_equal(con["anglex"], ax)
    assert (ax[con["ihc"] != 0] > 0).any()
    g = refined_grid(2, 8, 10, 50.0, (2, 5, 3, 6), seed=1)
    from modflow6_gb300.disu import disu_connections
    c = disu_connections(g["iac"], g["ja"], g["ihc"], g["cl12"], g["hwva"], angldegx=g["angldegx"])
    o = oracle.disu_connect(g["iac"], g["ja"], g["ihc"], g["cl12"], g["hwva"], angldegx=g["angldegx"])
    np.testing.assert_array_equal(c["anglex"], o["anglex"])
    # each connection n < m points from n to m: east 0, south 3 pi / 2
    assert set(np.round(np.degrees(c["anglex"][c["ihc"] != 0]))) <= {0.0, 270.0}


@pytest.mark.parametrize("name,make", GENERAL, ids=[g[0] for g in GENERAL])
def test_oracle_general_grid_reproduces_uniform_anisotropic_flow(name, make):
    tol = dict(dvclose=1e-12, rclose=1e-10, iter1=4000, ilinmeth=2)
    m, h = _general_linear(make())
    g = oracle.Gwf(m, oracle.settings(**tol))
    st = g.timestep(kper=1, kstp=1, delt=1.0, dvclose=1e-11, mxiter=20)
    assert st["converged"] == 1
    assert np.abs(g.x - h).max() < 1e-9
    ms, _ = _general_linear(make(), xt3d=False)
    gs = oracle.Gwf(ms, oracle.settings(**tol))
    gs.timestep(kper=1, kstp=1, delt=1.0, dvclose=1e-11, mxiter=20)
    assert np.abs(gs.x - h).max() > 0.05


@pytest.mark.gpu
@pytest.mark.parametrize("icelltype,newton,transient", [(0, 0, 0), (1, 0, 1), (1, 1, 1)],
                         ids=["confined", "convertible", "newton"])
@pytest.mark.parametrize("name,make", GENERAL, ids=[g[0] for g in GENERAL])
def test_gpu_general_grid_xt3d_fill_bitexact(gblib, name, make, icelltype, newton, transient):
    """The device fill with XT3D on DISV and DISU grids (cell-centre vectors,
    face normals from the edges or ANGLDEGX, DISU's centre-to-centre vertical
    vectors) against the oracle's, bit for bit."""
    m, h = _general_linear(make(), icelltype=icelltype, angle=35.0)
    m.inewton = newton
    if transient:
        m.ss, m.sy = np.full(m.nodes, 1e-5), np.full(m.nodes, 0.15)
    g, sol = _gpu_pair(m)
    rng = np.random.default_rng(4)
    cb = m.cell_bot
    hh = np.maximum(h, cb + 1.0) + rng.uniform(-12.0, 2.0, m.nodes)
    hold = h + rng.uniform(-1.0, 1.0, m.nodes)
    sol.heads = hh
    delt = 2.5 if transient else 0.0
    amat, rhs = sol.formulate(delt=delt, hold=hold if transient else None)
    ao, ro = g.assemble(hh, hold=hold, delt=delt, transient=bool(transient))
    assert amat.size == ao.size == g.con["nja"]
    np.testing.assert_array_equal(amat, ao)
    np.testing.assert_array_equal(rhs, ro)


@pytest.mark.gpu
@pytest.mark.parametrize("name,make", GENERAL, ids=[g[0] for g in GENERAL])
def test_gpu_general_grid_xt3d_timestep(gblib, name, make):
    from modflow6_gb300.ims import ImsLinearSettings
    from modflow6_gb300.solution import GwfSolution, Nonlinear
    tol = dict(dvclose=1e-12, rclose=1e-10, iter1=4000, ilinmeth=2)
    m, h = _general_linear(make())
    sol = GwfSolution(m, ImsLinearSettings(**tol), Nonlinear(dvclose=1e-11, mxiter=20))
    sg = sol.timestep(1, 1, 1.0)
    assert sg["converged"] == 1
    assert np.abs(sol.heads - h).max() < 1e-9


# ---- XT3D RHS and the flows -------------------------------------------------

def test_oracle_xt3d_flows_are_darcy_fluxes():
    """xt3d_flowja at the analytical heads of the 2-D case: the flow through
    every face between two cells of the same row is the Darcy flux of the
    uniform flow, (K grad h)_x times the face area, and through the faces
    between rows (where K grad h has no y component) it is zero."""
    m, h = aniso_model(*CASES[0])
    g = oracle.Gwf(m, oracle.settings())
    fj, _ = g.budget(h)
    K = ktensor(5.0, 1.0, 0.5, *CASES[0][3])
    b = -0.03 * K[1, 0] / K[1, 1]
    qx = K[0, 0] * 0.03 + K[0, 1] * b
    con = g.mcon
    rown = np.repeat(np.arange(m.nodes), np.diff(con["ia"]))
    ncol = m.ncol
    east = con["ja"] == rown + 1
    south = con["ja"] == rown + ncol
    area = m.delc[(rown % (m.nrow * ncol)) // ncol] * 10.0
    np.testing.assert_allclose(fj[east], qx * area[east], rtol=1e-10)
    assert np.abs(fj[south]).max() <= 1e-10 * abs(qx) * area.max()


@pytest.mark.parametrize("case", CASES, ids=["2d", "3d"])
def test_oracle_rhs_form_reaches_the_same_heads(case):
    """XT3D RHS (the neighbours' terms lagged on the right-hand side)
    converges over the outer iterations to the matrix form's heads."""
    tol = dict(dvclose=1e-12, rclose=1e-10, iter1=4000, ilinmeth=2)
    m, h = aniso_model(*case)
    m.ixt3d = 2
    g = oracle.Gwf(m, oracle.settings(**tol))
    assert g.con["nja"] == g.mcon["nja"]
    st = g.timestep(kper=1, kstp=1, delt=1.0, dvclose=1e-10, mxiter=400)
    assert st["converged"] == 1 and st["outer"] > 2
    assert np.abs(g.x - h).max() < 1e-8


@pytest.mark.gpu
@pytest.mark.parametrize("icelltype,newton,transient", [(0, 0, 0), (1, 1, 1)],
                         ids=["confined", "newton"])
def test_gpu_xt3d_rhs_fill_bitexact(gblib, icelltype, newton, transient):
    m, h = aniso_model(*CASES[1], icelltype=icelltype)
    m.ixt3d = 2
    m.inewton = newton
    if transient:
        m.ss, m.sy = np.full(m.nodes, 1e-5), np.full(m.nodes, 0.15)
    g, sol = _gpu_pair(m)
    rng = np.random.default_rng(5)
    hh = h + rng.uniform(-14.0, 2.0, m.nodes)
    hold = h + rng.uniform(-1.0, 1.0, m.nodes)
    sol.heads = hh
    delt = 2.5 if transient else 0.0
    amat, rhs = sol.formulate(delt=delt, hold=hold if transient else None)
    ao, ro = g.assemble(hh, hold=hold, delt=delt, transient=bool(transient))
    assert amat.size == ao.size == g.mcon["nja"]
    np.testing.assert_array_equal(amat, ao)
    np.testing.assert_array_equal(rhs, ro)


@pytest.mark.gpu
@pytest.mark.parametrize("grid", ["dis-3d", "disv", "disu-newton"])
def test_gpu_xt3d_budget_flows_bitexact(gblib, grid):
    """FLOW-JA-FACE of an XT3D model (xt3d_flowja) on the device against the
    oracle's, bit for bit, and the model budget to rounding."""
    if grid == "dis-3d":
        m, h = aniso_model(*CASES[1], icelltype=1)
        m.ss, m.sy = np.full(m.nodes, 1e-5), np.full(m.nodes, 0.15)
    elif grid == "disv":
        m, h = _general_linear(_disv(), icelltype=1)
    else:
        m, h = _general_linear(_disu(), icelltype=1)
        m.inewton = 1
    g, sol = _gpu_pair(m)
    rng = np.random.default_rng(6)
    hh = np.maximum(h, m.cell_bot + 1.0) + rng.uniform(-6.0, 1.0, m.nodes)
    hold = h.copy()
    transient = m.ss is not None
    delt = 2.0 if transient else 0.0
    sol.heads = hh
    sol.formulate(delt=delt, hold=hold if transient else None)
    fj, bg = sol.budget(flowja=True)
    fo, bo = g.budget(hh, hold=hold, delt=delt, transient=transient)
    np.testing.assert_array_equal(fj, fo)
    scale = max(1.0, float(np.abs(bo["rate_in"]).max()))
    np.testing.assert_allclose(bg["rate_in"], bo["rate_in"], rtol=1e-12, atol=1e-12 * scale)
    np.testing.assert_allclose(bg["rate_out"], bo["rate_out"], rtol=1e-12, atol=1e-12 * scale)


@pytest.mark.gpu
def test_gpu_xt3d_rhs_timestep(gblib):
    from modflow6_gb300.ims import ImsLinearSettings
    from modflow6_gb300.solution import GwfSolution, Nonlinear
    tol = dict(dvclose=1e-12, rclose=1e-10, iter1=4000, ilinmeth=2)
    m, h = aniso_model(*CASES[1])
    m.ixt3d = 2
    sol = GwfSolution(m, ImsLinearSettings(**tol), Nonlinear(dvclose=1e-10, mxiter=400))
    sg = sol.timestep(1, 1, 1.0)
    assert sg["converged"] == 1
    assert np.abs(sol.heads - h).max() < 1e-8


# ---- K22 and the angles in the standard formulation (hy_eff) ---------------

def test_oracle_k22_standard_conductances_by_hand():
    """K22 without XT3D: a connection along x takes K11, one along y K22
    (hy_eff with ANGLE1 0), in the harmonic mean of the transmissivities;
    ANGLE1 90 with K11 and K22 swapped gives the same matrix to rounding."""
    m, h = aniso_model(1, 4, 5, (0.0, 0.0, 0.0), False, xt3d=False)
    m.k22 = np.full(m.nodes, 1.0)
    m.angle1 = None
    g = oracle.Gwf(m, oracle.settings())
    a, _ = g.assemble(h)
    con = g.con
    p = 1 * m.ncol + 1
    row = slice(con["ia"][p], con["ia"][p + 1])
    cols = con["ja"][row]
    east = con["ia"][p] + int(np.flatnonzero(cols == p + 1)[0])
    south = con["ia"][p] + int(np.flatnonzero(cols == p + m.ncol)[0])
    i, j = 1, 1
    tx = 5.0 * 10.0
    hm = lambda t1, t2, c1, c2, w: w * t1 * t2 / (t1 * c2 + t2 * c1)
    assert a[east] == pytest.approx(hm(tx, tx, 0.5 * m.delr[j], 0.5 * m.delr[j + 1], m.delc[i]), rel=1e-14)
    ty = 1.0 * 10.0
    assert a[south] == pytest.approx(hm(ty, ty, 0.5 * m.delc[i], 0.5 * m.delc[i + 1], m.delr[j]), rel=1e-14)
    m.k11, m.k22 = np.full(m.nodes, 1.0), np.full(m.nodes, 5.0)
    m.angle1 = np.full(m.nodes, 90.0)
    a90, _ = oracle.Gwf(m, oracle.settings()).assemble(h)
    np.testing.assert_allclose(a90, a, rtol=1e-12, atol=1e-12 * np.abs(a).max())


@pytest.mark.gpu
@pytest.mark.parametrize("grid", ["dis", "dis-angle2", "disv", "disu"])
@pytest.mark.parametrize("iavgkeff", [0, 1])
def test_gpu_k22_angles_fill_bitexact(gblib, grid, iavgkeff):
    """K22 and ANGLE1..3 in the standard formulation: the effective K of each
    connection's direction (hy_eff, hyeff) made on the host, the saturated
    conductances and the fill on the device, against the oracle bit for bit
    (convertible cells, Newton, transient)."""
    if grid.startswith("dis") and not grid.startswith("disv") and not grid.startswith("disu"):
        m, h = aniso_model(*CASES[1], xt3d=False, icelltype=1)
        if grid == "dis":
            m.angle2 = m.angle3 = None
    elif grid == "disv":
        m, h = _general_linear(_disv(), xt3d=False, icelltype=1)
    else:
        m, h = _general_linear(_disu(), xt3d=False, icelltype=1)
    m.iavgkeff = iavgkeff
    m.inewton = 1
    m.ss, m.sy = np.full(m.nodes, 1e-5), np.full(m.nodes, 0.15)
    g, sol = _gpu_pair(m)
    rng = np.random.default_rng(7)
    hh = np.maximum(h, m.cell_bot + 1.0) + rng.uniform(-8.0, 2.0, m.nodes)
    hold = h + rng.uniform(-1.0, 1.0, m.nodes)
    sol.heads = hh
    amat, rhs = sol.formulate(delt=2.5, hold=hold)
    ao, ro = g.assemble(hh, hold=hold, delt=2.5, transient=True)
    np.testing.assert_array_equal(amat, ao)
    np.testing.assert_array_equal(rhs, ro)


def test_oracle_solves_the_xt3d_workload():
    """The seeded full-tensor workload that the bench measures (a scaled
    copy): the wider pattern, BiCGSTAB to closure in the oracle, heads
    between the CHD heads where the wells do not pull them down, and the
    model budget closing (percent discrepancy below 1e-6)."""
    from modflow6_gb300.dis import make_config
    m = make_config("xt3d", seed=0, scale=0.1)
    assert m.ixt3d == 1 and m.nodes == 3 * 20 * 20
    tol = dict(dvclose=1e-8, rclose=1e-6, iter1=4000, ilinmeth=2)
    g = oracle.Gwf(m, oracle.settings(**tol))
    assert g.con["nja"] > 7 * m.nodes  # neighbours of neighbours
    so = g.timestep(kper=1, kstp=1, delt=1.0, transient=False, dvclose=1e-8, mxiter=20)
    assert so["converged"] == 1
    assert g.x.max() <= 28.0 + 1e-9
    _, b = g.budget(g.x)
    assert abs(b["percent_discrepancy"]) < 1e-6
