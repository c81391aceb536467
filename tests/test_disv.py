"""DISV (vertex) grids: the library's connectivity (modflow6_gb300.disv)
equals the oracle's restatement of disvconnections / vertexconnect / cprops
(Connections.f90:702-796, 1272-1361; DisvGeom.f90:136-445) bit for bit, on
seeded hexagon meshes and a DIS-like quadrilateral mesh whose connectivity
must equal the DIS one; and the oracle solves a DISV model to closure."""
import numpy as np
import pytest

import oracle
from modflow6_gb300.dis import dis_connections
from modflow6_gb300.disv import close_vertex_lists, disv_connections, hex_mesh, make_disv_model


@pytest.mark.parametrize("nlay,nx,ny,seed", [(1, 6, 5, 0), (3, 12, 9, 1), (2, 25, 17, 2)])
def test_connectivity_matches_oracle(nlay, nx, ny, seed):
    m = make_disv_model(nlay, nx, ny, seed=seed)
    con = m.connections()
    iav, jav = m.vertex_lists
    o = oracle.disv_connect(nlay, iav, jav, m.vertices[:, 0], m.vertices[:, 1], m.xc, m.yc,
                            m.user_top, m.botm)
    for k in ("ia", "ja", "isym", "jas", "ihc"):
        np.testing.assert_array_equal(con[k], o[k], err_msg=k)
    for k in ("cl1", "cl2", "hwva", "area"):
        np.testing.assert_array_equal(con[k], o[k], err_msg=k)
    # hexagons: every interior cell has six horizontal neighbours
    deg = np.diff(con["ia"]) - 1 - (2 if nlay > 2 else (1 if nlay == 2 else 0))
    assert deg.max() == 6


@pytest.mark.parametrize("seed", [0, 1])
def test_reduced_connectivity_matches_oracle(seed):
    """IDOMAIN 0 (removed) and -1 (vertical pass-through) cells: the
    library's connectivity equals the oracle's restatement of vertexconnect
    (Connections.f90:1272-1361), and a vertical connection through a
    pass-through cell joins the cells above and below it."""
    rng = np.random.default_rng(seed)
    nlay, nx, ny = 4, 10, 8
    ncpl = nx * ny
    idomain = np.ones(nlay * ncpl, int)
    idomain[rng.choice(nlay * ncpl, 25, replace=False)] = 0
    mid = rng.choice(ncpl, 12, replace=False) + ncpl  # layer 2 pass-through cells
    idomain[mid] = -1
    idomain[mid - ncpl] = 1
    idomain[mid + ncpl] = 1
    m = make_disv_model(nlay, nx, ny, seed=seed, idomain=idomain)
    con = m.connections()
    iav, jav = m.vertex_lists
    o = oracle.disv_connect(nlay, iav, jav, m.vertices[:, 0], m.vertices[:, 1], m.xc, m.yc,
                            m.user_top, m.botm, idomain)
    assert con["nodes"] == o["nodes"] == int((idomain > 0).sum())
    for k in ("ia", "ja", "isym", "jas", "ihc", "cl1", "cl2", "hwva"):
        np.testing.assert_array_equal(con[k], o[k], err_msg=k)
    red = con["nodereduced"]
    a, b = red[mid[0] - ncpl] - 1, red[mid[0] + ncpl] - 1
    assert b in con["ja"][con["ia"][a]:con["ia"][a + 1]]
    # the oracle solves the reduced model
    g = oracle.Gwf(m, oracle.settings(dvclose=1e-8, rclose=1e-6, iter1=2000, ilinmeth=1))
    st = g.timestep(kper=1, kstp=1, delt=1.0, transient=False, dvclose=1e-8, mxiter=20)
    assert st["converged"] == 1


def test_rectangular_disv_equals_dis():
    """A DISV grid of unit rectangles numbered like DIS gives the DIS
    connectivity and geometry."""
    nlay, nrow, ncol = 2, 4, 5
    delr, delc = 10.0, 10.0
    vid = lambda i, j: i * (ncol + 1) + j
    verts = np.array([[j * delr, (nrow - i) * delc] for i in range(nrow + 1) for j in range(ncol + 1)])
    icvert = [[vid(i, j), vid(i, j + 1), vid(i + 1, j + 1), vid(i + 1, j)]
              for i in range(nrow) for j in range(ncol)]
    xc = np.array([(j + 0.5) * delr for i in range(nrow) for j in range(ncol)])
    yc = np.array([(nrow - i - 0.5) * delc for i in range(nrow) for j in range(ncol)])
    top = np.full(nlay * nrow * ncol, 10.0)
    top[nrow * ncol:] = 5.0
    bot = np.concatenate([np.full(nrow * ncol, 5.0), np.zeros(nrow * ncol)])
    iav, jav = close_vertex_lists(icvert)
    c = disv_connections(nlay, iav, jav, verts[:, 0], verts[:, 1], xc, yc, top, bot)
    d = dis_connections(nlay, nrow, ncol, np.full(ncol, delr), np.full(nrow, delc), top, bot)
    for k in ("ia", "ja", "isym", "jas", "ihc", "cl1", "cl2", "hwva"):
        np.testing.assert_array_equal(c[k], d[k], err_msg=k)


def test_oracle_solves_a_disv_model():
    m = make_disv_model(3, 20, 14, seed=4)
    g = oracle.Gwf(m, oracle.settings(dvclose=1e-8, rclose=1e-6, iter1=2000, ilinmeth=1))
    st = g.timestep(kper=1, kstp=1, delt=1.0, transient=False, dvclose=1e-8, mxiter=20)
    assert st["converged"] == 1
    # the residual of the converged heads on the assembled system is small
    amat, rhs = g.assemble(g.x)
    con = g.con
    r = rhs - oracle.amux(con["ia"], con["ja"], amat, g.x)
    act = m.ibound > 0
    assert np.max(np.abs(r[act])) < 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("newton", [False, True])
def test_gpu_fill_on_disv_bitexact(gblib, newton):
    """gbnpf_fill (npf_cf, npf_fc, npf_fn) on a DISV grid's connectivity
    against the oracle's, bit for bit."""
    import ctypes as C
    import torch
    from modflow6_gb300 import _lib
    m = make_disv_model(3, 18, 12, seed=5, newton=newton)
    g = oracle.Gwf(m, oracle.settings())
    con = m.connections()
    lib = oracle.load()
    dpp, ipp = C.POINTER(C.c_double), C.POINTER(C.c_int)
    lib.or_npf_cf.argtypes = [C.POINTER(oracle.GwfModel), ipp, dpp, dpp]
    lib.or_npf_fc.argtypes = [C.POINTER(oracle.GwfModel), ipp, dpp, dpp, dpp, dpp, dpp]
    lib.or_npf_fn.argtypes = [C.POINTER(oracle.GwfModel), ipp, dpp, dpp, dpp, dpp]
    rng = np.random.default_rng(6)
    h = np.ascontiguousarray(m.strt + rng.uniform(-15.0, 3.0, m.nodes))
    ib = np.ascontiguousarray(m.ibound, np.int32)
    sat = np.ones(m.nodes)  # npf_ar initial saturation
    ao, ro = np.zeros(con["nja"]), np.zeros(m.nodes)
    lib.or_npf_cf(C.byref(g.model), oracle.ip(ib), oracle.dp(h), oracle.dp(sat))
    lib.or_npf_fc(C.byref(g.model), oracle.ip(ib), oracle.dp(g.condsat), oracle.dp(sat),
                  oracle.dp(h), oracle.dp(ao), oracle.dp(ro))
    if newton:
        lib.or_npf_fn(C.byref(g.model), oracle.ip(ib), oracle.dp(g.condsat), oracle.dp(h),
                      oracle.dp(ao), oracle.dp(ro))
    keep = {k: np.ascontiguousarray(v) for k, v in con.items() if isinstance(v, np.ndarray)}
    arrs = dict(top=np.ascontiguousarray(m.cell_top), bot=np.ascontiguousarray(m.cell_bot),
                k11=np.ascontiguousarray(m.k11), k33=np.ascontiguousarray(m.k33),
                ict=np.ascontiguousarray(m.icelltype, np.int32))
    opt = _lib.GbnpfOptions(int(newton), 0, 0, 0, 1.0e-6, 0, 0)
    hh = C.c_void_p()
    assert gblib.gbnpf_create(C.byref(opt), m.nodes, con["nja"], con["njas"],
                              _lib.iptr(keep["ia"]), _lib.iptr(keep["ja"]), _lib.iptr(keep["jas"]),
                              _lib.iptr(keep["isym"]), _lib.iptr(keep["ihc"]),
                              _lib.dptr(keep["cl1"]), _lib.dptr(keep["cl2"]),
                              _lib.dptr(keep["hwva"]), _lib.dptr(arrs["top"]),
                              _lib.dptr(arrs["bot"]), _lib.dptr(arrs["k11"]),
                              _lib.dptr(arrs["k33"]), _lib.iptr(arrs["ict"]), C.byref(hh)) == 0
    dev = torch.device("cuda")
    d_amat = torch.zeros(con["nja"], dtype=torch.float64, device=dev)
    d_rhs = torch.zeros(m.nodes, dtype=torch.float64, device=dev)
    d_ib = torch.from_numpy(ib).to(dev)
    d_h = torch.from_numpy(h).to(dev)
    torch.cuda.synchronize()
    assert gblib.gbnpf_fill(hh, d_ib.data_ptr(), d_h.data_ptr(), d_amat.data_ptr(),
                            d_rhs.data_ptr()) == 0
    gblib.gbnpf_destroy(hh)
    np.testing.assert_array_equal(d_amat.cpu().numpy(), ao)
    np.testing.assert_array_equal(d_rhs.cpu().numpy(), ro)


@pytest.mark.gpu
@pytest.mark.parametrize("ilinmeth", [1, 2])
def test_gpu_solve_on_disv(gblib, ilinmeth):
    """The IMS solve of an assembled DISV system on the general-pattern path
    (SELL-32 product, level-scheduled ILU0): heads within 0.1 x INNER_DVCLOSE
    of the oracle's solve for PCG (the reference's sweep order), at closure
    parity for BiCGSTAB."""
    from modflow6_gb300.ims import ImsLinear, ImsLinearSettings
    from test_gpu_ims import assert_closure_parity
    m = make_disv_model(3, 24, 16, seed=7)
    g = oracle.Gwf(m, oracle.settings())
    x0 = g.x.copy()
    x0[m.chd_node] = m.chd_head
    amat, rhs = g.assemble(x0)
    amat, rhs = g.fixups(amat, rhs, x0, isymmetric=(ilinmeth == 1))
    tol = dict(dvclose=1e-8, rclose=1e-6, iter1=2000, ilinmeth=ilinmeth)
    o = oracle.Ims(oracle.settings(**tol), g.con["ia"], g.con["ja"])
    xo = x0.copy()
    icnvg_o, it_o, _ = o.apply(amat.copy(), rhs.copy(), xo)
    ims = ImsLinear(ImsLinearSettings(**tol)).imslinear_allocate(m.nodes, g.con["ia"], g.con["ja"])
    x = x0.copy()
    r = ims.imslinear_apply(amat.copy(), rhs.copy(), x)
    assert r.icnvg == 1 and icnvg_o == 1 and r.summary["structured"] == 0
    ts = oracle.settings(ilinmeth=ilinmeth, dvclose=1e-13, rclose=1e-11, iter1=20000)
    x_star = x0.copy()
    oracle.Ims(ts, g.con["ia"], g.con["ja"]).apply(amat.copy(), rhs.copy(), x_star)
    assert_closure_parity(x, xo, x_star, tol["dvclose"], ilinmeth == 1)


@pytest.mark.gpu
def test_gpu_timestep_on_reduced_disv(gblib):
    """A DISV grid with removed and pass-through cells through the
    device-resident time step (gbsln_create_grid), against the oracle's."""
    from modflow6_gb300.ims import ImsLinearSettings
    from modflow6_gb300.solution import GwfSolution, Nonlinear
    rng = np.random.default_rng(3)
    nlay, nx, ny = 3, 16, 12
    ncpl = nx * ny
    idomain = np.ones(nlay * ncpl, int)
    interior = np.flatnonzero((np.arange(ncpl) % nx > 0) & (np.arange(ncpl) % nx < nx - 1))
    idomain[rng.choice(interior, 8, replace=False)] = 0
    idomain[ncpl + rng.choice(interior, 10, replace=False)] = -1
    m = make_disv_model(nlay, nx, ny, seed=3, idomain=idomain)
    tol = dict(dvclose=1e-9, rclose=1e-7, iter1=2000, ilinmeth=1)
    g = oracle.Gwf(m, oracle.settings(**tol))
    so = g.timestep(kper=1, kstp=1, delt=1.0, dvclose=1e-7, mxiter=50)
    sol = GwfSolution(m, ImsLinearSettings(**tol), Nonlinear(dvclose=1e-7, mxiter=50))
    sg = sol.timestep(1, 1, 1.0)
    assert so["converged"] == 1 and sg["converged"] == 1
    assert abs(sg["outer"] - so["outer"]) <= 1
    assert np.max(np.abs(sol.heads - g.x)) <= 1e-8
