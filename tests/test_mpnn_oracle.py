"""The CPU oracle of the warm-start network: its backward pass against
central finite differences (float64, no BF16 rounding), so that the GPU
gradients can be checked against it."""
import numpy as np

import mpnn_oracle as mo
from modflow6_gb300.dis import dis_connections


def small_graph(seed=0):
    rng = np.random.default_rng(seed)
    nlay, nrow, ncol = 2, 3, 4
    con = dis_connections(nlay, nrow, ncol, np.full(ncol, 10.0), np.full(nrow, 10.0),
                          np.repeat([20.0, 10.0], nrow * ncol), np.repeat([10.0, 0.0], nrow * ncol))
    ia, ja = con["ia"], con["ja"]
    amat = -rng.uniform(0.5, 2.0, ja.size)
    # symmetric conductances: a_ij = a_ji
    n = ia.size - 1
    for i in range(n):
        for p in range(ia[i] + 1, ia[i + 1]):
            j = ja[p]
            if j < i:
                q = next(q for q in range(ia[j] + 1, ia[j + 1]) if ja[q] == i)
                amat[p] = amat[q]
    return ia, ja, amat, n


def test_oracle_gradient_matches_finite_differences():
    ia, ja, amat, n = small_graph()
    rng = np.random.default_rng(1)
    w = mo.edge_weights(ia, ja, amat, np.float64)
    X = rng.normal(size=(n, mo.FEATURES))
    t = rng.normal(size=n)
    mask = (rng.uniform(size=n) > 0.2).astype(float)
    inv = 1.0 / mask.sum()
    p = rng.normal(scale=0.2, size=mo.layout()["total"])
    loss, g, _ = mo.loss_and_grad(p, ia, ja, w, X, t, mask, inv, bf16_ops=False)
    o = mo.layout()
    idx = list(rng.choice(o["total"], size=40, replace=False)) + list(range(o["wout"], o["total"]))
    eps = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += eps
        pm[k] -= eps
        fd = (mo.loss_and_grad(pp, ia, ja, w, X, t, mask, inv, False)[0]
              - mo.loss_and_grad(pm, ia, ja, w, X, t, mask, inv, False)[0]) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-5 * max(1.0, abs(fd)), (k, fd, g[k])


def test_bf16_rounding_is_nearest_even():
    a = np.array([1.0, 1.00390625, 1.0078125, 3.14159265, -2.5e-3], np.float32)
    b = mo.bf16(a)
    # 1 + 2^-8 is halfway between 1 and 1 + 2^-7: ties go to the even mantissa (1.0)
    assert b[0] == 1.0 and b[1] == 1.0 and b[2] == np.float32(1.0078125)
    assert abs(b[3] - 3.140625) < 1e-7
    assert np.all(np.abs(b - a) <= np.abs(a) * 2.0 ** -8)
