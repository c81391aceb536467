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


def gwf_like_matrix(ia, ja, amat_sym, n, storage=0.1):
    """A GWF-shaped matrix on the pattern: off-diagonal +c (symmetric, c > 0),
    diagonal -(sum c + storage), so that -A is symmetric positive definite."""
    a = -np.asarray(amat_sym, float)  # off-diagonal conductances, positive
    for i in range(n):
        a[ia[i]] = -(a[ia[i] + 1:ia[i + 1]].sum() + storage)
    return a


def test_oracle_energy_gradient_matches_finite_differences():
    """The energy loss (relative e'(-A)e of the predicted head change) and
    its gradient, against central finite differences in float64."""
    ia, ja, amat, n = small_graph(3)
    A = gwf_like_matrix(ia, ja, amat, n)
    rng = np.random.default_rng(4)
    w = mo.edge_weights(ia, ja, A, np.float64)
    X = rng.normal(size=(n, mo.FEATURES))
    t = rng.normal(scale=0.5, size=n)
    mask = (rng.uniform(size=n) > 0.2).astype(float)
    inv = 1.0 / mask.sum()
    p = rng.normal(scale=0.2, size=mo.layout()["total"])
    # a unit scale that keeps sinh(y * scale) in its curved but finite range
    y0 = mo.loss_and_grad(p, ia, ja, w, X, t, mask, inv, bf16_ops=False)[2]
    en = dict(amat=A, soft=0.01, scale=2.0 / np.max(np.abs(y0)), mse_weight=0.05)
    loss, g, y = mo.loss_and_grad(p, ia, ja, w, X, t, mask, inv, bf16_ops=False, energy=en)
    # the loss of a zero change is 1 (the previous heads' own error), up to the MSE term
    l0, _ = mo._energy_terms(ia, ja, A, np.zeros(n), t, mask, en["soft"], en["scale"])
    assert abs(l0 - 1.0) < 1e-12
    o = mo.layout()
    idx = list(rng.choice(o["total"], size=40, replace=False)) + list(range(o["wout"], o["total"]))
    eps = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += eps
        pm[k] -= eps
        fd = (mo.loss_and_grad(pp, ia, ja, w, X, t, mask, inv, False, energy=en)[0]
              - mo.loss_and_grad(pm, ia, ja, w, X, t, mask, inv, False, energy=en)[0]) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-5 * max(1.0, abs(fd)), (k, fd, g[k])
