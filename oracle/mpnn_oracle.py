"""CPU oracle of the warm-start network (test infrastructure only).

A numpy restatement of the message-passing network that the GPU trains and
evaluates (modflow6_gb300/csrc/k_mpnn.cu), forward and backward, used to
check the GPU gradients.  With `bf16=True` the GEMM operands are rounded to
bfloat16 (round to nearest even) exactly where the GPU rounds them and the
rest runs in float32, so the GPU and the oracle differ only by summation
order; with `bf16=False` everything is float64, for finite-difference checks
of the oracle itself.

Network (hidden 64, 8 layers, 16 input features):
  H0 = relu(X W0 + b0);  A_l = S H_{l-1};  Z_l = [H_{l-1}, A_l] W_l + b_l;
  H_l = H_{l-1} + relu(Z_l);  y = H_8 wout + bout;
  loss = sum(((y - t) * mask)^2) * inv_count, or with `energy` (the loss of
  gbmpnn_set_loss mode 1, k_mpnn.cu k_energy_*): with dh(u) = soft*sinh(u*scale),
  e = mask*(dh(y) - dh(t)), t' = mask*dh(t) and W = -A over the active rows,
  loss = e'We / t''Wt' + mse_weight * sum(((y - t) * mask)^2) * inv_count.
S_ij = c_ij / sqrt(d_i d_j) with c_ij = max(-a_ij, 0) over the off-diagonal
CSR entries and d_i = sum_j c_ij.
"""
from __future__ import annotations

import numpy as np

HIDDEN, LAYERS, FEATURES = 64, 8, 16
CAT = 2 * HIDDEN


def layout():
    """Offsets of W0, b0, (W_l, b_l) l=1..8, wout, bout in the flat vector."""
    off = {"w0": 0, "b0": FEATURES * HIDDEN}
    o = off["b0"] + HIDDEN
    for l in range(1, LAYERS + 1):
        off[f"w{l}"] = o
        off[f"b{l}"] = o + CAT * HIDDEN
        o += CAT * HIDDEN + HIDDEN
    off["wout"] = o
    off["bout"] = o + HIDDEN
    off["total"] = o + HIDDEN + 1
    return off


def bf16(a: np.ndarray) -> np.ndarray:
    """float32 -> bfloat16 (round to nearest even) -> float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def edge_weights(ia, ja, amat, dtype=np.float32):
    n = ia.size - 1
    c = np.maximum(-amat, 0.0)
    diag = ia[:-1]
    c[diag] = 0.0
    rows = np.repeat(np.arange(n), np.diff(ia))
    deg = np.zeros(n)
    np.add.at(deg, rows, c)
    deg = deg.astype(dtype)
    dd = deg[rows] * deg[ja]
    w = np.where(dd > 0, c.astype(dtype) / np.sqrt(np.where(dd > 0, dd, 1)).astype(dtype), 0)
    w = w.astype(dtype)
    w[diag] = 0
    return w


def _spmm(ia, ja, w, H):
    n = ia.size - 1
    rows = np.repeat(np.arange(n), np.diff(ia))
    out = np.zeros((n, H.shape[1]), dtype=H.dtype)
    np.add.at(out, rows, w[:, None].astype(H.dtype) * H[ja])
    return out


def unpack(p, dtype):
    o = layout()
    W = {"w0": p[o["w0"]:o["b0"]].reshape(FEATURES, HIDDEN).astype(dtype),
         "b0": p[o["b0"]:o["b0"] + HIDDEN].astype(dtype)}
    for l in range(1, LAYERS + 1):
        W[f"w{l}"] = p[o[f"w{l}"]:o[f"b{l}"]].reshape(CAT, HIDDEN).astype(dtype)
        W[f"b{l}"] = p[o[f"b{l}"]:o[f"b{l}"] + HIDDEN].astype(dtype)
    W["wout"] = p[o["wout"]:o["bout"]].astype(dtype)
    W["bout"] = p[o["bout"]:o["bout"] + 1].astype(dtype)
    return W


def _energy_terms(ia, ja, amat, y, target, mask, soft, scale):
    """(e'We / t'Wt, dLoss/dy) of the energy loss, in float64."""
    y = np.asarray(y, np.float64)
    m = (np.asarray(mask) > 0).astype(np.float64)
    n = m.size
    rows = np.repeat(np.arange(n), np.diff(ia))
    dh_t = soft * np.sinh(np.asarray(target, np.float64) * scale)
    e = m * (soft * np.sinh(y * scale) - dh_t)
    t = m * dh_t
    we = -np.bincount(rows, weights=amat * e[ja], minlength=n) * m
    wt = -np.bincount(rows, weights=amat * t[ja], minlength=n) * m
    den = float(t @ wt)
    inv = 1.0 / den if den > 0.0 else 0.0
    return float(e @ we) * inv, m * 2.0 * we * inv * soft * scale * np.cosh(y * scale)


def loss_and_grad(p, ia, ja, w, X, target, mask, inv_count, bf16_ops=True, energy=None):
    """(loss, flat gradient, y) of the network; see the module docstring.
    `energy`: None, or dict(amat=, soft=, scale=, mse_weight=)."""
    dt = np.float32 if bf16_ops else np.float64
    r = bf16 if bf16_ops else (lambda a: np.asarray(a, dtype=dt))
    P = unpack(np.asarray(p, dtype=np.float64), dt)
    wq = {k: (r(v) if k.startswith("w") and k != "wout" else v) for k, v in P.items()}
    w = w.astype(dt)
    Xq = r(X.astype(dt))
    Z0 = (Xq @ wq["w0"]).astype(dt) + P["b0"]
    H = [np.maximum(Z0, 0)]
    masks = [Z0 > 0]
    Hq, Aq = [r(H[0])], [None]
    for l in range(1, LAYERS + 1):
        A = _spmm(ia, ja, w, H[l - 1])
        Aq.append(r(A))
        Zl = (np.concatenate([Hq[l - 1], Aq[l]], axis=1) @ wq[f"w{l}"]).astype(dt) + P[f"b{l}"]
        masks.append(Zl > 0)
        H.append(H[l - 1] + np.maximum(Zl, 0))
        Hq.append(r(H[l]))
    y = H[LAYERS] @ P["wout"] + P["bout"][0]
    e = (y - target.astype(dt)) * mask.astype(dt)
    mw = 1.0 if energy is None else float(energy["mse_weight"])
    loss = float(np.sum(e * e) * inv_count * mw)
    dy = 2 * e * dt(inv_count * mw)
    if energy is not None:
        le, dye = _energy_terms(ia, ja, energy["amat"], y, target, mask, energy["soft"],
                                energy["scale"])
        loss += le
        dy = (dy + dye).astype(dt)
    G = {"wout": H[LAYERS].T @ dy, "bout": np.array([dy.sum()])}
    dH = np.outer(dy, P["wout"]).astype(dt)
    for l in range(LAYERS, 0, -1):
        dZ = np.where(masks[l], dH, 0).astype(dt)
        G[f"b{l}"] = dZ.sum(axis=0)
        dZq = r(dZ)
        G[f"w{l}"] = np.concatenate([Hq[l - 1], Aq[l]], axis=1).T @ dZq
        dX = (dZq @ wq[f"w{l}"].T).astype(dt)
        dH = dH + dX[:, :HIDDEN] + _spmm(ia, ja, w, dX[:, HIDDEN:])
    dZ0 = np.where(masks[0], dH, 0).astype(dt)
    G["b0"] = dZ0.sum(axis=0)
    G["w0"] = Xq.T @ r(dZ0)
    o = layout()
    g = np.zeros(o["total"])
    g[o["w0"]:o["b0"]] = G["w0"].ravel()
    g[o["b0"]:o["b0"] + HIDDEN] = G["b0"]
    for l in range(1, LAYERS + 1):
        g[o[f"w{l}"]:o[f"b{l}"]] = G[f"w{l}"].ravel()
        g[o[f"b{l}"]:o[f"b{l}"] + HIDDEN] = G[f"b{l}"]
    g[o["wout"]:o["bout"]] = G["wout"]
    g[o["bout"]] = G["bout"][0]
    return loss, g, y
