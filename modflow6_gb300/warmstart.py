"""Learned warm start for transient time steps (gbmpnn_* + gbsln_timestep_guess).

MODFLOW 6 starts every time step's outer loop from the previous heads.  Here
a message-passing network over the graph of the IMS matrix (hidden width 64,
8 layers, BF16 tensor-core GEMMs, trained on the GPU by the library's own
forward and backward kernels) predicts the head change of the step from the
cell's K, the previous heads, the previous step's head change, the well
rates and the boundary mask.  The
prediction is only an initial guess: PCG + ILU0 still runs to the same
INNER_DVCLOSE / INNER_RCLOSE closure, so the plain solver decides the heads.
The first iterate is the point of the plane through the previous heads,
spanned by the last step's head change and the network's predicted change,
that is closest to the solution in the energy norm of the step's first
system (one SpMV and five dot products on the device).  A transient step's
change is close to a multiple of the last one once the first steps have
passed, and the projection takes that multiple; the network's direction adds
what the last change lacks (the first steps, new stresses), and a noisy
prediction is shrunk instead of taken whole.  The warm step may spend at
most the inner iterations the plain solver took on the previous step; past
that it is solved again from the previous heads (gbsln_timestep_warm).

`Graph.features` builds the 16 input features of the cells, `generate` the
training samples (heads from the plain solver), `WarmStartNet` wraps the C
ABI, `train` runs Adam on the GPU and `evaluate` compares inner iterations
from the previous heads, from the last change alone and with the network on
held-out models.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .dis import GwfDisModel, make_config
from .ims import ImsLinearSettings
from .solution import GwfSolution, Nonlinear

NFEAT = 16
HEAD_REF, HEAD_SCALE = 22.5, 5.0   # c5 CHD heads are 25 m (west) and 20 m (east)
Q_SCALE = 100.0                    # well rate scale, m3/d
DH_SOFT = 0.01                     # m: head changes are learnt as asinh(dh / DH_SOFT)


def to_unit(dh):
    """Head change (m) -> network units: asinh(dh / DH_SOFT), so that the
    error of a prediction scales with the size of the change (near-zero far
    from the wells, relative near them) instead of being spread evenly."""
    import torch
    return torch.asinh(dh / DH_SOFT)


def from_unit(y):
    import torch
    return torch.sinh(y) * DH_SOFT


class Graph:
    """Static per-model inputs on the device: standardised ln K, well rate,
    CHD mask, layer position, the active-cell mask and the CSR pattern."""

    def __init__(self, m: GwfDisModel, device="cuda"):
        import torch

        self.m = m
        n = m.nodes
        lnk = np.log(m.k11)
        lnk = (lnk - lnk.mean()) / (lnk.std() + 1e-12)
        q = np.zeros(n)
        np.add.at(q, m.wel_node, m.wel_q)
        chd = np.zeros(n)
        chd[m.chd_node] = 1.0
        lay = np.repeat(np.arange(m.nlay) / max(1, m.nlay - 1), m.nrow * m.ncol)
        static = np.zeros((n, NFEAT), np.float32)
        static[:, 0] = lnk
        static[:, 2] = q / Q_SCALE
        static[:, 3] = chd
        static[:, 4] = lay
        static[:, 5] = 1.0
        self.static = torch.from_numpy(static).to(device)
        self.active = torch.from_numpy((m.ibound > 0).astype(np.float32)).to(device)
        self.active64 = self.active.double()
        con = m.connections()
        self.ia, self.ja = con["ia"], con["ja"]
        self.nja = int(con["nja"])

    def features(self, h_prev, dh_prev, dh_scale: float):
        """Device float64 previous heads and previous step's head change
        (nodes) -> float32 features (nodes x 16)."""
        x = self.static.clone()
        x[:, 1] = ((h_prev - HEAD_REF) / HEAD_SCALE).float()
        x[:, 6] = (to_unit(dh_prev) / dh_scale).float()
        return x


def c5_model(seed: int, scale: float = 1.0) -> GwfDisModel:
    return make_config("c5", seed=seed, scale=scale)


C5_IMS = dict(dvclose=1e-6, rclose=1e-4, iter1=2000, ilinmeth=1)
C5_DELT = 0.5      # days per time step
C5_STEPS = 20


def new_solution(m: GwfDisModel) -> GwfSolution:
    return GwfSolution(m, ImsLinearSettings(structure=(m.nlay, m.nrow, m.ncol), **C5_IMS),
                       Nonlinear(dvclose=C5_IMS["dvclose"], mxiter=25))


@dataclass
class Sample:
    x: object        # features (device, nodes x 16, float32)
    target: object   # scaled head change (device, nodes, float32)


def generate(seeds, steps: int = C5_STEPS, scale: float = 1.0, delt: float = C5_DELT):
    """Training data from the plain solver: per model its Graph, its
    assembled matrix (device, for the edge weights) and one Sample per step,
    and the scale (standard deviation over the active cells of every step of
    the asinh-transformed head change) that normalises the targets and the
    previous-change feature."""
    import torch

    runs = []
    for s in seeds:
        m = c5_model(s, scale)
        g = Graph(m)
        sol = new_solution(m)
        amat, _ = sol.formulate(delt, hold=m.strt)
        d_amat = torch.from_numpy(amat).cuda()
        hs = [torch.from_numpy(sol.heads).cuda()]
        for kstp in range(1, steps + 1):
            sol.timestep(1, kstp, delt)
            hs.append(torch.from_numpy(sol.heads).cuda())
        sol.close()
        runs.append((g, d_amat, hs))
    sq, cnt = 0.0, 0.0
    for g, _, hs in runs:
        for k in range(1, len(hs)):
            d = to_unit(hs[k] - hs[k - 1]) * g.active64
            sq += float((d * d).sum().item())
            cnt += float(g.active64.sum().item())
    dh_scale = max(1e-3, (sq / max(1.0, cnt)) ** 0.5)
    data = []
    for g, d_amat, hs in runs:
        samples = []
        for k in range(1, len(hs)):
            dh_prev = hs[k - 1] - hs[k - 2] if k >= 2 else torch.zeros_like(hs[0])
            x = g.features(hs[k - 1], dh_prev * g.active64, dh_scale)
            t = (to_unit(hs[k] - hs[k - 1]) / dh_scale * g.active64).float()
            samples.append(Sample(x, t))
        data.append((g, d_amat, samples))
    return data, dh_scale


class WarmStartNet:
    def __init__(self, g: Graph, seed: int = 0):
        self._lib = _lib.load()
        self._h = C.c_void_p()
        ia = np.ascontiguousarray(g.ia, np.int32)
        ja = np.ascontiguousarray(g.ja, np.int32)
        rc = self._lib.gbmpnn_create(g.m.nodes, g.nja, _lib.iptr(ia), _lib.iptr(ja), seed,
                                     C.byref(self._h))
        if rc < 0:
            raise _lib.GbimsError(rc, self._err())
        self.nodes = g.m.nodes
        self.nparams = int(self._lib.gbmpnn_param_count())
        self.dh_scale = 1.0  # output scale in asinh units, set by training
        self.unit_max = 0.0  # bound on |output| (normalised units), set by training; 0 = none

    def _err(self):
        return self._lib.gbmpnn_last_error(self._h).decode() if self._h else ""

    def _chk(self, rc):
        if rc < 0:
            raise _lib.GbimsError(rc, self._err())

    def set_graph(self, d_amat):
        self._chk(self._lib.gbmpnn_set_graph(self._h, C.c_void_p(d_amat.data_ptr())))

    def set_loss(self, mode: str, mse_weight: float = 0.0):
        """gbmpnn_set_loss: "mse" (squared error in network units) or
        "energy" (relative energy error of the predicted head change under
        the matrix of the last set_graph, plus mse_weight times the squared
        error); the unit scalings are the network's current ones."""
        m = {"mse": 0, "energy": 1}[mode]
        sc = scaling(self)
        self._chk(self._lib.gbmpnn_set_loss(self._h, m, C.byref(sc), float(mse_weight)))

    def predict(self, x):
        import torch
        y = torch.empty(self.nodes, dtype=torch.float32, device=x.device)
        torch.cuda.synchronize()
        self._chk(self._lib.gbmpnn_forward(self._h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr())))
        return y

    def train_step(self, x, target, mask, lr: float) -> float:
        import torch
        inv = 1.0 / max(1.0, float(mask.sum().item()))
        loss = C.c_float()
        torch.cuda.synchronize()
        self._chk(self._lib.gbmpnn_train_step(self._h, C.c_void_p(x.data_ptr()),
                                              C.c_void_p(target.data_ptr()),
                                              C.c_void_p(mask.data_ptr()), inv, lr, C.byref(loss)))
        return loss.value

    def gradients(self, x, target, mask, inv_count: float):
        import torch
        loss = C.c_float()
        g = np.zeros(self.nparams, np.float32)
        torch.cuda.synchronize()
        self._chk(self._lib.gbmpnn_gradients(self._h, C.c_void_p(x.data_ptr()),
                                             C.c_void_p(target.data_ptr()),
                                             C.c_void_p(mask.data_ptr()), inv_count, C.byref(loss),
                                             g.ctypes.data_as(C.POINTER(C.c_float))))
        return loss.value, g

    @property
    def params(self) -> np.ndarray:
        p = np.zeros(self.nparams, np.float32)
        self._chk(self._lib.gbmpnn_get_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float))))
        return p

    @params.setter
    def params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        self._chk(self._lib.gbmpnn_set_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float))))

    def close(self):
        if self._h:
            self._lib.gbmpnn_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def train(net: WarmStartNet, data, dh_scale: float, epochs: int = 4,
          lr: float = 1e-3, loss: str = "mse", mse_weight: float = 0.05) -> list[float]:
    """Adam over every sample of every model, `epochs` times, the learning
    rate halved each epoch; mean loss per epoch.  loss "mse" (the default)
    is the squared error in network units; "energy" the relative energy
    error of the predicted change (gbmpnn_set_loss), the error a
    conjugate-gradient solve started from the guess has to remove.  The warm
    step projects the guess in that norm anyway (gbsln_timestep_warm), so
    only the direction of the prediction matters there, and the squared
    error has proven the better teacher of directions."""
    net.dh_scale = dh_scale
    # predictions are bounded by the largest head change seen in training,
    # with a 25 % margin in metres (not in the asinh units, where the same
    # margin would allow changes many times larger): the network does not
    # extrapolate beyond its data
    tmax = 0.0
    for g, _, samples in data:
        for s in samples:
            tmax = max(tmax, float(s.target.abs().max().item()))
    dh_max = float(np.sinh(tmax * dh_scale)) * DH_SOFT
    net.unit_max = float(np.arcsinh(1.25 * dh_max / DH_SOFT)) / dh_scale
    net.set_loss(loss, mse_weight)
    hist = []
    for ep in range(epochs):
        tot, cnt = 0.0, 0
        for g, d_amat, samples in data:
            net.set_graph(d_amat)
            for s in samples:
                tot += net.train_step(s.x, s.target, g.active, lr * (0.5 ** ep))
                cnt += 1
        hist.append(tot / max(1, cnt))
    return hist


def scaling(net: WarmStartNet) -> _lib.GbmpnnScaling:
    """The head <-> network-unit scalings of gbsln_warm_guess."""
    return _lib.GbmpnnScaling(HEAD_REF, HEAD_SCALE, DH_SOFT, float(net.dh_scale), float(net.unit_max))


def warm_guess(sol: GwfSolution, net: WarmStartNet, g: Graph, guess, first: bool) -> float:
    """The network's guess for `sol`'s next step into the device tensor
    `guess`, built and evaluated on the device on the solution's stream
    (gbsln_warm_guess); returns its device time in ms."""
    lib = _lib.load()
    ms = C.c_float(0.0)
    sc = scaling(net)
    rc = lib.gbsln_warm_guess(sol._h, net._h, C.c_void_p(g.static.data_ptr()), C.byref(sc),
                              1 if first else 0, C.c_void_p(guess.data_ptr()), C.byref(ms))
    if rc < 0:
        raise _lib.GbimsError(rc, net._err())
    return float(ms.value)


def timestep_warm(sol: GwfSolution, kper: int, kstp: int, delt: float, guess, inner_cap: int):
    """gbsln_timestep_warm: the step from the energy projection of the
    previous heads onto the plane of the last step's change and the guess's
    (guess None: the last change alone), dropped in favour of the previous
    heads once it has spent inner_cap inner iterations without closing.
    Returns (stats, fell_back)."""
    lib = _lib.load()
    st = _lib.GbslnStats()
    gp = C.c_void_p(guess.data_ptr()) if guess is not None else None
    rc = lib.gbsln_timestep_warm(sol._h, kper, kstp, delt, gp, int(inner_cap), C.byref(st))
    if rc < 0:
        raise _lib.GbimsError(rc, lib.gbsln_last_error(sol._h).decode())
    return {f: getattr(st, f) for f, _ in st._fields_}, rc == _lib.GBIMS_WARN_FALLBACK


def evaluate(net: WarmStartNet, seeds, steps: int = C5_STEPS, scale: float = 1.0,
             delt: float = C5_DELT) -> dict:
    """Held-out models, each solved three times to the same closure: every
    step from the previous heads (the plain solver, as MODFLOW 6 does); from
    the energy projection onto the last step's change alone ("extrap", no
    network); and from the projection onto the last change and the
    network's predicted change ("warm").  Both projected paths keep the
    fallback rule (gbsln_timestep_warm: at most the inner iterations the
    plain solver took on the previous step, then the step again from the
    previous heads, those iterations counted too).  The guess is built,
    evaluated and used on the device with no host round trip in between.
    Reported: inner iterations and device time of the three paths (the warm
    path's time includes inference), fallbacks, the projection factors, the
    energy errors e'(-A)e of each path's first iterate relative to that of
    the previous heads (A the step's matrix), and the RMS and maximum error
    of the raw network guess and of the previous heads against the converged
    heads."""
    import torch

    it_prev, it_ext, it_warm, fell = [], [], [], 0
    rms_g, rms_p, max_g, max_p = [], [], [], []
    en_ext, en_warm, a_prev, a_net = [], [], [], []
    ms_prev, ms_ext, ms_warm, ms_net = 0.0, 0.0, 0.0, 0.0
    converged = True
    for s in seeds:
        m = c5_model(s, scale)
        g = Graph(m)
        base, ext, warm = new_solution(m), new_solution(m), new_solution(m)
        amat, _ = base.formulate(delt, hold=m.strt)
        d_amat = torch.from_numpy(amat).cuda()
        net.set_graph(d_amat)
        rows = torch.from_numpy(np.repeat(np.arange(m.nodes), np.diff(g.ia))).cuda()
        cols = torch.from_numpy(np.asarray(g.ja, np.int64)).cuda()

        def energy(e):
            # e'(-A)e over the active cells (e is zero elsewhere)
            we = torch.zeros_like(e).index_add_(0, rows, -d_amat * e[cols]) * g.active64
            return float((e * we).sum().item())

        nact = float(g.active64.sum().item())
        guess = torch.empty(m.nodes, dtype=torch.float64, device="cuda")
        last_plain = None
        prev_w = prev_e = None   # the last step's change on each projected path
        for kstp in range(1, steps + 1):
            st_b = base.timestep(1, kstp, delt)
            cap = 10 ** 9 if last_plain is None else max(1, last_plain)
            last_plain = st_b["inner_total"]
            # extrapolation only
            he0 = torch.from_numpy(ext.heads).cuda()
            st_e, fb_e = timestep_warm(ext, 1, kstp, delt, None, cap)
            he1 = torch.from_numpy(ext.heads).cuda()
            # network + extrapolation
            hw0 = torch.from_numpy(warm.heads).cuda()
            ms_net += warm_guess(warm, net, g, guess, first=(kstp == 1))
            st_w, fb_w = timestep_warm(warm, 1, kstp, delt, guess, cap)
            hw1 = torch.from_numpy(warm.heads).cuda()
            fell += int(fb_e) + int(fb_w)
            # first-iterate errors against each path's own converged heads
            act = g.active64
            ep_w = (hw0 - hw1) * act
            eg = (guess - hw1) * act
            d1w = prev_w if prev_w is not None else torch.zeros_like(ep_w)
            e0_w = ep_w + st_w["prev_alpha"] * d1w + st_w["guess_alpha"] * (eg - ep_w)
            ep_e = (he0 - he1) * act
            d1e = prev_e if prev_e is not None else torch.zeros_like(ep_e)
            e0_e = ep_e + st_e["prev_alpha"] * d1e
            Ew, Ee = energy(ep_w), energy(ep_e)
            if Ew > 0.0 and Ee > 0.0:
                en_warm.append(energy(e0_w) / Ew)
                en_ext.append(energy(e0_e) / Ee)
            prev_w, prev_e = (hw1 - hw0) * act, (he1 - he0) * act
            a_prev.append(st_w["prev_alpha"])
            a_net.append(st_w["guess_alpha"])
            rms_g.append(float(torch.sqrt((eg * eg).sum() / nact).item()))
            rms_p.append(float(torch.sqrt((ep_w * ep_w).sum() / nact).item()))
            max_g.append(float(eg.abs().max().item()))
            max_p.append(float(ep_w.abs().max().item()))
            it_prev.append(st_b["inner_total"])
            it_ext.append(st_e["inner_total"])
            it_warm.append(st_w["inner_total"])
            ms_prev += st_b["total_ms"]
            ms_ext += st_e["total_ms"]
            ms_warm += st_w["total_ms"]
            converged = converged and all(x["converged"] == 1 for x in (st_b, st_e, st_w))
        for sol in (base, ext, warm):
            sol.close()
    ip, ie, iw = np.array(it_prev), np.array(it_ext), np.array(it_warm)
    return {"models": len(seeds), "steps": int(ip.size), "all_converged": converged,
            "inner_prev_heads": int(ip.sum()), "inner_extrap": int(ie.sum()),
            "inner_warm": int(iw.sum()), "fallbacks": fell,
            "steps_warm_better": int((iw < ip).sum()), "steps_warm_worse": int((iw > ip).sum()),
            "iteration_ratio": float(iw.sum() / max(1, ip.sum())),
            "iteration_ratio_extrap": float(ie.sum() / max(1, ip.sum())),
            "solve_ms_prev_heads": ms_prev, "solve_ms_extrap": ms_ext, "solve_ms_warm": ms_warm,
            "inference_ms": ms_net, "inference_ms_per_guess": ms_net / max(1, ip.size),
            "time_ratio": (ms_warm + ms_net) / max(1e-9, ms_prev),
            "time_ratio_extrap": ms_ext / max(1e-9, ms_prev),
            "energy_err_warm_rel": float(np.mean(en_warm)) if en_warm else None,
            "energy_err_extrap_rel": float(np.mean(en_ext)) if en_ext else None,
            "energy_err_warm_first_step_rel": en_warm[0] if en_warm else None,
            "alpha_prev_mean": float(np.mean(a_prev)), "alpha_net_mean": float(np.mean(a_net)),
            "rms_err_guess": float(np.mean(rms_g)), "rms_err_prev_heads": float(np.mean(rms_p)),
            "max_err_guess": float(np.max(max_g)), "max_err_prev_heads": float(np.max(max_p)),
            "inner_per_step_prev_heads": ip.tolist(), "inner_per_step_extrap": ie.tolist(),
            "inner_per_step_warm": iw.tolist()}
