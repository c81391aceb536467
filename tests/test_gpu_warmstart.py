"""Learned warm start on the GPU: the network's gradients against the CPU
oracle (same BF16 rounding of the GEMM operands) for both losses, training
that lowers the loss, and on held-out models a trained network whose first
iterate is closer to the converged heads than the previous heads in the
energy norm of the step's matrix and saves inner iterations, while every
step still reaches the same closure."""
import numpy as np
import pytest

import mpnn_oracle as mo
from modflow6_gb300.warmstart import (Graph, WarmStartNet, c5_model, evaluate, generate,
                                      new_solution, train, C5_DELT, DH_SOFT)

pytestmark = pytest.mark.gpu


def test_gradients_match_oracle(gblib):
    import torch
    m = c5_model(3, scale=0.05)
    g = Graph(m)
    sol = new_solution(m)
    amat, _ = sol.formulate(C5_DELT, hold=m.strt)
    sol.close()
    net = WarmStartNet(g, seed=5)
    net.set_graph(torch.from_numpy(amat).cuda())
    rng = np.random.default_rng(0)
    h = torch.from_numpy(m.strt + rng.normal(scale=1.0, size=m.nodes)).cuda()
    dh = torch.from_numpy(rng.normal(scale=0.3, size=m.nodes)).cuda()
    x = g.features(h, dh, 1.0).contiguous()
    t = torch.from_numpy(rng.normal(scale=0.5, size=m.nodes).astype(np.float32)).cuda()
    mask = g.active
    inv = 1.0 / float(mask.sum().item())
    loss_gpu, grad_gpu = net.gradients(x, t, mask, inv)
    w = mo.edge_weights(g.ia, g.ja, amat, np.float32)
    loss_o, grad_o, _ = mo.loss_and_grad(net.params.astype(np.float64), g.ia, g.ja, w,
                                         x.cpu().numpy(), t.cpu().numpy(), mask.cpu().numpy(),
                                         inv, bf16_ops=True)
    assert abs(loss_gpu - loss_o) <= 1e-3 * abs(loss_o), (loss_gpu, loss_o)
    rel = np.linalg.norm(grad_gpu - grad_o) / np.linalg.norm(grad_o)
    cos = float(grad_gpu @ grad_o / (np.linalg.norm(grad_gpu) * np.linalg.norm(grad_o)))
    assert rel <= 2e-2 and cos >= 0.9995, (rel, cos)
    net.close()


def test_energy_gradients_match_oracle(gblib):
    """The energy loss (gbmpnn_set_loss mode 1) and its gradients against the
    oracle on a C5-type model's own matrix."""
    import torch
    m = c5_model(4, scale=0.05)
    g = Graph(m)
    sol = new_solution(m)
    amat, _ = sol.formulate(C5_DELT, hold=m.strt)
    sol.close()
    net = WarmStartNet(g, seed=6)
    net.dh_scale, net.unit_max = 1.5, 0.0
    net.set_graph(torch.from_numpy(amat).cuda())
    net.set_loss("energy", mse_weight=0.05)
    rng = np.random.default_rng(2)
    h = torch.from_numpy(m.strt + rng.normal(scale=1.0, size=m.nodes)).cuda()
    dh = torch.from_numpy(rng.normal(scale=0.3, size=m.nodes)).cuda()
    x = g.features(h, dh, 1.0).contiguous()
    t = (torch.from_numpy(rng.normal(scale=0.5, size=m.nodes).astype(np.float32)).cuda()
         * g.active)
    mask = g.active
    inv = 1.0 / float(mask.sum().item())
    loss_gpu, grad_gpu = net.gradients(x, t, mask, inv)
    w = mo.edge_weights(g.ia, g.ja, amat, np.float32)
    en = dict(amat=amat, soft=DH_SOFT, scale=1.5, mse_weight=0.05)
    loss_o, grad_o, _ = mo.loss_and_grad(net.params.astype(np.float64), g.ia, g.ja, w,
                                         x.cpu().numpy(), t.cpu().numpy(), mask.cpu().numpy(),
                                         inv, bf16_ops=True, energy=en)
    assert abs(loss_gpu - loss_o) <= 1e-3 * abs(loss_o), (loss_gpu, loss_o)
    rel = np.linalg.norm(grad_gpu - grad_o) / np.linalg.norm(grad_o)
    cos = float(grad_gpu @ grad_o / (np.linalg.norm(grad_gpu) * np.linalg.norm(grad_o)))
    assert rel <= 2e-2 and cos >= 0.9995, (rel, cos)
    net.close()


def test_training_lowers_loss_and_improves_the_initial_guess(gblib):
    data, dh_scale = generate(range(100, 110), steps=10, scale=0.25)
    net = WarmStartNet(data[0][0], seed=1)
    hist = train(net, data, dh_scale, epochs=6, lr=2e-3)
    assert hist[-1] < 0.5 * hist[0], hist
    res = evaluate(net, [900, 901], steps=10, scale=0.25)
    print(res)
    # every step of the three paths reaches the same closure
    assert res["all_converged"], res
    # the warm path takes strictly fewer inner iterations than MODFLOW 6's
    # start from the previous heads, its fallbacks and their wasted
    # iterations counted
    assert res["inner_warm"] < res["inner_prev_heads"], res
    # what the network adds to the last step's change: on the first step
    # there is no last change, and the network's direction alone removes a
    # clear part of the energy error of the previous heads; over all steps
    # the plane is no worse than the last change alone
    assert res["energy_err_warm_first_step_rel"] < 0.97, res
    assert res["energy_err_warm_rel"] <= res["energy_err_extrap_rel"] + 1e-3, res
    net.close()


def test_fallback_drops_a_bad_guess(gblib):
    """A guess far from the heads (every head +50 m) spends its budget and
    is dropped: the step is solved again from the previous heads, reaches the
    same closure and heads as the plain step, and reports the fallback with
    both attempts' iterations."""
    import torch
    from modflow6_gb300.warmstart import timestep_warm
    m = c5_model(7, scale=0.1)
    plain, warm = new_solution(m), new_solution(m)
    s0 = plain.timestep(1, 1, C5_DELT)
    guess = torch.from_numpy(m.strt + 50.0).cuda()
    st, fell = timestep_warm(warm, 1, 1, C5_DELT, guess, inner_cap=max(1, s0["inner_total"] // 4))
    assert fell and st["converged"] == 1
    assert st["inner_total"] > s0["inner_total"]
    assert np.max(np.abs(warm.heads - plain.heads)) <= 1e-6
    plain.close()
    warm.close()
