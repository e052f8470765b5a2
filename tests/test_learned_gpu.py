"""GPU checks of the learned Poisson preconditioner.

* FP32 training kernels (forward, loss gradient, Adam) against the FP64 CPU
  oracle of the network (itself pinned by finite differences and torch conv3d).
* BF16 tcgen05 inference kernels against the oracle / the FP32 forward, at the
  BF16 tolerance (activations and weights rounded to 8 mantissa bits per layer).
* The learned Poisson mode: every inner preconditioner (hybrid, net, none,
  V-cycle) converges to the FP64 true-residual tolerance and agrees with the
  FP64 multigrid solution; broken weights fall back to the V-cycle.
"""
import ctypes as C
import os

import numpy as np
import pytest
import torch

import intfadv as ia
from intfadv import _lib, learned
from intfadv.fields import fzeros, ptr
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def rand_case(B, nx, ny, nz, seed, dev="cuda"):
    rng = np.random.default_rng(seed)
    x0 = np.zeros((B, nz + 2, ny + 2, nx + 2, 4), np.float32)
    x0[:, 1:-1, 1:-1, 1:-1, :] = rng.standard_normal((B, nz, ny, nx, 4))
    tgt = np.zeros((B, nz + 2, ny + 2, nx + 2), np.float32)
    tgt[:, 1:-1, 1:-1, 1:-1] = rng.standard_normal((B, nz, ny, nx))
    return x0, tgt, torch.tensor(x0, device=dev), torch.tensor(tgt, device=dev)


def params(seed):
    w = learned.init_params(seed)
    rng = np.random.default_rng(seed + 7)
    for (wo, bo), co in zip(learned.layer_offsets(), learned.COUT):
        w[bo:bo + co] = 0.1 * rng.standard_normal(co)
    return w


@pytest.fixture(scope="module")
def net(cuda):
    return learned.Net()


def test_fp32_forward_matches_oracle(net):
    w = params(1)
    net.set_params(w)
    x0, _, gx, _ = rand_case(2, 8, 12, 16, seed=3)
    ref = O.nn_forward(w.astype(np.float64), x0.astype(np.float64))
    out = net.forward(gx).cpu().numpy()
    assert np.all(out[:, 0] == 0) and np.all(out[:, :, :, -1] == 0)
    err = np.abs(out - ref).max() / np.abs(ref).max()
    assert err < 2e-6, err


def test_loss_gradient_matches_oracle(net):
    w = params(2)
    net.set_params(w)
    x0, tgt, gx, gt = rand_case(2, 8, 8, 12, seed=5)
    loss_o, g_o = O.nn_loss_grad(w.astype(np.float64), x0.astype(np.float64), tgt.astype(np.float64))
    loss_g, g_g = net.loss_grad(gx, gt)
    g_g = g_g.cpu().numpy().astype(np.float64)
    assert abs(loss_g - loss_o) < 1e-5 * loss_o
    for l, ((wo, bo), co) in enumerate(zip(learned.layer_offsets(), learned.COUT)):
        for a, b in ((wo, bo), (bo, bo + co)):
            e = np.abs(g_g[a:b] - g_o[a:b]).max() / np.abs(g_o[a:b]).max()
            assert e < 5e-5, (l, a, e)


def test_energy_loss_gradient_matches_oracle(net):
    w = params(3)
    net.set_params(w)
    x0, tgt, gx, gt = rand_case(2, 8, 12, 8, seed=9)
    x0[..., 1:] = np.abs(x0[..., 1:])
    gx = torch.tensor(x0, device="cuda")
    loss_o, g_o = O.nn_loss_grad(w.astype(np.float64), x0.astype(np.float64), tgt.astype(np.float64), "energy")
    net.set_loss("energy")
    try:
        loss_g, g_g = net.loss_grad(gx, gt)
    finally:
        net.set_loss("mse")
    g_g = g_g.cpu().numpy().astype(np.float64)
    assert abs(loss_g - loss_o) < 1e-5 * loss_o
    for l, ((wo, bo), co) in enumerate(zip(learned.layer_offsets(), learned.COUT)):
        for a, b in ((wo, bo), (bo, bo + co)):
            e = np.abs(g_g[a:b] - g_o[a:b]).max() / np.abs(g_o[a:b]).max()
            assert e < 5e-5, (l, a, e)


def test_adam_step_matches_oracle(net):
    w = params(4)
    net.set_params(w)
    x0, tgt, gx, gt = rand_case(1, 8, 8, 8, seed=6)
    lr = 1e-3
    net.train_step(gx, gt, lr)
    w1 = net.get_params().astype(np.float64)
    wo64 = w.astype(np.float64)
    _, g = O.nn_loss_grad(wo64, x0.astype(np.float64), tgt.astype(np.float64))
    m, v = np.zeros_like(wo64), np.zeros_like(wo64)
    O.nn_adam(wo64, g, m, v, lr, 1)
    sel = np.abs(g) > 1e-3 * np.abs(g).max()    # elsewhere ε and FP32 gradients decide the sign
    assert sel.sum() > 1000
    assert np.abs(w1[sel] - wo64[sel]).max() < 2e-5 * lr / 1e-3 + 1e-6


def test_training_reduces_loss(net):
    # a learnable target: the negated first input channel
    net.set_params(learned.init_params(0))
    _, _, gx, _ = rand_case(2, 16, 16, 16, seed=8)
    gt = (-gx[..., 0]).contiguous()
    first = net.train_step(gx, gt, 3e-3)
    for _ in range(60):
        last = net.train_step(gx, gt, 3e-3)
    assert last < 0.5 * first, (first, last)


@pytest.mark.parametrize("dims", [(1, 12, 12, 12), (2, 16, 8, 8), (1, 8, 20, 12), (1, 136, 8, 4)])
def test_tensor_core_forward_matches_oracle(net, dims):
    # (1, 136, 8, 4): rows longer than one 128-cell tile (a full tile plus a masked 8-cell tail)
    B, nx, ny, nz = dims
    w = params(10)
    net.set_params(w)
    x0, _, gx, _ = rand_case(B, nx, ny, nz, seed=12)
    ref = O.nn_forward(w.astype(np.float64), x0.astype(np.float64))
    out = net.forward(gx, tensor_cores=True).cpu().numpy()
    assert np.isfinite(out).all()
    assert np.all(out[:, 0] == 0) and np.all(out[:, :, 0] == 0)
    d = out - ref
    rel2 = np.linalg.norm(d) / np.linalg.norm(ref)
    relmax = np.abs(d).max() / np.abs(ref).max()
    assert rel2 < 2e-2 and relmax < 6e-2, (rel2, relmax)


def test_tensor_core_forward_many_tiles(net):
    # 64³ and 256 x 32 x 16: thousands of tiles over the persistent CTAs (stages reused across tiles)
    w = params(11)
    net.set_params(w)
    for dims in ((1, 64, 64, 64), (1, 256, 32, 16)):
        _, _, gx, _ = rand_case(*dims, seed=13)
        ref = net.forward(gx).cpu().numpy()
        out = net.forward(gx, tensor_cores=True).cpu().numpy()
        rel2 = np.linalg.norm(out - ref) / np.linalg.norm(ref)
        assert rel2 < 2e-2, (dims, rel2)


# ------------------------------------------------------------------ learned Poisson mode
def bubble_system(N=32):
    """Face coefficients and a right-hand side of a bubbly pressure system (one step of a run)."""
    sim = ia.TwoPhaseSimulation((N, N, N), (0.0, 0.0, 0.0), float(N), perdir=(0, 2), λρ=1e-3, λμ=1e-2, ν=0.01,
                                η=0.02, g=(0.0, -1e-3, 0.0),
                                InterfaceSDF=learned.bubbles_sdf(learned.bubble_layout(1000, N)),
                                poisson="mixed", poisson_tol=1e-9, poisson_itmx=300)
    ia.sim_step(sim)
    return sim.flow.mu0.clone(), sim.flow.sigma.clone()


def solve(poisson, L, z, precond="hybrid", weights=None, tol=1e-8, inner_max=30):
    N = L.shape[0] - 2
    h = ia.Handle(ia.make_config((N, N, N), perdir=(0, 2), poisson=poisson, lrho=1e-3))
    if poisson == "learned":
        ia.set_learned(h, precond=precond, weights=weights, inner_max=inner_max)
    x = fzeros(z.shape)
    it, res = C.c_int32(), C.c_double()
    rc = h.call("ia_poisson_solve", ptr(x), ptr(z), ptr(L), tol, 2000, C.byref(it), C.byref(res))
    _lib.check(rc, "ia_poisson_solve")
    st = ia.poisson_stats(h) if poisson == "learned" else None
    return x, it.value, res.value, st


def centred(x):
    xi = x[1:-1, 1:-1, 1:-1]
    return xi - xi.mean()


@pytest.fixture(scope="module")
def system(cuda):
    return bubble_system()


def test_learned_modes_converge_and_agree(system):
    L, z = system
    xref, it_ref, res_ref, _ = solve("fp64", L, z)
    assert res_ref <= 1e-8
    wts = params(21)
    for precond in ("hybrid", "net", "none", "vcycle"):
        x, it, res, st = solve("learned", L, z, precond=precond, weights=wts, inner_max=400)
        assert res <= 1e-8, (precond, res, st)
        e = float((centred(x) - centred(xref)).abs().max() / centred(xref).abs().max())
        assert e < 1e-5, (precond, e)
        if precond in ("hybrid", "net"):
            assert st["net"] > 0
        if precond == "vcycle":
            assert st["net"] == 0 and st["vcycles"] > 0


def test_broken_weights_fall_back_to_vcycle(system):
    L, z = system
    bad = np.full(learned.param_count(), np.nan, dtype=np.float32)
    x, it, res, st = solve("learned", L, z, precond="net", weights=bad)
    assert res <= 1e-8
    assert st["fallbacks"] == 1 and st["vcycles"] > 0


def test_untrained_hybrid_matches_vcycle_iterations_when_net_is_zero(system):
    # zero weights: the net outputs zero, ω = 0 and the hybrid is exactly the V-cycle preconditioner
    # of the same solver settings
    L, z = system
    zero = np.zeros(learned.param_count(), dtype=np.float32)
    x_h, it_h, res_h, st = solve("learned", L, z, precond="hybrid", weights=zero)
    x_v, it_v, res_v, _ = solve("learned", L, z, precond="vcycle", weights=zero)
    assert it_h == it_v and res_h <= 1e-8 and st["fallbacks"] == 0
    assert torch.equal(x_h, x_v)


def _cos(a, b):
    a, b = a.double().flatten(), b.double().flatten()
    return float((a @ b) / (a.norm() * b.norm()))


@pytest.mark.skipif(not os.path.exists(learned.WEIGHTS), reason="no trained weights shipped")
def test_trained_net_predicts_held_out_corrections(net):
    # what training gains: on patch pairs from runs the training never saw (seeds 5000+), the
    # shipped net's output is aligned with the multigrid correction; the untrained net's is not
    gen = learned.PairGenerator(N=128, P=64, seed_base=5000, steps_per_run=1)
    pairs = []
    for k, pr in enumerate(gen.pairs()):
        pairs.append(pr)
        if k >= 9:
            break
    net.set_params(learned.load_params()[0])
    trained = [_cos(net.forward(x0)[0, 1:-1, 1:-1, 1:-1], t[0, 1:-1, 1:-1, 1:-1]) for x0, t in pairs]
    net.set_params(learned.init_params(7))
    untrained = [_cos(net.forward(x0)[0, 1:-1, 1:-1, 1:-1], t[0, 1:-1, 1:-1, 1:-1]) for x0, t in pairs]
    assert np.median(trained) > 0.6, trained
    assert np.median(trained) > np.median(np.abs(untrained)) + 0.2, (trained, untrained)


@pytest.mark.skipif(not os.path.exists(learned.WEIGHTS), reason="no trained weights shipped")
def test_trained_hybrid_converges_without_fallback(system):
    # the shipped net inside the hybrid preconditioner converges to the FP64 tolerance with no
    # fallback.  It does not reduce the iteration count (on this 32³ system it needs more FCG
    # iterations than the V-cycle alone); the bound only pins that it stays within 2x.
    L, z = system
    _, it_v, res_v, _ = solve("learned", L, z, precond="vcycle")
    _, it_h, res_h, st = solve("learned", L, z, precond="hybrid")
    assert res_v <= 1e-8 and res_h <= 1e-8
    assert st["fallbacks"] == 0 and st["net"] == it_h
    assert it_h <= 2 * it_v + 2, (it_h, it_v)
