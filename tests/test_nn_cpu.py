"""CPU checks of the learned preconditioner's oracle and host logic (no GPU calls).

The reference has no learned component, so the FP64 oracle of the network
(oracle/nn_oracle.cpp) is pinned two independent ways: its backward pass
against central finite differences of its own loss, and its forward pass
against a restatement with torch CPU conv3d / avg_pool3d / nearest upsampling.
"""
import ctypes as C

import numpy as np
import pytest
import torch
import torch.nn.functional as F

from intfadv import learned
from oracle import pyoracle as O


def rand_case(B, nx, ny, nz, seed):
    rng = np.random.default_rng(seed)
    x0 = np.zeros((B, nz + 2, ny + 2, nx + 2, 4))
    x0[:, 1:-1, 1:-1, 1:-1, :] = rng.standard_normal((B, nz, ny, nx, 4))
    tgt = np.zeros((B, nz + 2, ny + 2, nx + 2))
    tgt[:, 1:-1, 1:-1, 1:-1] = rng.standard_normal((B, nz, ny, nx))
    return x0, tgt


def params(seed):
    w = learned.init_params(seed).astype(np.float64)
    # non-zero biases so every bias gradient path is exercised
    rng = np.random.default_rng(seed + 7)
    for (wo, bo), co in zip(learned.layer_offsets(), learned.COUT):
        w[bo:bo + co] = 0.1 * rng.standard_normal(co)
    return w


def torch_forward(w, x0):
    X = torch.tensor(x0[:, 1:-1, 1:-1, 1:-1, :]).permute(0, 4, 1, 2, 3)   # B, C, z, y, x

    def conv(X, l):
        (wo, bo), ci, co = learned.layer_offsets()[l], learned.CIN[l], learned.COUT[l]
        W = torch.tensor(w[wo:bo]).reshape(3, 3, 3, co, ci).permute(3, 4, 0, 1, 2)
        return F.conv3d(X, W, torch.tensor(w[bo:bo + co]), padding=1)

    up = lambda a: F.interpolate(a, scale_factor=2, mode="nearest")
    a1 = F.relu(conv(X, 0))
    a2 = F.relu(conv(F.avg_pool3d(a1, 2), 1))
    a3 = F.relu(conv(F.avg_pool3d(a2, 2), 2))
    a4 = F.relu(conv(up(a3) + a2, 3))
    a5 = F.relu(conv(up(a4), 4)) + a1
    return conv(a5, 5)[:, 0].numpy()                                       # B, z, y, x


def test_param_layout_agrees_everywhere(lib):
    assert learned.param_count() == O.nn_param_count() == lib.ia_nn_param_count() == 85233


def test_oracle_forward_matches_torch_conv3d():
    x0, _ = rand_case(2, 8, 12, 16, seed=1)
    w = params(3)
    out = O.nn_forward(w, x0)
    ref = torch_forward(w, x0)
    assert np.all(out[:, 0, :, :] == 0) and np.all(out[:, :, :, 0] == 0)   # halo untouched
    err = np.abs(out[:, 1:-1, 1:-1, 1:-1] - ref).max() / np.abs(ref).max()
    assert err < 1e-12, err


def test_oracle_gradient_matches_finite_differences():
    x0, tgt = rand_case(1, 8, 8, 8, seed=2)
    w = params(5)
    loss, g = O.nn_loss_grad(w, x0, tgt)
    rng = np.random.default_rng(11)
    idx = []
    for (wo, bo), co in zip(learned.layer_offsets(), learned.COUT):
        idx += list(rng.integers(wo, bo, size=6)) + list(range(bo, bo + min(co, 3)))
    h = 1e-5
    floor = 1e-4 * np.abs(g).max()   # central-difference round-off ~1e-11 absolute
    worst = 0.0
    for i in idx:
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (O.nn_loss_grad(wp, x0, tgt)[0] - O.nn_loss_grad(wm, x0, tgt)[0]) / (2 * h)
        worst = max(worst, abs(fd - g[i]) / max(floor, abs(g[i])))
    assert worst < 1e-5, worst
    assert loss > 0


def test_oracle_energy_loss_gradient_matches_finite_differences():
    x0, tgt = rand_case(1, 8, 8, 8, seed=3)
    x0[..., 1:] = np.abs(x0[..., 1:])          # coefficient channels are non-negative in use
    w = params(6)
    loss, g = O.nn_loss_grad(w, x0, tgt, kind="energy")
    rng = np.random.default_rng(12)
    idx = []
    for (wo, bo), co in zip(learned.layer_offsets(), learned.COUT):
        idx += list(rng.integers(wo, bo, size=5)) + list(range(bo, bo + min(co, 2)))
    h, floor, errs = 1e-5, 1e-4 * np.abs(g).max(), []
    for i in idx:
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (O.nn_loss_grad(wp, x0, tgt, "energy")[0] - O.nn_loss_grad(wm, x0, tgt, "energy")[0]) / (2 * h)
        errs.append(abs(fd - g[i]) / max(floor, abs(g[i])))
    errs = np.array(errs)
    # a perturbation that moves a ReLU pre-activation across zero breaks the difference quotient
    # itself; allow one such parameter
    assert (errs < 1e-5).sum() >= len(errs) - 1 and errs.max() < 1e-2, errs
    assert loss > 0


def test_oracle_input_gradient_path_reaches_every_layer():
    # every layer's weight gradient is non-zero on a generic case (no dead layer)
    x0, tgt = rand_case(1, 8, 8, 8, seed=4)
    _, g = O.nn_loss_grad(params(9), x0, tgt)
    for wo, bo in learned.layer_offsets():
        assert np.abs(g[wo:bo]).max() > 0


def test_oracle_adam_first_step_is_signed_lr():
    n = 64
    rng = np.random.default_rng(0)
    w = rng.standard_normal(n)
    g = rng.standard_normal(n)
    m, v = np.zeros(n), np.zeros(n)
    w0 = w.copy()
    O.nn_adam(w, g, m, v, 1e-3, 1)
    # bias-corrected first step: m̂ = g, v̂ = g², Δw = -lr g / (|g| + ε)
    assert np.allclose(w0 - w, 1e-3 * g / (np.abs(g) + 1e-8), rtol=1e-12, atol=0)


def test_init_params_deterministic():
    a, b = learned.init_params(4), learned.init_params(4)
    assert a.dtype == np.float32 and np.array_equal(a, b)
    assert not np.array_equal(a, learned.init_params(5))


def test_bubble_layout_is_seeded_and_non_overlapping():
    for seed in range(1000, 1010):
        bl = learned.bubble_layout(seed, 128)
        assert 1 <= len(bl) <= 8
        assert bl == learned.bubble_layout(seed, 128)
        for i, (c, r) in enumerate(bl):
            assert 0.05 * 128 <= r <= 0.15 * 128
            assert all(r <= ci <= 128 - r for ci in c)
            for c2, r2 in bl[i + 1:]:
                assert np.linalg.norm(np.subtract(c, c2)) > r + r2


def test_learned_mode_config_validation(lib):
    from intfadv import _lib, core
    h = C.c_void_p()
    cfg = core.make_config((8, 8), poisson="learned")
    assert lib.ia_create(C.byref(cfg), C.byref(h)) == _lib.IA_ERR_UNSUPPORTED        # 3D only
    cfg = core.make_config((8, 8, 10), poisson="learned")
    assert lib.ia_create(C.byref(cfg), C.byref(h)) == _lib.IA_ERR_UNSUPPORTED        # multiples of 4
    cfg = core.make_config((8, 8, 8))
    cfg.poisson_mode = 3
    assert lib.ia_create(C.byref(cfg), C.byref(h)) == _lib.IA_ERR_INVALID
    assert lib.ia_poisson_precond(None, 0, 30, 1e-4) == _lib.IA_ERR_INVALID
    assert lib.ia_nn_forward(None, None, None, 1, 8, 8, 8, 0) == _lib.IA_ERR_INVALID
