"""GPU checks of the FP32 V-cycle smoothers.

The blocked smoother (all half-sweeps of a smoothing in one z-wavefront launch,
with the widened tile recomputed in shared memory) does the half-sweep kernels'
arithmetic in their order, so a mixed-precision solve must take the same
iterations and land on the same pressure whichever smoother runs, on periodic
and wall dimensions, on sizes that are not multiples of the 32 x 16 tile and
on every level of the hierarchy (relaxation factor 1, where both apply).
Over-relaxed half-sweeps (the default factor) must reach the same pressure in no
more iterations.  These comparisons run on the FP32 face coefficients; the FP16
copy of the finest level's coefficients is checked on its own at the end.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import intfadv as ia
from intfadv import _lib, learned
from intfadv.fields import fzeros, ptr

pytestmark = pytest.mark.gpu


def system(dims, perdir):
    """Face coefficients and right-hand side of a bubbly pressure system (after one step)."""
    N = min(dims)
    sim = ia.TwoPhaseSimulation(dims, (0.0, 0.0, 0.0), float(N), perdir=perdir, λρ=1e-3, λμ=1e-2, ν=0.01,
                                η=0.02, g=(0.0, -1e-3, 0.0),
                                InterfaceSDF=learned.bubbles_sdf(learned.bubble_layout(1003, N)),
                                poisson="mixed", poisson_tol=1e-9, poisson_itmx=300)
    ia.sim_step(sim)
    return sim.flow.mu0.clone(), sim.flow.sigma.clone()


def solve(dims, perdir, L, z, smoother, nu=(2, 2), omega=1.0, coef16=False, slab=0):
    # the smoother comparisons run on the FP32 coefficients (the blocked smoother has no FP16 form)
    # and whole-level half-sweeps (slab 0) unless asked
    h = ia.Handle(ia.make_config(dims, perdir=perdir, poisson="mixed", lrho=1e-3))
    ia.set_poisson_coef16(h, coef16)
    ia.set_poisson_slab_rows(h, slab)
    ia.set_smoother(h, smoother, omega)
    _lib.check(h.call("ia_poisson_mg_params", nu[0], nu[1], 16), "ia_poisson_mg_params")
    x = fzeros(z.shape)
    it, res = C.c_int32(), C.c_double()
    _lib.check(h.call("ia_poisson_solve", ptr(x), ptr(z), ptr(L), 1e-8, 2000, C.byref(it), C.byref(res)),
               "ia_poisson_solve")
    return x, it.value, res.value, ia.poisson_stats(h)


@pytest.mark.parametrize("dims,perdir", [((32, 32, 32), (0, 2)), ((40, 24, 36), ()), ((48, 40, 24), (0, 1, 2))])
@pytest.mark.parametrize("nu", [(2, 2), (1, 1), (1, 2)])
def test_blocked_smoother_matches_halfsweeps(cuda, dims, perdir, nu):
    L, z = system(dims, perdir)
    xa, ita, resa, sta = solve(dims, perdir, L, z, "halfsweep", nu)
    xb, itb, resb, stb = solve(dims, perdir, L, z, "blocked", nu)
    assert resa <= 1e-8 and resb <= 1e-8
    # same sums, but FP32 contraction (fma) choices differ between the kernels: on the singular
    # all-periodic system the FCG count moves by up to two iterations with last-bit differences
    assert abs(ita - itb) <= max(2, ita // 10), (ita, itb)
    assert sta["vcycles"] > 0 and stb["vcycles"] > 0
    xi = lambda x: x[1:-1, 1:-1, 1:-1] - x[1:-1, 1:-1, 1:-1].mean()
    e = float((xi(xa) - xi(xb)).abs().max() / xi(xa).abs().max())
    assert e < 1e-6, e


def test_blocked_smoother_is_deterministic(cuda):
    dims, perdir = (32, 32, 32), (0, 2)
    L, z = system(dims, perdir)
    x1, it1, _, _ = solve(dims, perdir, L, z, "blocked")
    x2, it2, _, _ = solve(dims, perdir, L, z, "blocked")
    assert it1 == it2 and torch.equal(x1, x2)


@pytest.mark.parametrize("dims,perdir", [((32, 32, 32), (0, 2)), ((40, 24, 36), ())])
def test_over_relaxed_smoother_converges_to_the_same_pressure(cuda, dims, perdir):
    L, z = system(dims, perdir)
    xa, ita, resa, _ = solve(dims, perdir, L, z, "halfsweep", omega=1.0)
    xb, itb, resb, _ = solve(dims, perdir, L, z, "halfsweep", omega=1.15)
    assert resa <= 1e-8 and resb <= 1e-8
    assert itb <= ita, (ita, itb)
    xi = lambda x: x[1:-1, 1:-1, 1:-1] - x[1:-1, 1:-1, 1:-1].mean()
    e = float((xi(xa) - xi(xb)).abs().max() / xi(xa).abs().max())
    assert e < 1e-6, e


def test_smoother_switch_rejects_unknown_kind(cuda):
    h = ia.Handle(ia.make_config((16, 16, 16), poisson="mixed"))
    assert h.call("ia_poisson_smoother", 7) == _lib.IA_ERR_INVALID
    assert h.call("ia_poisson_mg_relax", 2.5) == _lib.IA_ERR_INVALID


def test_fp16_smoother_coefficients_give_the_same_step(cuda):
    # the finest-level smoother of the mixed V-cycle on an FP16 copy of the face coefficients
    # (ia_poisson_coef16, the default) against the FP32 coefficients: the V-cycle is only the inner
    # preconditioner, so both solves stop on the same FP64 true residual and the steps agree to the
    # solver tolerance.  The FP16 copy costs no convergence: the iteration totals agree to 10 % (a
    # count of a 1e-12 solve moves by a few under any rounding-level change of the FP32 smoother)
    import torch
    import intfadv as ia
    from intfadv import workloads
    N = 24
    p = workloads.bubble_params(N)
    c, r = (11.7, 24.3, 12.2), p["radius"]

    def mk(on):
        sdf = lambda x: r - torch.sqrt((x[0] - c[0]) ** 2 + (x[1] - c[1]) ** 2 + (x[2] - c[2]) ** 2)
        sim = ia.TwoPhaseSimulation(p["dims"], (0.0, 0.0, 0.0), float(N), perdir=p["perdir"], λρ=p["lrho"],
                                    λμ=p["lmu"], ν=p["mu"], η=p["sigma"], g=(0.0, -p["G"], 0.0), InterfaceSDF=sdf,
                                    poisson="mixed", poisson_tol=1e-12, poisson_itmx=500)
        ia.set_poisson_coef16(sim.handle, on)
        return sim

    a, b = mk(True), mk(False)
    ia_, ib = [], []
    for _ in range(3):
        sa, sb = ia.sim_step(a), ia.sim_step(b)
        assert max(sa.poisson_resid) <= 1e-12 and max(sb.poisson_resid) <= 1e-12
        ia_.append(sum(sa.poisson_iters))
        ib.append(sum(sb.poisson_iters))
    du = float((a.flow.u - b.flow.u).abs().max()) / float(a.flow.u.abs().max())
    assert du < 1e-10, du
    assert abs(sum(ia_) - sum(ib)) <= 0.1 * sum(ib), (ia_, ib)
    assert all(abs(x - y) <= 4 for x, y in zip(ia_, ib)), (ia_, ib)


@pytest.mark.parametrize("nu", [(2, 2), (1, 1), (1, 2), (3, 2)])
@pytest.mark.parametrize("slab,coef16", [(8, True), (11, False), (16, True)])
def test_slab_wavefront_is_bit_identical(cuda, nu, slab, coef16):
    # the finest level's half-sweeps and restriction run slab by slab over y, each stage one row behind
    # the previous (ia_poisson_slab_rows): the same updates as whole-level half-sweeps, so the same
    # pressure bit for bit and the same iteration count; 46 interior rows leave a short last slab
    dims, perdir = (40, 46, 24), (0, 2)
    L, z = system(dims, perdir)
    xa, ita, resa, _ = solve(dims, perdir, L, z, "halfsweep", nu, omega=1.15, coef16=coef16, slab=0)
    xb, itb, resb, _ = solve(dims, perdir, L, z, "halfsweep", nu, omega=1.15, coef16=coef16, slab=slab)
    assert resa <= 1e-8 and ita == itb and resa == resb
    assert torch.equal(xa, xb)


@pytest.mark.parametrize("nu", [(2, 2), (1, 2)])
def test_slab_wavefront_is_bit_identical_unrelaxed(cuda, nu):
    # relaxation factor 1: the post-smoothing's first red half-sweep is a plain one and the first
    # half-sweep writes the red values only for nu1 = 1
    dims, perdir = (40, 46, 24), (0, 2)
    L, z = system(dims, perdir)
    xa, ita, resa, _ = solve(dims, perdir, L, z, "halfsweep", nu, omega=1.0, coef16=True, slab=0)
    xb, itb, resb, _ = solve(dims, perdir, L, z, "halfsweep", nu, omega=1.0, coef16=True, slab=8)
    assert resa <= 1e-8 and ita == itb and resa == resb
    assert torch.equal(xa, xb)


def test_slab_wavefront_skips_periodic_y(cuda):
    # with y periodic the wavefront would read rows across the wrap before they are final: the setting
    # is accepted and the half-sweeps run whole-level
    dims, perdir = (32, 32, 32), (0, 1, 2)
    L, z = system(dims, perdir)
    xa, ita, _, _ = solve(dims, perdir, L, z, "halfsweep", omega=1.15, slab=0)
    xb, itb, _, _ = solve(dims, perdir, L, z, "halfsweep", omega=1.15, slab=8)
    assert ita == itb and torch.equal(xa, xb)


def test_slab_rows_rejects_small_slabs(cuda):
    h = ia.Handle(ia.make_config((16, 16, 16), poisson="mixed"))
    assert h.call("ia_poisson_slab_rows", 4) == _lib.IA_ERR_INVALID
    assert h.call("ia_poisson_slab_rows", -1) == _lib.IA_ERR_INVALID
    assert h.call("ia_poisson_slab_rows", 0) == _lib.IA_OK


def test_finest_level_smoothing_override(cuda):
    # ia_poisson_mg_fine: other pre/post counts on the finest level only; the solve still converges to
    # the same pressure (to the solver tolerance), with its own iteration count
    dims, perdir = (40, 48, 24), (0, 2)
    L, z = system(dims, perdir)
    xa, ita, resa, _ = solve(dims, perdir, L, z, "halfsweep", omega=1.15)
    h = ia.Handle(ia.make_config(dims, perdir=perdir, poisson="mixed", lrho=1e-3))
    assert h.call("ia_poisson_mg_fine", -1, 2) == _lib.IA_ERR_INVALID
    _lib.check(h.call("ia_poisson_mg_fine", 1, 2), "ia_poisson_mg_fine")
    x = fzeros(z.shape)
    it, res = C.c_int32(), C.c_double()
    _lib.check(h.call("ia_poisson_solve", ptr(x), ptr(z), ptr(L), 1e-8, 2000, C.byref(it), C.byref(res)),
               "ia_poisson_solve")
    assert resa <= 1e-8 and res.value <= 1e-8
    xi = lambda v: v[1:-1, 1:-1, 1:-1] - v[1:-1, 1:-1, 1:-1].mean()
    e = float((xi(xa) - xi(x)).abs().max() / xi(xa).abs().max())
    assert e < 1e-5, e
