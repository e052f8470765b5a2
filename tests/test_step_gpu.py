"""GPU parity of the full two-phase step (MPFMomStep!) against the CPU oracle.

Both sides solve the pressure to an L∞ residual of 1e-12 (the reference's own
Poisson result is pinned only by its residual), so fractions and velocities are
compared to 1e-10 (f absolute; u relative to max|u|) and pressure up to its
free constant.
"""
import math

import numpy as np
import pytest
import torch

import intfadv as ia
from intfadv import _lib
from oracle.sim import OracleSim

pytestmark = pytest.mark.gpu
PTOL = 1e-12


def npf(t):
    return np.asfortranarray(t.detach().cpu().numpy())


def inner(a, D):
    return a[tuple(slice(1, -1) for _ in range(D))]


def compare(sim, orc, D, tol_u=1e-10, tol_f=1e-10):
    f_g, f_o = npf(sim.intf.f), orc.f
    u_g, u_o = npf(sim.flow.u), orc.u
    ef = float(np.abs(f_g - f_o).max())
    scale = max(1e-30, float(np.abs(u_o).max()))
    eu = float(np.abs(u_g - u_o).max()) / scale
    pg, po = inner(npf(sim.flow.p), D), inner(orc.p, D)
    pg, po = pg - pg.mean(), po - po.mean()
    ep = float(np.abs(pg - po).max()) / max(1e-30, float(np.abs(po).max()))
    return ef, eu, ep


# ------------------------------------------------------------------- reference integration tests
def test_quiescent_droplet_is_exact_noop(cuda):
    # test/maintests.jl:197-202, test/helper.jl:17-18
    N = 8
    sdf_t = lambda x: torch.sqrt((x[0] - N / 2) ** 2 + (x[1] - N / 2) ** 2) - N / 4
    sim = ia.TwoPhaseSimulation((N, N), (0.0, 0.0), float(N), InterfaceSDF=sdf_t, perdir=(0, 1))
    f0 = sim.intf.f.clone()
    ia.sim_step(sim)
    assert bool((sim.flow.u == 0).all())
    assert torch.equal(sim.intf.f, f0)
    assert bool(torch.isfinite(sim.flow.p).all())


def tgv_pair(N=16, poisson="fp64"):
    k = 2 * math.pi / N
    R = N / 4

    def u0_t(i, x):
        return -torch.sin(x[0] * k) * torch.cos(x[1] * k) if i == 0 else torch.cos(x[0] * k) * torch.sin(x[1] * k)

    def u0_n(i, x):
        return -np.sin(x[0] * k) * np.cos(x[1] * k) if i == 0 else np.cos(x[0] * k) * np.sin(x[1] * k)

    sdf_t = lambda x: torch.sqrt((x[0] - N / 2) ** 2 + (x[1] - N / 2) ** 2) - R
    sdf_n = lambda x: np.sqrt((x[0] - N / 2) ** 2 + (x[1] - N / 2) ** 2) - R
    sim = ia.TwoPhaseSimulation((N, N), (0.0, 0.0), float(N), λμ=0.1, λρ=0.1, InterfaceSDF=sdf_t, u0=u0_t,
                                perdir=(0, 1), poisson=poisson, poisson_tol=PTOL, poisson_itmx=500)
    orc = OracleSim((N, N), (0.0, 0.0), sdf=sdf_n, u0=u0_n, perdir=(0, 1), lrho=0.1, lmu=0.1, ptol=PTOL)
    return sim, orc


def test_tgv_droplet_conserves_mass_and_matches_oracle(cuda):
    # test/maintests.jl:206-215, test/helper.jl:6-13
    sim, orc = tgv_pair()
    assert abs(sim.flow.Δt[-1] - orc.Δt[-1]) < 1e-14
    ia.sim_step(sim)
    orc.step()
    V0 = sim.intf.mass()
    for _ in range(3):
        st = ia.sim_step(sim)
        orc.step()
        assert st.poisson_resid[1] <= PTOL
    assert bool(torch.isfinite(sim.flow.u).all()) and bool(torch.isfinite(sim.intf.f).all())
    assert abs(sim.intf.mass() - V0) <= 1e-4 * V0
    ef, eu, ep = compare(sim, orc, 2)
    assert ef < 1e-10 and eu < 1e-10 and ep < 1e-6, (ef, eu, ep)
    assert abs(sim.flow.Δt[-1] - orc.Δt[-1]) < 1e-12 * orc.Δt[-1]


def dam_pair(Nx=32, Ny=16, poisson="fp64", steps=0):
    a, b = 0.25 * Nx, 0.5 * Ny
    sdf_t = lambda x: torch.maximum(x[0] - a, x[1] - b)
    sdf_n = lambda x: np.maximum(x[0] - a, x[1] - b)
    kw = dict(λμ=1 / 55, λρ=1e-3, ν=0.02, g=(0.0, -0.01))
    sim = ia.TwoPhaseSimulation((Nx, Ny), (0.0, 0.0), float(Ny), InterfaceSDF=sdf_t, poisson=poisson,
                                poisson_tol=PTOL, poisson_itmx=500, **kw)
    orc = OracleSim((Nx, Ny), (0.0, 0.0), sdf=sdf_n, lrho=1e-3, lmu=1 / 55, ν=0.02, g=(0.0, -0.01), ptol=PTOL,
                    pitmx=20000)
    return sim, orc


@pytest.mark.parametrize("poisson", ["fp64", "mixed"])
def test_dam_break_walls_gravity_viscosity_matches_oracle(cuda, poisson):
    sim, orc = dam_pair(poisson=poisson)
    for s in range(4):
        st = ia.sim_step(sim)
        orc.step()
        assert st.poisson_resid[0] <= PTOL and st.poisson_resid[1] <= PTOL
    ef, eu, ep = compare(sim, orc, 2)
    assert ef < 1e-10 and eu < 1e-10 and ep < 1e-6, (ef, eu, ep)


def bubble_pair(N=12, poisson="fp64", eta=0.05, nu=0.01):
    # rising-bubble shape: periodic x/z, walls in y, light bubble in heavy fluid
    dims = (N, 2 * N, N)
    c = (N / 2, N / 2 + 2, N / 2)
    r = 0.25 * N
    sdf_t = lambda x: r - torch.sqrt((x[0] - c[0]) ** 2 + (x[1] - c[1]) ** 2 + (x[2] - c[2]) ** 2)
    sdf_n = lambda x: r - np.sqrt((x[0] - c[0]) ** 2 + (x[1] - c[1]) ** 2 + (x[2] - c[2]) ** 2)
    kw = dict(λμ=1e-2, λρ=1e-3, ν=nu, g=(0.0, -0.02, 0.0), η=eta)
    sim = ia.TwoPhaseSimulation(dims, (0.0, 0.0, 0.0), float(N), perdir=(0, 2), InterfaceSDF=sdf_t,
                                poisson=poisson, poisson_tol=PTOL, poisson_itmx=500, **kw)
    orc = OracleSim(dims, (0.0, 0.0, 0.0), sdf=sdf_n, perdir=(0, 2), lrho=1e-3, lmu=1e-2, ν=nu,
                    g=(0.0, -0.02, 0.0), eta=eta, ptol=PTOL, pitmx=50000)
    return sim, orc


@pytest.mark.parametrize("poisson", ["fp64", "mixed"])
def test_rising_bubble_3d_matches_oracle(cuda, poisson):
    sim, orc = bubble_pair(poisson=poisson)
    assert abs(sim.flow.Δt[-1] - orc.Δt[-1]) < 1e-14
    for s in range(3):
        st = ia.sim_step(sim)
        orc.step()
        assert st.poisson_resid[1] <= PTOL
    ef, eu, ep = compare(sim, orc, 3)
    assert ef < 1e-10 and eu < 1e-10 and ep < 1e-6, (ef, eu, ep)
    ru_g, ru_o = inner(npf(sim.intf.rhou), 3), inner(orc.rhou, 3)
    # ρu interior (the Dirichlet wall faces y=1 are overwritten by BC! in the reference only)
    ru_g, ru_o = ru_g[:, 1:, :, :], ru_o[:, 1:, :, :]
    assert np.abs(ru_g - ru_o).max() < 1e-9 * max(1.0, np.abs(ru_o).max())


def test_mixed_poisson_agrees_with_fp64(cuda):
    a, _ = bubble_pair(poisson="fp64")
    b, _ = bubble_pair(poisson="mixed")
    for _ in range(2):
        ia.sim_step(a)
        ia.sim_step(b)
    du = float((a.flow.u - b.flow.u).abs().max()) / float(a.flow.u.abs().max())
    assert du < 1e-9
    assert b.last_status.poisson_iters[1] >= a.last_status.poisson_iters[1] - 1


def test_wide_offset_variants_give_the_same_steps(cuda):
    # the momentum and viscous flux bulk passes run with 32-bit cell offsets on grids this size; their
    # 64-bit variants (grids past 2^31 vector entries) forced with ia_wide_offsets give the same steps
    a, _ = bubble_pair(poisson="mixed")
    b, _ = bubble_pair(poisson="mixed")
    assert b.handle.call("ia_wide_offsets", 2) == _lib.IA_ERR_INVALID
    _lib.check(b.handle.call("ia_wide_offsets", 1), "ia_wide_offsets")
    for _ in range(3):
        ia.sim_step(a)
        ia.sim_step(b)
    assert torch.equal(a.flow.u, b.flow.u) and torch.equal(a.intf.f, b.intf.f) and torch.equal(a.flow.p, b.flow.p)


def test_mpcfl_matches_oracle(cuda):
    sim, orc = bubble_pair()
    ia.sim_step(sim)
    orc.step()
    assert abs(ia.MPCFL(sim) - orc.mpcfl()) < 1e-12 * orc.mpcfl()


@pytest.mark.parametrize("arith", ["fp64", "ff"])
@pytest.mark.parametrize("limiter", ["Koren", "upwind", "minmod", "vanAlbada1", "Sweby", "superbee", "TVDcen",
                                     "TVDdown"])
def test_every_limiter_matches_oracle(cuda, limiter, arith):
    # the λ(u,c,d) keyword of TwoPhaseSimulation (src/flow.jl:5-15), on a sheared 2D droplet, with the
    # momentum kernels in FP64 and in FP32 pairs
    N = 24
    k = 2 * math.pi / N
    u0_t = lambda i, x: 0.3 * torch.sin(x[1] * k) if i == 0 else 0.2 * torch.cos(x[0] * k)
    u0_n = lambda i, x: 0.3 * np.sin(x[1] * k) if i == 0 else 0.2 * np.cos(x[0] * k)
    sdf_t = lambda x: torch.sqrt((x[0] - 10) ** 2 + (x[1] - 12) ** 2) - 5
    sdf_n = lambda x: np.sqrt((x[0] - 10) ** 2 + (x[1] - 12) ** 2) - 5
    sim = ia.TwoPhaseSimulation((N, N), (0.0, 0.0), float(N), λρ=0.05, λμ=0.1, ν=0.01, InterfaceSDF=sdf_t, u0=u0_t,
                                perdir=(0, 1), λ=limiter, poisson_tol=PTOL, poisson_itmx=500, momentum_arith=arith)
    orc = OracleSim((N, N), (0.0, 0.0), sdf=sdf_n, u0=u0_n, perdir=(0, 1), lrho=0.05, lmu=0.1, ν=0.01,
                    limiter=limiter, ptol=PTOL)
    for _ in range(3):
        ia.sim_step(sim)
        orc.step()
    ef, eu, ep = compare(sim, orc, 2)
    assert ef < 1e-10 and eu < 1e-10 and ep < 1e-6, (limiter, ef, eu, ep)


@pytest.mark.parametrize("dims,per,eta,uBC", [((16, 12), (), 0.0, None), ((12, 10, 8), (0, 2), 0.05, None),
                                              ((16, 12), (1,), 0.0, (0.05, 0.0)),
                                              ((12, 10, 8), (2,), 0.0, (0.04, -0.03, 0.0))])
def test_float_float_momentum_agrees_with_fp64(cuda, dims, per, eta, uBC):
    # the same step with the momentum kernels in FP32 pairs and in FP64 (both with the FP64 solver):
    # the pair arithmetic carries ~2^-46 relative error per operation.  A wall-normal uBC puts the
    # Dirichlet value on the low wall face, which the fused uStar passes write
    D = len(dims)
    uBC = uBC or (0.0,) * D
    c = tuple(0.5 * n + 0.7 for n in dims)
    sdf = lambda x: torch.sqrt(sum((x[d] - c[d]) ** 2 for d in range(D))) - 0.3 * dims[0]
    g = (0.0, -0.01) + ((0.0,) if D == 3 else ())
    mk = lambda arith: ia.TwoPhaseSimulation(dims, uBC, float(dims[0]), perdir=per, InterfaceSDF=sdf, λρ=1e-3,
                                             λμ=1e-2, ν=0.02, g=g, η=(eta or None), poisson="fp64", poisson_tol=PTOL,
                                             poisson_itmx=500, momentum_arith=arith)
    a, b = mk("fp64"), mk("ff")
    for _ in range(3):
        ia.sim_step(a)
        ia.sim_step(b)
    du = float((a.flow.u - b.flow.u).abs().max()) / float(a.flow.u.abs().max())
    df = float((a.intf.f - b.intf.f).abs().max())
    assert du < 1e-11 and df < 1e-11, (du, df)
    assert du > 0.0, "the two arithmetics must differ at the rounding level (is the pair path running?)"


@pytest.mark.parametrize("dims,per", [((10, 7), ()), ((10, 7), (0, 1)), ((10, 7), (1,)), ((8, 6, 5), (0, 2)),
                                      ((8, 6, 5), ())])
def test_velocity_bc_matches_oracle(cuda, dims, per):
    # WaterLily BC!(a, u_BC, false, perdir) on a random vector field, the C-ABI ia_bc_velocity
    import ctypes as C
    from oracle import pyoracle as O
    rng = np.random.default_rng(len(dims) * 7 + len(per))
    D = len(dims)
    ng = tuple(n + 2 for n in dims)
    a = np.asfortranarray(rng.standard_normal(ng + (D,)))
    uBC = (0.3, -0.2, 0.1)[:D]
    h = ia.Handle(ia.make_config(dims, perdir=per, uBC=uBC))
    ga = ia.ffrom(a)
    _lib.check(h.call("ia_bc_velocity", ia.fields.ptr(ga)), "ia_bc_velocity")
    ref = a.copy(order="F")
    A = np.zeros(3)
    A[:D] = uBC
    O.lib().orc_bc_vel(C.byref(O.grid(ng, per)), O.ptr(ref), A.ctypes.data)
    assert np.array_equal(npf(ga), ref)
