"""The configurations at their full sizes: the CPU-runnable 2D dam break against the oracle, and the
3D workloads through size-independent properties (mass conservation, bounded fractions, finite
fields, converged pressure)."""
import math

import numpy as np
import pytest
import torch

import intfadv as ia
from intfadv import learned
from oracle.sim import OracleSim

pytestmark = pytest.mark.gpu
PTOL = 1e-12


def npf(t):
    return np.asfortranarray(t.detach().cpu().numpy())


def test_c1_dam_break_128x64_matches_oracle(cuda):
    # 128x64, walls everywhere, water column x < 0.25 Lx, y < 0.5 Ly; L = 64 cells, U = 1 so
    # g = U²/L = 1/64 in grid units, ν = U L / Re with Re = 1000; λρ = 1e-3, λμ = 1/55
    Nx, Ny = 128, 64
    a, b = 0.25 * Nx, 0.5 * Ny
    g = (0.0, -1.0 / 64)
    nu = 64 / 1000
    sim = ia.TwoPhaseSimulation((Nx, Ny), (0.0, 0.0), float(Ny), InterfaceSDF=lambda x: torch.maximum(x[0] - a, x[1] - b),
                                λμ=1 / 55, λρ=1e-3, ν=nu, g=g, poisson="mixed", poisson_tol=PTOL, poisson_itmx=1000)
    orc = OracleSim((Nx, Ny), (0.0, 0.0), sdf=lambda x: np.maximum(x[0] - a, x[1] - b), lrho=1e-3, lmu=1 / 55, ν=nu,
                    g=g, ptol=PTOL, pitmx=200000)
    m0 = sim.intf.mass()
    for _ in range(30):
        st = ia.sim_step(sim)
        orc.step()
        assert st.poisson_resid[1] <= PTOL
    ef = float(np.abs(npf(sim.intf.f) - orc.f).max())
    eu = float(np.abs(npf(sim.flow.u) - orc.u).max()) / float(np.abs(orc.u).max())
    assert ef < 1e-9 and eu < 1e-9, (ef, eu)
    assert abs(sim.intf.mass() - m0) <= 1e-12 * m0


def bubbly(dims, bubbles, G, Eo, perdir=(0, 2), poisson="mixed"):
    D = 0.25 * dims[0] if bubbles is None else 2 * max(r for _, r in bubbles)
    sigma = G * D * D / Eo
    mu = (1e-3 * sigma ** 3 / G) ** 0.25
    return ia.TwoPhaseSimulation(dims, (0.0, 0.0, 0.0), float(dims[0]), perdir=perdir, λρ=1e-3, λμ=1e-2, ν=mu,
                                 η=sigma, g=(0.0, -G, 0.0), InterfaceSDF=learned.bubbles_sdf(bubbles),
                                 poisson=poisson, poisson_tol=1e-8, poisson_itmx=400)


def check_properties(sim, steps, mass_tol):
    m0 = sim.intf.mass()
    for _ in range(steps):
        st = ia.sim_step(sim)
        assert st.code == 0 and st.poisson_resid[1] <= 1e-8
    f = sim.intf.f
    assert bool(torch.isfinite(f).all()) and bool(torch.isfinite(sim.flow.u).all())
    assert float(f.min()) >= 0.0 and float(f.max()) <= 1.0
    drift = abs(sim.intf.mass() - m0) / m0
    assert drift <= mass_tol, drift
    return drift


def test_c3_rising_bubble_256x512x256_properties(cuda):
    N = 256
    sim = bubbly((N, 2 * N, N), [((N / 2, N / 2, N / 2), 0.125 * N)], G=1e-3, Eo=10.0)
    check_properties(sim, 2, 1e-12)


def swarm_layout(seed=5, n=64, rmin=0.02, rmax=0.05, N=512, max_tries=200000):
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(max_tries):
        if len(out) == n:
            break
        r = rng.uniform(rmin, rmax)
        c = rng.uniform(r + 0.01, 1 - r - 0.01, size=3)
        if all(np.linalg.norm(c - c2) > r + r2 + 0.01 for c2, r2 in out):
            out.append((c, r))
    assert len(out) == n
    return [(tuple(float(v) * N for v in c), float(r) * N) for c, r in out]


def test_c5_swarm_512_properties(cuda):
    # 512³ unit cube, 64 non-overlapping bubbles r ∈ U[0.02, 0.05] (seed 5), Eö = 5
    N = 512
    sim = bubbly((N, N, N), swarm_layout(N=N), G=1e-3, Eo=5.0)
    check_properties(sim, 2, 1e-12)
