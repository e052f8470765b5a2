"""GPU parity of surface tension (surfTen!, src/surfaceTension.jl:8-102) against the oracle.

* ia_surften alone (2D and 3D; walled and periodic; droplets that reach the high walls, so that
  height columns and WY stencils read the buffer positions BCf!(d, ·) never writes; a non-zero
  prior buffer content, which the reference reads at the high x ghost).
* the full step with η > 0 in 2D (the 2D curvature, surfaceTension.jl:50-59) and 3D, droplets
  touching the high walls, 1e-10 on f (absolute) and u (relative to max|u|).
"""
import ctypes as C

import numpy as np
import pytest
import torch

import intfadv as ia
from intfadv import _lib
from oracle import pyoracle as O
from oracle.sim import OracleSim, sdf_samples

pytestmark = pytest.mark.gpu
PTOL = 1e-12


def npf(t):
    return np.asfortranarray(t.detach().cpu().numpy())


def droplet_fraction(dims, per, centre, r):
    """Oracle applyVOF! of a droplet (dark inside) on a ghost-padded grid, BCf! ghosts."""
    ng = tuple(n + 2 for n in dims)
    sdf = lambda x: np.sqrt(sum((x[d] - centre[d]) ** 2 for d in range(len(dims)))) - r
    f = O.zeros(ng)
    f[...] = 1.0
    al, nh = O.zeros(ng), O.zeros(ng + (len(dims),))
    samples = sdf_samples(ng, sdf)
    arr = (C.c_void_p * len(samples))(*[s.ctypes.data for s in samples])
    g = O.grid(ng, per)
    O.lib().orc_apply_vof(C.byref(g), O.ptr(f), O.ptr(al), O.ptr(nh), arr)
    O.lib().orc_bcf(C.byref(g), O.ptr(f))
    return f


CASES = [((24, 20), (), (18.5, 17.0), 5.3), ((24, 20), (0, 1), (18.5, 17.0), 5.3), ((24, 20), (0,), (6.0, 17.5), 5.1),
         ((14, 12, 10), (), (10.5, 9.5, 5.2), 3.9), ((14, 12, 10), (0, 2), (10.5, 9.5, 5.2), 3.9),
         ((12, 14, 12), (1,), (9.4, 7.0, 9.1), 3.6)]


@pytest.mark.parametrize("dims,per,centre,r", CASES)
def test_surften_matches_oracle(cuda, dims, per, centre, r):
    D = len(dims)
    ng = tuple(n + 2 for n in dims)
    f = droplet_fraction(dims, per, centre, r)
    rng = np.random.default_rng(D * 10 + len(per))
    forcing = np.asfortranarray(rng.standard_normal(ng + (D,)) * 1e-3)
    fbuf = np.asfortranarray(rng.uniform(0.0, 1.0, ng))     # prior buffer content (read at the high x ghost)
    eta = 0.07
    h = ia.Handle(ia.make_config(dims, perdir=per, eta=eta))
    gF, gf, gb = ia.ffrom(forcing), ia.ffrom(f), ia.ffrom(fbuf)
    _lib.check(h.call("ia_surften", ia.fields.ptr(gF), ia.fields.ptr(gf), ia.fields.ptr(gb), C.c_double(eta)),
               "ia_surften")
    ref = forcing.copy(order="F")
    nh = O.zeros(ng + (D,))
    fbuf_orc = fbuf.copy(order="F")       # the oracle writes its buffer; keep the copy alive across the call
    grid = O.grid(ng, per)
    O.lib().orc_surften(C.byref(grid), O.ptr(ref), O.ptr(f), O.ptr(nh), O.ptr(fbuf_orc), eta)
    got = npf(gF)
    assert np.abs(ref - forcing).max() > 1e-6, "the case must produce a surface-tension force"
    scale = float(np.abs(ref - forcing).max())
    assert np.abs(got - ref).max() <= 1e-12 * scale, (np.abs(got - ref).max(), scale)
    # the buffer is read, not written
    assert np.array_equal(npf(gb), fbuf)


def compare(sim, orc):
    ef = float(np.abs(npf(sim.intf.f) - orc.f).max())
    eu = float(np.abs(npf(sim.flow.u) - orc.u).max()) / max(1e-30, float(np.abs(orc.u).max()))
    return ef, eu


def droplet_pair(dims, per, centre, r, eta, g, poisson):
    sdf_t = lambda x: torch.sqrt(sum((x[d] - centre[d]) ** 2 for d in range(len(dims)))) - r
    sdf_n = lambda x: np.sqrt(sum((x[d] - centre[d]) ** 2 for d in range(len(dims)))) - r
    kw = dict(λμ=0.05, λρ=0.05, ν=0.02, g=g, η=eta)
    uBC = (0.0,) * len(dims)
    sim = ia.TwoPhaseSimulation(dims, uBC, float(dims[0]), perdir=per, InterfaceSDF=sdf_t, poisson=poisson,
                                poisson_tol=PTOL, poisson_itmx=500, **kw)
    orc = OracleSim(dims, uBC, sdf=sdf_n, perdir=per, lrho=0.05, lmu=0.05, ν=0.02, g=g, eta=eta, ptol=PTOL,
                    pitmx=50000)
    return sim, orc


@pytest.mark.parametrize("per", [(), (0, 1)])
@pytest.mark.parametrize("poisson", ["fp64", "mixed"])
def test_surface_tension_2d_step_matches_oracle(cuda, per, poisson):
    # a droplet that reaches the high x and y walls (walled case) or wraps around them (periodic case).
    # Its centre is off every cell centre: at a cell centre that is a critical point of the SDF the
    # reference's finite-difference normal is zero and applyVOF! gives 0/0 (src/VOFutil.jl:19-35).
    sim, orc = droplet_pair((24, 20), per, (18.3, 16.2), 5.2, 0.05, (0.0, -0.005), poisson)
    assert abs(sim.flow.Δt[-1] - orc.Δt[-1]) < 1e-14
    for _ in range(4):
        st = ia.sim_step(sim)
        orc.step()
        assert st.poisson_resid[1] <= PTOL
    ef, eu = compare(sim, orc)
    assert ef < 1e-10 and eu < 1e-10, (ef, eu)


def test_surface_tension_3d_step_touching_walls_matches_oracle(cuda):
    sim, orc = droplet_pair((12, 14, 10), (2,), (8.6, 10.8, 5.0), 3.6, 0.05, (0.0, -0.005, 0.0), "fp64")
    for _ in range(3):
        st = ia.sim_step(sim)
        orc.step()
        assert st.poisson_resid[1] <= PTOL
    ef, eu = compare(sim, orc)
    assert ef < 1e-10 and eu < 1e-10, (ef, eu)
