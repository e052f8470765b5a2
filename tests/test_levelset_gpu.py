"""GPU level-set reinitialisation (src/redistaning.jl) against the oracle and the reference's checks."""
import numpy as np
import pytest
import torch

import intfadv as ia
from intfadv.fields import ffrom, fzeros
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def npf(t):
    return np.asfortranarray(t.detach().cpu().numpy())


@pytest.mark.parametrize("dims,per", [((14, 11), ()), ((14, 11), (0,)), ((10, 9, 8), (0, 2)), ((10, 9, 8), ())])
def test_rhs_matches_oracle(cuda, dims, per):
    rng = np.random.default_rng(len(dims) + len(per))
    ng = tuple(n + 2 for n in dims)
    phi = np.asfortranarray(rng.standard_normal(ng))
    ini = np.asfortranarray(rng.standard_normal(ng))
    h = ia.Handle(ia.make_config(dims, perdir=per))
    L = fzeros(ng)
    ia.computeL(h, L, ffrom(phi), ffrom(ini))
    ref = O.levelset_rhs(phi, ini, per=per)
    assert np.abs(npf(L) - ref).max() < 1e-12 * max(1.0, np.abs(ref).max())


def test_planar_interface_matches_reference_checks_and_oracle(cuda):
    # maintests.jl:305-317 on the GPU path
    sim = ia.TwoPhaseSimulation((16, 16), (0.0, 0.0), 16.0, InterfaceSDF=lambda x: x[0] - 8, perdir=(1,))
    f0 = npf(sim.intf.f)
    ls = ia.LevelSet(sim)
    assert ls.ϕ.data_ptr() == sim.intf.f0.data_ptr()
    assert np.array_equal(npf(ls.ϕ), 2 * f0 - 1)
    ia.redistaning(ls, d=4.0, dτ=0.05)
    phi = npf(ls.ϕ)
    assert np.isfinite(phi).all()
    assert np.all(np.diff(phi[1:-1, 8]) <= 0)
    assert np.array_equal(phi[:, 0], phi[:, -2]) and np.array_equal(phi[:, -1], phi[:, 1])
    for ix in range(8, 12):
        assert abs(phi[ix - 1, 8] + (ix - 1.5 - 8)) <= 0.01
    ref = O.redistance(f0, d=4.0, dtau=0.05, per=(1,))
    assert np.abs(phi - ref).max() < 1e-10


def test_sphere_3d_matches_oracle(cuda):
    N = 20
    sdf = lambda x: torch.sqrt((x[0] - 9.3) ** 2 + (x[1] - 10.1) ** 2 + (x[2] - 9.7) ** 2) - 5.2
    sim = ia.TwoPhaseSimulation((N, N, N), (0.0, 0.0, 0.0), float(N), InterfaceSDF=sdf, perdir=(0,))
    f0 = npf(sim.intf.f)
    ls = ia.LevelSet(sim)
    ia.redistaning(ls, d=2.0, dτ=0.25)
    ref = O.redistance(f0, d=2.0, dtau=0.25, per=(0,))
    assert np.abs(npf(ls.ϕ) - ref).max() < 1e-10
