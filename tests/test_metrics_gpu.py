"""GPU diagnostics (ia_metrics) against the oracle's sums of the src/metrics.jl per-cell functions."""
import numpy as np
import pytest
import torch

import intfadv as ia
from intfadv.fields import ffrom
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims", [(12, 9), (10, 8, 6)])
@pytest.mark.parametrize("with_omega", [False, True])
def test_metrics_match_oracle(cuda, dims, with_omega):
    rng = np.random.default_rng(len(dims) + 3 * with_omega)
    D = len(dims)
    ng = tuple(n + 2 for n in dims)
    u = np.asfortranarray(rng.standard_normal(ng + (D,)))
    f = np.asfortranarray(rng.uniform(0, 1, ng))
    w = np.asfortranarray(rng.standard_normal(ng + ((D,) if D == 3 else ()))) if with_omega else None
    U, g, wl = (0.3, -0.2, 0.1)[:D], (0.0, -1.0, 0.5)[:D], (0.0, 2.5, 1.0)[:D]
    h = ia.Handle(ia.make_config(dims, lrho=0.05))
    got = ia.metrics(h, ffrom(u), ffrom(f), omega=None if w is None else ffrom(w), U=U, g=g, statwl=wl)
    ref = O.metrics(u, f, 0.05, U=U, g=g, statwl=wl, omega=w)
    for k in ("ke", "pe", "ens"):
        assert got[k] == pytest.approx(ref[k], rel=1e-12, abs=1e-12), k
    assert np.allclose(got["rhou"], ref["rhou"], rtol=1e-12, atol=1e-12)


def test_sim_metrics_of_a_resting_droplet_are_potential_only(cuda):
    N = 16
    sdf = lambda x: torch.sqrt((x[0] - N / 2) ** 2 + (x[1] - N / 2) ** 2) - N / 4
    sim = ia.TwoPhaseSimulation((N, N), (0.0, 0.0), float(N), InterfaceSDF=sdf, g=(0.0, -1.0), λρ=0.1)
    m = ia.sim_metrics(sim)
    assert m["ke"] == 0.0 and m["rhou"] == [0.0, 0.0] and m["ens"] == 0.0
    assert m["pe"] > 0.0
