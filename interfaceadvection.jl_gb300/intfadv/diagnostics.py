"""Step diagnostics of src/metrics.jl as GPU domain sums (C-ABI ``ia_metrics``).

The reference defines per-cell functions (ρkeI, ρuI, ρgh, EnsI) that callers sum over the
domain; here one fused pass returns the sums over interior cells.
"""
from __future__ import annotations

import ctypes as C

from . import _lib
from .fields import ptr


def metrics(handle, u, f, omega=None, U=None, g=None, statwl=None) -> dict:
    """Σ ρkeI(I,u,f,λρ,U), Σ ρgh(I,g,f,λρ,StatWL), Σ EnsI(I,ω) (0 without ω) and Σ ρuI(i,I,u,f,λρ,U)
    for each component over interior cells (src/metrics.jl:13-58); λρ is the handle's."""
    D = handle.cfg.D

    def vec(v):
        if v is None:
            return None
        a = (C.c_double * 3)()
        for i in range(D):
            a[i] = float(v[i])
        return a

    out = (C.c_double * 6)()
    rc = handle.call("ia_metrics", ptr(u), ptr(f), ptr(omega) if omega is not None else None, vec(U), vec(g),
                     vec(statwl), out)
    _lib.check(rc, "ia_metrics")
    return {"ke": out[0], "pe": out[1], "ens": out[2], "rhou": [out[3 + i] for i in range(D)]}


def sim_metrics(sim, omega=None, U=None, statwl=None) -> dict:
    """metrics() of a TwoPhaseSimulation's current u and f, with its gravity."""
    g = [float(v) for v in sim.handle.cfg.g][:sim.handle.cfg.D] if sim.handle.cfg.has_g else None
    return metrics(sim.handle, sim.flow.u, sim.intf.f, omega=omega, U=U, g=g, statwl=statwl)
