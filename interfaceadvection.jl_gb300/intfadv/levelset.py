"""Level-set reinitialisation — host mirror of src/redistaning.jl (C-ABI ia_levelset_* /
ia_redistance).  Boundary conditions follow the simulation's handle (its periodic dimensions)."""
from __future__ import annotations

from . import _lib
from .fields import ptr


class LevelSet:
    """LevelSet(sim) (src/redistaning.jl:13-25): ϕ = 2f - 1 stored in sim.intf.f0, with ϕ⁰ in
    sim.intf.alpha, ϕ_ini (a copy of ϕ) in sim.intf.fF and L in sim.flow.sigma — the reference's
    buffer reuse, so no memory is allocated."""

    def __init__(self, sim):
        it = sim.intf
        self.handle = sim.handle
        self.ϕ, self.ϕ0, self.ϕini, self.L = it.f0, it.alpha, it.fF, sim.flow.sigma
        _lib.check(self.handle.call("ia_levelset_init", ptr(it.f), ptr(self.ϕ), ptr(self.ϕini)), "ia_levelset_init")

    @property
    def phi(self):
        return self.ϕ


def redistaning(ls: LevelSet, d: float = 5.0, dτ: float = 0.5) -> None:
    """redistaning!(ls; d, dτ) (src/redistaning.jl:42-54): round(d/dτ) SSP-RK3 pseudo-time steps of
    ∂τϕ = sign(ϕ_ini)(1 - |∇ϕ|) with BCf! ghosts after every stage."""
    _lib.check(ls.handle.call("ia_redistance", ptr(ls.ϕ), ptr(ls.ϕ0), ptr(ls.ϕini), ptr(ls.L), float(d), float(dτ)),
               "ia_redistance")


def computeL(handle, L, phi, phi_ini) -> None:
    """computeL!(L, ϕ, ϕ_ini) (src/redistaning.jl:64-83) on the handle's grid."""
    _lib.check(handle.call("ia_levelset_rhs", ptr(L), ptr(phi), ptr(phi_ini)), "ia_levelset_rhs")


redistaning_ = redistaning
