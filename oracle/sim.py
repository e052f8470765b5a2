"""ORACLE — test infrastructure, not product code.

Host-side restatement of TwoPhaseSimulation (src/InterfaceAdvection.jl:64-85)
driving the C++ oracle: WaterLily Flow initialisation (face velocities from
u0 at loc(i,I) = I - 1.5 - 0.5 e_i, then BC!), cVOF from an SDF, the initial
MPCFL clip, and sim_step! → MPFMomStep! with push!(Δt, min(MPCFL, 1.2δt)).
Used by the tests and by bench.py's CPU baseline / reference arm only.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import pyoracle as O


def _coords(ng, shift_dim=None):
    idx = np.meshgrid(*[np.arange(n, dtype=np.float64) for n in ng], indexing="ij")
    x = [c - 0.5 for c in idx]
    if shift_dim is not None:
        x[shift_dim] = x[shift_dim] - 0.5
    return x


def sdf_samples(ng, sdf, h=0.01):
    xc = _coords(ng)
    out = [np.asfortranarray(sdf(xc))]
    for d in range(len(ng)):
        for s in (+h, -h):
            x = [xc[e] + (s if e == d else 0.0) for e in range(len(ng))]
            out.append(np.asfortranarray(sdf(x)))
    return out


class OracleSim:
    """Fields of Flow + cVOF in host memory, stepped by the oracle."""

    def __init__(self, N, uBC, *, sdf=None, u0=None, Δt=0.25, ν=0.0, g=None, perdir=(), lrho=1e-3, lmu=1e-2,
                 eta=None, scheme="WH", limiter="Koren", ptol=1e-12, pitmx=5000, mu=None, psolver="jacobi"):
        self.N = tuple(N)
        self.D = len(N)
        self.ng = tuple(n + 2 for n in N)
        self.per = tuple(perdir)
        self.g = O.grid(self.ng, self.per)
        ng, D = self.ng, self.D
        nv = ng + (D,)
        z = lambda shape=ng: O.zeros(shape)
        self.u = z(nv)
        for i in range(D):
            if u0 is None:
                self.u[..., i] = uBC[i]
            else:
                self.u[..., i] = u0(i, _coords(ng, i))
        self.uBC = (C.c_double * 3)(*(list(uBC) + [0.0] * (3 - D)))
        O.lib().orc_bc_vel(C.byref(self.g), O.ptr(self.u), self.uBC)
        self.u0 = self.u.copy(order="F")
        self.force, self.sigma, self.p, self.mu0 = z(nv), z(), z(), z(nv)
        self.mu0[...] = 1.0
        self.pr, self.peps, self.pz, self.pD, self.piD = z(), z(), z(), z(), z()
        self.f = z()
        self.f[...] = 1.0
        self.alpha, self.nhat = z(), z(nv)
        if sdf is not None:
            samples = sdf_samples(ng, sdf)
            arr = (C.c_void_p * len(samples))(*[s.ctypes.data for s in samples])
            O.lib().orc_apply_vof(C.byref(self.g), O.ptr(self.f), O.ptr(self.alpha), O.ptr(self.nhat), arr)
            O.lib().orc_bcf(C.byref(self.g), O.ptr(self.f))
        self.f0 = self.f.copy(order="F")
        self.fF = z()
        self.rhou, self.rhouf = z(nv), z(nv)
        self.drho = z(nv)
        self.drho[...] = 1.0
        self.cbar = O.zeros(ng, np.int8)
        s = O.State()
        for name in ("u", "u0", "force", "sigma", "p", "mu0", "pr", "peps", "pz", "pD", "piD", "f", "f0", "alpha",
                     "nhat", "fF", "rhou", "rhouf", "drho", "cbar"):
            setattr(s, name, getattr(self, name).ctypes.data)
        s.lrho, s.lmu = lrho, lmu
        # cVOF(...; μ=flow.ν): the dark fluid's dynamic viscosity is WaterLily's ν (src/InterfaceAdvection.jl:78)
        mu_eff = ν if mu is None else mu
        s.mu = 0.0 if not mu_eff else float(mu_eff)
        s.eta = 0.0 if not eta else float(eta)
        s.nu = float(ν)
        if g is not None:
            s.has_g = 1
            for i in range(D):
                s.g[i] = float(g[i])
        s.scheme = O.SCHEMES[scheme]
        s.limiter = O.LIMITERS[limiter]
        for i in range(D):
            s.uBC[i] = float(uBC[i])
        s.ptol, s.pitmx = ptol, pitmx
        # "jacobi": the reference's psolver! (src/flow.jl:300-326); "mg": multigrid-preconditioned CG in
        # the role of WaterLily's MultiLevelPoisson, the reference's default (src/flow.jl:343-347)
        s.psolver = {"jacobi": 0, "mg": 1}[psolver]
        self.s = s
        self.Δt = [float(Δt)]
        self.Δt[-1] = min(self.Δt[-1], self.mpcfl())      # src/InterfaceAdvection.jl:81

    def mpcfl(self) -> float:
        return O.lib().orc_mpcfl(C.byref(self.g), C.byref(self.s), 0.0)

    def step(self, dt=None):
        """sim_step! (src/InterfaceAdvection.jl:100-103) → MPFMomStep! (src/flow.jl:60-109)."""
        dt = self.Δt[-1] if dt is None else float(dt)
        st = O.FillStatus()
        O.lib().orc_mom_step(C.byref(self.g), C.byref(self.s), dt, sum(self.Δt), len(self.Δt), C.byref(st))
        self.Δt.append(min(self.mpcfl(), 1.2 * dt))
        return st

    def mass(self):
        inner = tuple(slice(1, -1) for _ in range(self.D))
        return float(self.f[inner].sum())
