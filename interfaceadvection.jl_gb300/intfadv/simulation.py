"""TwoPhaseSimulation, sim_step!, MPFMomStep!, MPCFL — host mirror of
src/InterfaceAdvection.jl:64-107 and src/flow.jl:60-109, 262-281.

The Flow and cVOF fields live on the device in the reference layout and are
bound to one library handle; every compute call is a C-ABI call.
"""
from __future__ import annotations

import ctypes as C
import math
import warnings

import torch

from . import _lib
from .core import FP64, Flow, Handle, _raise_or_warn, apply_vof, cVOF, make_config
from .fields import ptr


class NoBody:
    """Placeholder of WaterLily.NoBody (BDIM bodies are not supported by the reference's step either)."""


class TwoPhaseSimulation:
    """TwoPhaseSimulation(dims, u_BC, L; U, Δt, ν, g, u0, perdir, λμ, λρ, η, InterfaceSDF, λ,
    normalScheme) — src/InterfaceAdvection.jl:64-85.

    ``u0(i, x)`` initialises the face velocities (0-based component, coordinate tensors at
    WaterLily loc(i,I)); ``g`` is a constant gravity vector; ``InterfaceSDF`` a vectorised
    SDF (dark fluid where negative).  ``poisson`` selects "fp64" (FP64 V-cycles) or "mixed"
    (FP32 V-cycles inside FP64 flexible CG); ``poisson_tol`` is the L∞ residual of the
    dt-scaled pressure system (the reference passes tol=1e-4 to WaterLily's solver!).
    ``poisson="learned"`` (3D, dims multiples of 4) preconditions the inner FCG of the mixed
    solver with the conv net: ``precond`` is "hybrid" (net then V-cycle), "net", "none" or
    "vcycle"; ``nn_weights`` a parameter vector or a weights file (default: the trained
    weights shipped with the package).  ``momentum_arith`` selects the arithmetic of the
    momentum kernels: "fp64", "ff" (FP32 pairs) or "default" (pairs with the mixed and learned
    solvers, FP64 with the FP64 solver).
    """

    def __init__(self, dims, u_BC, L, *, U=None, Δt=0.25, ν=0.0, g=None, u0=None, perdir=(), exitBC=False,
                 λμ=1e-2, λρ=1e-3, η=None, InterfaceSDF=None, λ="Koren", normalScheme="WH", T=FP64,
                 poisson="fp64", poisson_tol=1e-4, poisson_itmx=200, device="cuda", body=None, ϵ=1,
                 precond="hybrid", nn_weights=None, inner_max=30, inner_rtol=1e-4, momentum_arith="default"):
        if T != FP64:
            raise NotImplementedError("the GB300 path computes in FP64 (Poisson V-cycles optionally FP32)")
        if exitBC:
            raise NotImplementedError("exitBC is not supported")
        if body is not None and not isinstance(body, NoBody):
            raise NotImplementedError("BDIM bodies are not supported (the reference's sim_step! ignores them)")
        dims = tuple(int(n) for n in dims)
        self.L = float(L)
        self.U = math.sqrt(sum(float(x) ** 2 for x in u_BC)) if U is None else float(U)
        self.ϵ = ϵ
        self.body = NoBody()
        self.flow = Flow(dims, u_BC, Δt=Δt, ν=ν, g=g, u0fn=u0, perdir=perdir, device=device)
        cfg = make_config(dims, perdir=perdir, lrho=λρ, lmu=λμ, mu=(None if ν == 0 else ν),
                          eta=(None if (η is None or η == 0) else η), nu=ν, g=g, uBC=u_BC,
                          normalScheme=normalScheme, limiter=λ, poisson=poisson, poisson_tol=poisson_tol,
                          poisson_itmx=poisson_itmx)
        # cVOF(dims; μ=flow.ν, ...) (src/InterfaceAdvection.jl:78)
        self.intf = cVOF(dims, device=device, InterfaceSDF=InterfaceSDF, mu=ν, lmu=λμ, lrho=λρ, eta=η,
                         normalScheme=normalScheme, perdir=perdir, _config=cfg)
        self.handle: Handle = self.intf.handle
        fl, it = self.flow, self.intf
        self.handle.bind(u=fl.u, u0=fl.u0, force=fl.f, sigma=fl.sigma, p=fl.p, mu0=fl.mu0, f=it.f, f0=it.f0,
                         alpha=it.alpha, nhat=it.nhat, fF=it.fF, rhou=it.rhou, rhouf=it.rhouf, drho=it.drho,
                         cbar=it.cbar)
        set_momentum_arith(self.handle, momentum_arith)
        if poisson == "learned":
            set_learned(self.handle, precond=precond, weights=nn_weights, inner_max=inner_max, inner_rtol=inner_rtol)
        _lib.check(self.handle.call("ia_bc_velocity", ptr(fl.u)), "ia_bc_velocity")   # Flow: BC!(u)
        fl.u0.copy_(fl.u)
        fl.Δt[-1] = min(fl.Δt[-1], MPCFL(self))                                       # :81
        self.pois = None
        self.last_status = None

    # property forwarding of the Julia wrapper (src/InterfaceAdvection.jl:86-87)
    @property
    def sim(self):
        return self

    def sim_time(self) -> float:
        return sum(self.flow.Δt[:-1]) * (self.U / self.L if self.L else 1.0)


def set_learned(handle, precond="hybrid", weights=None, inner_max=30, inner_rtol=1e-4):
    """Load the net parameters into a learned-mode handle and select its inner preconditioner."""
    import os

    import numpy as np

    from . import learned
    if weights is None:
        if os.path.exists(learned.WEIGHTS):
            weights = learned.WEIGHTS
        else:
            warnings.warn("no trained weights for the learned preconditioner: the net outputs zero and the "
                          "hybrid preconditioner reduces to the V-cycle")
    if weights is not None:
        w = learned.load_params(weights)[0] if isinstance(weights, str) else np.asarray(weights, np.float32)
        learned.Net(handle).set_params(w)
    _lib.check(handle.call("ia_poisson_precond", _lib.PRECONDS[precond] if isinstance(precond, str) else int(precond),
                           int(inner_max), float(inner_rtol)), "ia_poisson_precond")


def set_momentum_arith(handle, kind: str = "default") -> None:
    """Arithmetic of the momentum kernels: "fp64", "ff" (FP32 pairs) or "default" (ia_momentum_arith)."""
    _lib.check(handle.call("ia_momentum_arith", C.c_int32(_lib.ARITH[kind])), "ia_momentum_arith")


def set_poisson_coef16(handle, on: bool) -> None:
    """FP16 face coefficients for the finest-level smoother of the mixed V-cycle (ia_poisson_coef16)."""
    _lib.check(handle.call("ia_poisson_coef16", C.c_int32(1 if on else 0)), "ia_poisson_coef16")


def set_poisson_slab_rows(handle, rows: int) -> None:
    """Rows per slab of the finest-level smoothing wavefront (ia_poisson_slab_rows; 0 = whole-level
    half-sweeps); the results do not depend on it."""
    _lib.check(handle.call("ia_poisson_slab_rows", C.c_int32(int(rows))), "ia_poisson_slab_rows")


def set_smoother(handle, kind: str = "halfsweep", omega: float | None = None) -> None:
    """Smoother of the FP32 V-cycle: "halfsweep" (one launch per red-black half-sweep, the default)
    or "blocked" (all half-sweeps of a smoothing in one z-wavefront launch, relaxation factor 1 only);
    same arithmetic.  omega sets the half-sweeps' over-relaxation x += ω (x_GS - x) (default 1.15)."""
    _lib.check(handle.call("ia_poisson_smoother", _lib.SMOOTHERS[kind]), "ia_poisson_smoother")
    if omega is not None:
        _lib.check(handle.call("ia_poisson_mg_relax", float(omega)), "ia_poisson_mg_relax")


def poisson_stats(handle) -> dict:
    """Counters of the Poisson solver: net applications, V-cycles, fallbacks, inner and outer iterations."""
    out = (C.c_int64 * 5)()
    _lib.check(handle.call("ia_poisson_stats", out), "ia_poisson_stats")
    return dict(zip(("net", "vcycles", "fallbacks", "inner", "outer"), list(out)))


def MPCFL(sim) -> float:
    """MPCFL(flow, intf) — src/flow.jl:262-281."""
    out = C.c_double()
    _lib.check(sim.handle.call("ia_cfl", C.byref(out)), "ia_cfl")
    return out.value


def surfTen(intf: cVOF, forcing, f=None, fbuffer=None, η=None) -> None:
    """surfTen!(forcing, f, α, n̂, fbuffer, η; perdir) — src/surfaceTension.jl:8-20.

    Accumulates η κ (−∂(d,I,f)) into the device vector field ``forcing`` for every direction d.
    ``fbuffer`` (default: the cVOF's fᶠ, which the reference passes) supplies the buffer content the
    reference reads at its never-written high x ghost; it is not modified.  α and n̂ are not touched.
    """
    f = intf.f if f is None else f
    fbuffer = intf.fF if fbuffer is None else fbuffer
    eta = intf.eta if η is None else η
    _lib.check(intf.handle.call("ia_surften", ptr(forcing), ptr(f), ptr(fbuffer), C.c_double(eta or 0.0)),
               "ia_surften")


def MPFMomStep(sim, δt=None) -> _lib.Status:
    """MPFMomStep!(flow, pois, intf, body; δt=last(Δt)) — src/flow.jl:60-109 (push!(Δt, ...) included)."""
    fl = sim.flow
    dt = fl.Δt[-1] if δt is None else float(δt)
    st = _lib.Status()
    code = sim.handle.call("ia_mom_step", C.c_double(dt), C.c_int64(len(fl.Δt)), C.c_double(sum(fl.Δt)),
                           C.byref(st))
    sim.last_status = st
    if code in (_lib.IA_ERR_NAN, _lib.IA_ERR_DIVERGENCE):
        _raise_or_warn(st, "ia_mom_step")
    _lib.check(code, "ia_mom_step", allow=(_lib.IA_OK, _lib.IA_WARN_FILL, _lib.IA_WARN_NOT_CONVERGED))
    if code == _lib.IA_WARN_FILL:
        _raise_or_warn(st, "ia_mom_step")
    fl.Δt.append(st.dt_next)
    return st


def sim_step(sim, *, remeasure=False, udf=None):
    """sim_step!(sim::TwoPhaseSimulation; remeasure, udf) — src/InterfaceAdvection.jl:100-103."""
    if udf is not None:
        raise NotImplementedError("udf is not supported")
    return MPFMomStep(sim)


def sim_info(sim):
    print(f"    tU/L={sim.sim_time():10.6f}, ΔtU/L={sim.flow.Δt[-1] * sim.U / sim.L:.10f}")
