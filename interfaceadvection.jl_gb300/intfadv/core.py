"""Host-side mirror of InterfaceAdvection.jl's cVOF / Flow types and VOF calls.

Every compute call goes through libintfadv_gb300.so (CUDA, sm_103a).  Names
and argument meaning follow the reference (file:line cited per function);
Python indices are 0-based and time-step history is the list ``Δt``.
"""
from __future__ import annotations

import ctypes as C
import math
import warnings

import torch

from . import _lib
from .fields import cell_coords, evaluate, face_coords, fones, fzeros, ptr

FP64 = torch.float64


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class Handle:
    """Owns one ia_handle (library scratch on the current device)."""

    def __init__(self, cfg: _lib.Config):
        L = _lib.load()
        self.cfg = cfg
        h = C.c_void_p()
        _lib.check(L.ia_create(C.byref(cfg), C.byref(h)), "ia_create")
        self.h = h
        self._fields = _lib.Fields()

    def __del__(self):
        try:
            if getattr(self, "h", None) and self.h.value:
                _lib.load().ia_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def call(self, name, *args):
        L = _lib.load()
        L.ia_set_stream(self.h, _stream())
        return getattr(L, name)(self.h, *args)

    def bind(self, **fields):
        for k, v in fields.items():
            setattr(self._fields, k, ptr(v) if v is not None else None)
        _lib.check(self.call("ia_bind_fields", C.byref(self._fields)), "ia_bind_fields")


def make_config(N, *, perdir=(), lrho=1e-3, lmu=1e-2, mu=None, eta=None, nu=0.0, g=None, uBC=None,
                normalScheme="WH", limiter="Koren", poisson="fp64", poisson_tol=1e-8, poisson_itmx=200,
                exitBC=False) -> _lib.Config:
    D = len(N)
    if D not in (2, 3):
        raise ValueError("only 2D and 3D grids are supported")
    c = _lib.Config()
    c.D = D
    c.perdir = sum(1 << int(j) for j in perdir)
    for d in range(D):
        c.N[d] = int(N[d])
    c.lrho, c.lmu = float(lrho), float(lmu)
    c.mu = 0.0 if mu is None else float(mu)
    c.eta = 0.0 if eta is None else float(eta)
    c.nu = float(nu)
    if g is not None:
        c.has_g = 1
        for d in range(D):
            c.g[d] = float(g[d])
    if uBC is not None:
        for d in range(D):
            c.uBC[d] = float(uBC[d])
    c.normal_scheme = _lib.NORMAL_SCHEMES[normalScheme] if isinstance(normalScheme, str) else int(normalScheme)
    c.limiter = _lib.LIMITERS[limiter] if isinstance(limiter, str) else int(limiter)
    c.poisson_mode = _lib.POISSON_MODES[poisson] if isinstance(poisson, str) else int(poisson)
    c.poisson_tol = float(poisson_tol)
    c.poisson_itmx = int(poisson_itmx)
    c.exitBC = 1 if exitBC else 0
    return c


def _raise_or_warn(st: _lib.Status, where: str):
    """Error behaviour of reportFillError (src/advection.jl:145-189)."""
    code = st.code
    if code == _lib.IA_ERR_NAN:
        raise FloatingPointError("NaN!")
    if code == _lib.IA_ERR_DIVERGENCE:
        raise FloatingPointError("divergence is exploding!")
    if code == _lib.IA_WARN_FILL:
        if st.flags & _lib.FLAG_OVERFILL:
            warnings.warn(f"max VOF @ {st.maxid} ∉ [0,1] @ direction {st.fill_dir}, Δf = {st.maxf - 1}")
        if st.flags & _lib.FLAG_UNDERFILL:
            warnings.warn(f"min VOF @ {st.minid} ∉ [0,1] @ direction {st.fill_dir}, Δf = {-st.minf}")
        return
    if code == _lib.IA_WARN_NOT_CONVERGED:
        return
    _lib.check(code, where)


class cVOF:
    """cVOF(N; InterfaceSDF, μ, λμ, λρ, η, normalScheme, perdir) — src/cVOF.jl:45-89.

    Holds the device fields f, f0 (f⁰), alpha (α), nhat (n̂), fF (fᶠ), cbar (c̄,
    int8), rhou (ρu), rhouf (ρuf), drho (dρ) in the reference layout.
    ``InterfaceSDF`` is a vectorised signed-distance function of the
    coordinate tensors (dark fluid where it is negative).
    """

    def __init__(self, N, *, T=FP64, device="cuda", InterfaceSDF=None, mu=1e-3, lmu=1e-2, lrho=1e-3, eta=None,
                 normalScheme="WH", perdir=(), _config=None):
        if T != FP64:
            raise NotImplementedError("the GB300 path computes fractions in FP64 only")
        self.N = tuple(int(n) for n in N)
        self.D = len(self.N)
        self.Ng = tuple(n + 2 for n in self.N)
        self.device = device
        Nv = self.Ng + (self.D,)
        self.f = fones(self.Ng, FP64, device)
        self.alpha = fzeros(self.Ng, FP64, device)
        self.nhat = fzeros(Nv, FP64, device)
        self.cbar = fzeros(self.Ng, torch.int8, device)
        self.mu = None if (mu is None or mu == 0) else float(mu)
        self.lmu, self.lrho = float(lmu), float(lrho)
        self.eta = None if (eta is None or eta == 0) else float(eta)
        self.normalScheme = normalScheme
        self.perdir = tuple(perdir)
        cfg = _config or make_config(self.N, perdir=self.perdir, lrho=lrho, lmu=lmu, mu=self.mu, eta=self.eta,
                                     normalScheme=normalScheme)
        self.handle = Handle(cfg)
        if InterfaceSDF is not None:
            apply_vof(self, InterfaceSDF)
        self.f0 = _fclone(self.f)
        self.fF = fzeros(self.Ng, FP64, device)
        self.rhou = fzeros(Nv, FP64, device)
        self.rhouf = fzeros(Nv, FP64, device)
        self.drho = fones(Nv, FP64, device)
        self.handle.bind(f=self.f, f0=self.f0, alpha=self.alpha, nhat=self.nhat, fF=self.fF, rhou=self.rhou,
                         rhouf=self.rhouf, drho=self.drho, cbar=self.cbar)

    def mass(self, f=None) -> float:
        """Σ f over interior cells (FP64, deterministic)."""
        out = C.c_double()
        _lib.check(self.handle.call("ia_mass", ptr(self.f if f is None else f), C.byref(out)), "ia_mass")
        return out.value


def _fclone(t: torch.Tensor) -> torch.Tensor:
    out = fzeros(tuple(t.shape), t.dtype, t.device)
    out.copy_(t)
    return out


def apply_vof(intf: cVOF, sdf, f=None, alpha=None, nhat=None, h=0.01):
    """applyVOF!(f, α, n̂, InterfaceSDF) + BCf! — src/VOFutil.jl:9-37, src/cVOF.jl:56.

    The SDF is sampled at cell centres and at ±0.01 e_d exactly as the reference's
    finite-difference normal, on the device; the PLIC fractions come from the library.
    """
    f = intf.f if f is None else f
    alpha = intf.alpha if alpha is None else alpha
    nhat = intf.nhat if nhat is None else nhat
    ng, D = intf.Ng, intf.D
    samples = torch.empty((1 + 2 * D,) + tuple(reversed(ng)), dtype=FP64, device=intf.device)
    xc = cell_coords(ng, intf.device)
    samples[0] = evaluate(sdf, xc, ng, intf.device).permute(*reversed(range(D)))
    for d in range(D):
        for k, s in enumerate((+h, -h)):
            x = [c + (s if e == d else 0.0) for e, c in enumerate(xc)]
            samples[1 + 2 * d + k] = evaluate(sdf, x, ng, intf.device).permute(*reversed(range(D)))
    L = intf.handle
    _lib.check(L.call("ia_apply_vof", C.c_void_p(samples.data_ptr()), ptr(f), ptr(alpha), ptr(nhat)),
               "ia_apply_vof")
    del samples


class Flow:
    """The WaterLily Flow members the step reads: u, u⁰ (u0), f (force), σ (sigma), p, μ₀ (mu0), Δt.

    ``u0fn(i, x)`` (0-based component, coordinate tensors) initialises u on the
    faces (WaterLily loc(i,I)); without it u = u_BC everywhere.
    """

    def __init__(self, N, uBC, *, Δt=0.25, ν=0.0, g=None, u0fn=None, perdir=(), exitBC=False, device="cuda"):
        self.N = tuple(int(n) for n in N)
        self.D = len(self.N)
        self.Ng = tuple(n + 2 for n in self.N)
        Nv = self.Ng + (self.D,)
        self.uBC = tuple(float(x) for x in uBC)
        self.ν = float(ν)
        self.g = None if g is None else tuple(float(x) for x in g)
        self.perdir = tuple(perdir)
        self.exitBC = bool(exitBC)
        self.Δt = [float(Δt)]
        self.device = device
        self.u = fzeros(Nv, FP64, device)
        for i in range(self.D):
            if u0fn is None:
                self.u[..., i].fill_(self.uBC[i])
            else:
                self.u[..., i].copy_(evaluate(lambda x, i=i: u0fn(i, x), face_coords(self.Ng, i, device),
                                              self.Ng, device))
        self.u0 = fzeros(Nv, FP64, device)
        self.f = fzeros(Nv, FP64, device)
        self.sigma = fzeros(self.Ng, FP64, device)
        self.p = fzeros(self.Ng, FP64, device)
        self.mu0 = fones(Nv, FP64, device)


def advect(a: Flow, c: cVOF, f=None, u1=None, u2=None, dt=None) -> _lib.Status:
    """advect!(a, c, f=c.f, u¹=a.u⁰, u²=a.u, dt=last(a.Δt)) — src/advection.jl:17-23.

    Lie–Trotter split VOF advection of ``f`` in place with split order
    dirO[i] = mod(length(Δt)+i, D).  Raises FloatingPointError on NaN or exploding
    divergence and warns on over/under-fill, like reportFillError.
    """
    f = c.f if f is None else f
    u1 = a.u0 if u1 is None else u1
    u2 = a.u if u2 is None else u2
    dt = a.Δt[-1] if dt is None else float(dt)
    st = _lib.Status()
    c.handle.call("ia_advect_vof", ptr(f), ptr(u1), ptr(u2), C.c_double(dt), C.c_int64(len(a.Δt)),
                  C.byref(st))
    _raise_or_warn(st, "ia_advect_vof")
    return st


def advect_vof_raw(c: cVOF, f, u1, u2, dt: float, n_dt: int) -> _lib.Status:
    """advectVOF! with explicit arguments (src/advection.jl:34-78); no error raising."""
    st = _lib.Status()
    c.handle.call("ia_advect_vof", ptr(f), ptr(u1), ptr(u2), C.c_double(dt), C.c_int64(n_dt), C.byref(st))
    return st


def reconstruct_interface(c: cVOF, f=None, alpha=None, nhat=None):
    """reconstructInterface!(f, α, n̂, normalScheme; perdir) — src/normalEstimation.jl:10-28."""
    f = c.f if f is None else f
    alpha = c.alpha if alpha is None else alpha
    nhat = c.nhat if nhat is None else nhat
    _lib.check(c.handle.call("ia_reconstruct", ptr(f), ptr(alpha), ptr(nhat)), "ia_reconstruct")


def get_vof_flux(c: cVOF, fF, f, alpha, nhat, u, u0, dt, d, rhouf=None):
    """getVOFFlux!(fᶠ, f, α, n̂, u, u⁰, δt, d, ρuf, λρ) — src/advection.jl:108-112 (d 0-based)."""
    _lib.check(c.handle.call("ia_vof_flux", ptr(fF), ptr(f), ptr(alpha), ptr(nhat), ptr(u), ptr(u0),
                             C.c_double(dt), C.c_int32(d), ptr(rhouf)), "ia_vof_flux")


# reference spellings
advectVOF = advect_vof_raw
reconstructInterface = reconstruct_interface
getVOFFlux = get_vof_flux
applyVOF = apply_vof
