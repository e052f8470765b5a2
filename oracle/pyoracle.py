"""ORACLE — test infrastructure, not product code.

ctypes binding of the C++ CPU restatement in ``oracle.cpp`` (the checker for
the CUDA path and the timed CPU baseline).  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (cpu_baseline and the
``--impl reference`` arm) import this module.

Arrays are numpy arrays in Fortran (column-major) order with the reference's
shapes: scalars ``Ng``, vectors ``Ng + (D,)``, where ``Ng = N + 2``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "oracle.cpp")
SRC_NN = os.path.join(HERE, "nn_oracle.cpp")
SRC_MET = os.path.join(HERE, "metrics_oracle.cpp")
SRC_LS = os.path.join(HERE, "levelset_oracle.cpp")
LIB = os.path.join(HERE, "liboracle.so")

SCHEMES = {"WH": 0, "WY": 1, "MYC": 2, "Y": 3, "Column": 4, "PCD": 5, "SLIC": 6, "CD": 7, "XYLIC": 8}
LIMITERS = {"Koren": 0, "upwind": 1, "minmod": 2, "vanAlbada1": 3, "Sweby": 4, "superbee": 5,
            "TVDcen": 6, "TVDdown": 7}


def build(force: bool = False) -> str:
    """Compile liboracle.so with g++ (OpenMP, IEEE FP64, no FMA contraction)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(SRC), os.path.getmtime(SRC_NN), os.path.getmtime(SRC_MET), os.path.getmtime(SRC_LS),
            os.path.getmtime(os.path.join(HERE, "oracle.h"))):
        cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
               SRC, SRC_NN, SRC_MET, SRC_LS, "-o", LIB + ".tmp"]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


class Grid(C.Structure):
    _fields_ = [("D", C.c_int32), ("per", C.c_int32), ("n", C.c_int64 * 3)]


class FillStatus(C.Structure):
    _fields_ = [("nan", C.c_int32), ("over", C.c_int32), ("under", C.c_int32), ("diverge", C.c_int32),
                ("dir", C.c_int32), ("pad", C.c_int32), ("maxf", C.c_double), ("minf", C.c_double),
                ("maxid", C.c_int64), ("minid", C.c_int64)]


class State(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("u", "u0", "force", "sigma", "p", "mu0", "pr", "peps", "pz", "pD",
                                           "piD", "f", "f0", "alpha", "nhat", "fF", "rhou", "rhouf", "drho",
                                           "cbar")] + [
        ("lrho", C.c_double), ("lmu", C.c_double), ("mu", C.c_double), ("eta", C.c_double), ("nu", C.c_double),
        ("g", C.c_double * 3), ("has_g", C.c_int32), ("scheme", C.c_int32), ("limiter", C.c_int32),
        ("pad", C.c_int32), ("uBC", C.c_double * 3), ("ptol", C.c_double), ("pitmx", C.c_int32),
        ("piters", C.c_int32), ("presid", C.c_double), ("psolver", C.c_int32), ("pad2", C.c_int32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        d, i, i64, p = C.c_double, C.c_int, C.c_int64, C.c_void_p
        f = C.c_float
        sig = {
            "orc_get_intercept2": (d, [d, d, d]), "orc_get_intercept3": (d, [d, d, d, d]),
            "orc_get_volume_fraction2": (d, [d, d, d]), "orc_get_volume_fraction3": (d, [d, d, d, d]),
            "orc_get_intercept2f": (f, [f, f, f]), "orc_get_intercept3f": (f, [f, f, f, f]),
            "orc_get_volume_fraction2f": (f, [f, f, f]), "orc_get_volume_fraction3f": (f, [f, f, f, f]),
            "orc_proot": (d, [d, d, d, d]),
            "orc_normal": (i, [p, i, p, p, i64]),
            "orc_reconstruct": (None, [p, i, p, p, p]),
            "orc_bcvof": (None, [p, p, p, p]), "orc_bcf": (None, [p, p]), "orc_bcf_d": (None, [p, i, p]),
            "orc_bcv": (None, [p, p]), "orc_bc_vel": (None, [p, p, p]), "orc_perbc": (None, [p, p]),
            "orc_clean_wisp": (None, [p, p, d]), "orc_f2face": (None, [p, p, p]),
            "orc_get3cellheight": (d, [p, p, i64, i]), "orc_getmu": (d, [p, i, i, i64, p, d, d, d]),
            "orc_apply_vof": (None, [p, p, p, p, p]),
            "orc_vof_flux": (None, [p, p, p, p, p, p, p, d, i, p, d]),
            "orc_advect_vof": (None, [p, i, p, p, p, p, p, p, d, p, p, d, p, p]),
            "orc_popinet_height": (d, [p, p, i64, i]), "orc_curvature": (d, [p, p, i64, i]),
            "orc_surften": (None, [p, p, p, p, p, d]),
            "orc_mom_step": (None, [p, p, d, d, i64, p]), "orc_mpcfl": (d, [p, p, d]),
            "orc_poisson": (None, [p, p]),
            "orc_argabsmax": (i, [i, p]), "orc_get_xdir": (i, [i]), "orc_get_xydir": (None, [i, p, p]),
            "orc_getrho_cell": (d, [d, d]), "orc_getrho_face": (d, [p, i, i64, p, d]),
            "orc_vof_flux_face": (None, [p, p, p, p, p, d, i, i64, p, d]),
            "orc_rhoke": (d, [p, i64, p, p, d, p]), "orc_rhou": (d, [p, i, i64, p, p, d, p]),
            "orc_rhogh": (d, [p, i64, p, p, d, p]), "orc_ens": (d, [p, i64, p]),
            "orc_metrics": (None, [p, p, p, p, d, p, p, p, p]),
            "orc_levelset_init": (None, [p, p, p, p]), "orc_levelset_rhs": (None, [p, p, p, p]),
            "orc_levelset_stage": (None, [p, p, p, p, p, d, d]),
            "orc_redistance": (None, [p, p, p, p, p, d, d]),
            "orc_nn_param_count": (i64, []),
            "orc_nn_forward": (None, [p, p, i, i, i, i, p]),
            "orc_nn_loss_grad": (d, [p, p, p, i, i, i, i, p]),
            "orc_nn_loss_grad_kind": (d, [p, p, p, i, i, i, i, i, p]),
            "orc_nn_adam": (None, [i64, p, p, p, p, d, i64]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags.f_contiguous, "oracle arrays must be Fortran-ordered"
    return a.ctypes.data


def grid(ng, per=()) -> Grid:
    """Grid descriptor from the ghost-inclusive shape and the 0-based periodic dimensions."""
    g = Grid()
    g.D = len(ng)
    g.per = sum(1 << j for j in per)
    g.n[0], g.n[1] = ng[0], ng[1]
    g.n[2] = ng[2] if len(ng) == 3 else 1
    return g


def lin(ng, idx) -> int:
    """0-based linear index of a 0-based coordinate tuple."""
    s, m = 0, 1
    for k, c in enumerate(idx):
        s += c * m
        m *= ng[k]
    return s


def zeros(shape, dtype=np.float64):
    return np.zeros(shape, dtype=dtype, order="F")


# ---- thin wrappers used by the tests ---------------------------------------------------------

def get_intercept(*args, dtype=np.float64):
    L = lib()
    if dtype == np.float32:
        return (L.orc_get_intercept2f if len(args) == 3 else L.orc_get_intercept3f)(*map(float, args))
    return (L.orc_get_intercept2 if len(args) == 3 else L.orc_get_intercept3)(*map(float, args))


def get_volume_fraction(*args, dtype=np.float64):
    L = lib()
    if dtype == np.float32:
        return (L.orc_get_volume_fraction2f if len(args) == 3 else L.orc_get_volume_fraction3f)(*map(float, args))
    return (L.orc_get_volume_fraction2 if len(args) == 3 else L.orc_get_volume_fraction3)(*map(float, args))


def normal(f, idx, scheme="WH"):
    """Apply one normal scheme at the 0-based cell ``idx`` of ``f``; returns n̂[I,:]."""
    f = np.asfortranarray(f, dtype=np.float64)
    nh = zeros(f.shape + (f.ndim,))
    g = grid(f.shape)
    rc = lib().orc_normal(C.byref(g), SCHEMES[scheme], ptr(f), ptr(nh), lin(f.shape, idx))
    assert rc == 0
    return nh[tuple(idx) + (slice(None),)].copy()


def reconstruct(f, scheme="WH", per=()):
    g = grid(f.shape, per)
    al = zeros(f.shape)
    nh = zeros(f.shape + (f.ndim,))
    lib().orc_reconstruct(C.byref(g), SCHEMES[scheme], ptr(f), ptr(al), ptr(nh))
    return al, nh


def advect_vof(f, u, u0, dt, dirO, lrho=1e-3, scheme="WH", per=(), fF=None, alpha=None, nhat=None):
    """advectVOF! in place on ``f``; returns (status, cbar, rhouf, fF, alpha, nhat)."""
    g = grid(f.shape, per)
    D = f.ndim
    fF = zeros(f.shape) if fF is None else fF
    alpha = zeros(f.shape) if alpha is None else alpha
    nhat = zeros(f.shape + (D,)) if nhat is None else nhat
    cbar = zeros(f.shape, np.int8)
    rhouf = zeros(f.shape + (D,))
    st = FillStatus()
    dirs = (C.c_int * 3)(*list(dirO) + [0] * (3 - len(dirO)))
    lib().orc_advect_vof(C.byref(g), SCHEMES[scheme], ptr(f), ptr(fF), ptr(alpha), ptr(nhat), ptr(u), ptr(u0),
                         float(dt), ptr(cbar), ptr(rhouf), float(lrho), dirs, C.byref(st))
    return st, cbar, rhouf, fF, alpha, nhat


def dir_order(n_dt: int, D: int):
    """Split order of advect!/advectfq!: dirO[i] = mod(length(Δt)+i, D) (0-based)."""
    return [(n_dt + i) % D for i in range(1, D + 1)]


# ---- learned preconditioner network (nn_oracle.cpp) -------------------------------------------

def _c64(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data


def nn_param_count() -> int:
    return int(lib().orc_nn_param_count())


def nn_forward(w, x0):
    """x0: C-ordered [B, nz+2, ny+2, nx+2, 4]; returns [B, nz+2, ny+2, nx+2] (FP64)."""
    B, nzp, nyp, nxp, _ = x0.shape
    w, pw = _c64(w)
    x0, px = _c64(x0)
    out = np.zeros((B, nzp, nyp, nxp), dtype=np.float64)
    lib().orc_nn_forward(pw, px, B, nxp - 2, nyp - 2, nzp - 2, out.ctypes.data)
    return out


def nn_loss_grad(w, x0, tgt, kind="mse"):
    """Training loss over interior cells ("mse" or "energy") and its gradient (FP64)."""
    B, nzp, nyp, nxp, _ = x0.shape
    w, pw = _c64(w)
    x0, px = _c64(x0)
    tgt, pt = _c64(tgt)
    g = np.zeros(w.size, dtype=np.float64)
    loss = lib().orc_nn_loss_grad_kind(pw, px, pt, B, nxp - 2, nyp - 2, nzp - 2, {"mse": 0, "energy": 1}[kind],
                                       g.ctypes.data)
    return float(loss), g


def nn_adam(w, g, m, v, lr, t):
    """One Adam step in place on FP64 arrays (t = step number, from 1)."""
    for a in (w, g, m, v):
        assert a.dtype == np.float64 and a.flags.c_contiguous
    lib().orc_nn_adam(w.size, w.ctypes.data, g.ctypes.data, m.ctypes.data, v.ctypes.data, float(lr), int(t))


# ---- diagnostics (metrics_oracle.cpp) --------------------------------------------------------

def _dv(v, D):
    a = np.zeros(3)
    if v is not None:
        a[:D] = v
    return a


def metrics(u, f, lrho, U=None, g=None, statwl=None, omega=None, per=()):
    """Domain sums {ke, pe, ens, rhou[D]} of the src/metrics.jl per-cell functions."""
    gr = grid(f.shape, per)
    D = f.ndim
    out = np.zeros(3 + D)
    Ua, ga, wa = _dv(U, D), _dv(g, D), _dv(statwl, D)
    lib().orc_metrics(C.byref(gr), ptr(u), ptr(f), ptr(omega), float(lrho), Ua.ctypes.data, ga.ctypes.data,
                      wa.ctypes.data, out.ctypes.data)
    return {"ke": out[0], "pe": out[1], "ens": out[2], "rhou": out[3:].tolist()}


# ---- level-set reinitialisation (levelset_oracle.cpp) -----------------------------------------

def levelset_rhs(phi, ini, per=()):
    L = zeros(phi.shape)
    lib().orc_levelset_rhs(C.byref(grid(phi.shape, per)), ptr(L), ptr(phi), ptr(ini))
    return L


def levelset_stage(phi, phi0, ini, L, dtau, alpha, per=()):
    """In place on phi (and L), like _redistaningStage!; ini may be phi itself."""
    lib().orc_levelset_stage(C.byref(grid(phi.shape, per)), ptr(phi), ptr(phi0), ptr(ini), ptr(L), float(dtau),
                             float(alpha))


def redistance(f, d=5.0, dtau=0.5, per=()):
    """LevelSet from f, then redistaning!; returns ϕ."""
    g = grid(f.shape, per)
    phi, ini, phi0, L = zeros(f.shape), zeros(f.shape), zeros(f.shape), zeros(f.shape)
    lib().orc_levelset_init(C.byref(g), ptr(f), ptr(phi), ptr(ini))
    lib().orc_redistance(C.byref(g), ptr(phi), ptr(phi0), ptr(ini), ptr(L), float(d), float(dtau))
    return phi
