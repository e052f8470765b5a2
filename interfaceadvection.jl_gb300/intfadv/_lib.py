"""ctypes binding of libintfadv_gb300.so (the C-ABI in include/intfadv.h).

The library is the only compute path: when it is missing or fails to load,
every call raises — there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import re

from . import _build

HEADER = os.path.join(os.path.dirname(_build.PKG_ROOT), "include", "intfadv.h")

IA_OK = 0
IA_ERR_NAN = 1
IA_ERR_DIVERGENCE = 2
IA_ERR_UNSUPPORTED = 3
IA_ERR_INVALID = 4
IA_ERR_CUDA = 5
IA_ERR_NO_DEVICE = 6
IA_ERR_TOO_LARGE = 7
IA_WARN_FILL = 100
IA_WARN_NOT_CONVERGED = 101

FLAG_NAN, FLAG_OVERFILL, FLAG_UNDERFILL, FLAG_DIVERGENCE, FLAG_POISSON = 1, 2, 4, 8, 16

NORMAL_SCHEMES = {"WH": 0, "WY": 1, "MYC": 2, "Y": 3, "Column": 4, "PCD": 5, "SLIC": 6, "CD": 7, "XYLIC": 8}
LIMITERS = {"Koren": 0, "upwind": 1, "minmod": 2, "vanAlbada1": 3, "Sweby": 4, "superbee": 5,
            "TVDcen": 6, "TVDdown": 7}
POISSON_MODES = {"fp64": 0, "mixed": 1, "learned": 2}
PRECONDS = {"hybrid": 0, "net": 1, "none": 2, "vcycle": 3}
SMOOTHERS = {"halfsweep": 0, "blocked": 1}
ARITH = {"default": -1, "fp64": 0, "ff": 1}
TIMED_KERNELS = ["vof_bulk", "vof_cells", "ustar", "forcing", "mg_vcycle", "mg_residual", "mg_transfer",
                 "krylov", "other", "vof_faces", "momflux", "momupdate", "update_project", "mg_fine_rbgs", "nn_precond",
                 "mg_fine_first"]


class Config(C.Structure):
    _fields_ = [("D", C.c_int32), ("perdir", C.c_int32), ("N", C.c_int64 * 3),
                ("lrho", C.c_double), ("lmu", C.c_double), ("mu", C.c_double), ("eta", C.c_double),
                ("nu", C.c_double), ("g", C.c_double * 3), ("has_g", C.c_int32), ("normal_scheme", C.c_int32),
                ("limiter", C.c_int32), ("poisson_mode", C.c_int32), ("uBC", C.c_double * 3),
                ("poisson_tol", C.c_double), ("poisson_itmx", C.c_int32), ("exitBC", C.c_int32)]


class Fields(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("u", "u0", "force", "sigma", "p", "mu0", "f", "f0", "alpha", "nhat",
                                           "fF", "rhou", "rhouf", "drho", "cbar")]


class Status(C.Structure):
    _fields_ = [("code", C.c_int32), ("flags", C.c_uint32), ("maxf", C.c_double), ("minf", C.c_double),
                ("maxid", C.c_int64), ("minid", C.c_int64), ("fill_dir", C.c_int32),
                ("poisson_iters", C.c_int32 * 2), ("pad", C.c_int32), ("poisson_resid", C.c_double * 2),
                ("dt_next", C.c_double)]


_SIGS = {
    "ia_create": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_void_p)]),
    "ia_destroy": (C.c_int, [C.c_void_p]),
    "ia_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ia_bind_fields": (C.c_int, [C.c_void_p, C.POINTER(Fields)]),
    "ia_advect_vof": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int64,
                                C.POINTER(Status)]),
    "ia_reconstruct": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ia_vof_flux": (C.c_int, [C.c_void_p] + [C.c_void_p] * 6 + [C.c_double, C.c_int32, C.c_void_p]),
    "ia_apply_vof": (C.c_int, [C.c_void_p] * 5),
    "ia_mass": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]),
    "ia_error_string": (C.c_char_p, [C.c_int]),
    "ia_launch_count": (C.c_int64, []),
    "ia_timing": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32]),
    "ia_mom_step": (C.c_int, [C.c_void_p, C.c_double, C.c_int64, C.c_double, C.POINTER(Status)]),
    "ia_cfl": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "ia_bc_velocity": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ia_poisson_solve": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int32,
                                   C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
    "ia_project": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
    "ia_advect_momentum": (C.c_int, [C.c_void_p] * 5 + [C.c_double, C.c_int64, C.POINTER(Status)]),
    "ia_visc_surften": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ia_surften": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]),
    "ia_momentum_arith": (C.c_int, [C.c_void_p, C.c_int32]),
    "ia_poisson_coef16": (C.c_int, [C.c_void_p, C.c_int32]),
    "ia_poisson_slab_rows": (C.c_int, [C.c_void_p, C.c_int32]),
    "ia_poisson_mg_fine": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "ia_wide_offsets": (C.c_int, [C.c_void_p, C.c_int32]),
    "ia_probe_fma_rates": (C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "ia_advect_vof_noalloc": (C.c_int, [C.POINTER(Config), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_double, C.c_int64, C.c_void_p, C.c_void_p, C.POINTER(Status)]),
    "ia_nn_param_count": (C.c_int64, []),
    "ia_nn_set_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ia_nn_get_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ia_nn_set_loss": (C.c_int, [C.c_void_p, C.c_int32]),
    "ia_nn_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p] + [C.c_int32] * 5),
    "ia_nn_loss_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p] + [C.c_int32] * 4 +
                        [C.c_void_p, C.POINTER(C.c_double)]),
    "ia_nn_train_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p] + [C.c_int32] * 4 +
                         [C.c_float, C.POINTER(C.c_double)]),
    "ia_poisson_precond": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_double]),
    "ia_poisson_stats": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ia_poisson_mg_params": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    "ia_poisson_smoother": (C.c_int, [C.c_void_p, C.c_int32]),
    "ia_poisson_mg_relax": (C.c_int, [C.c_void_p, C.c_double]),
    "ia_poisson_residual": (C.c_int, [C.c_void_p] * 5 + [C.POINTER(C.c_double)]),
    "ia_metrics": (C.c_int, [C.c_void_p] * 8),
    "ia_levelset_init": (C.c_int, [C.c_void_p] * 4),
    "ia_levelset_rhs": (C.c_int, [C.c_void_p] * 4),
    "ia_redistance": (C.c_int, [C.c_void_p] * 5 + [C.c_double, C.c_double]),
}

_lib = None


class IAError(RuntimeError):
    def __init__(self, code: int, where: str = ""):
        self.code = code
        msg = error_string(code) if _lib is not None else str(code)
        super().__init__(f"{where}: {msg} (code {code})" if where else f"{msg} (code {code})")


def header_functions() -> list[str]:
    """Every ia_* function declared in include/intfadv.h."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(ia_\w+)\s*\(", text, re.M)))


def load(path: str | None = None, build_if_missing: bool = False):
    """Load the library (building it first only when asked)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or _build.LIBPATH
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        _build.build()
    L = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def error_string(code: int) -> str:
    return load().ia_error_string(int(code)).decode()


def check(code: int, where: str = "", allow=(IA_OK,)) -> int:
    if code not in allow:
        raise IAError(code, where)
    return code
