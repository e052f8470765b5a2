"""intfadv — GB300 (sm_103a) implementation of InterfaceAdvection.jl's per-step hot path.

Host mirror of the reference's Julia API over the C-ABI library
libintfadv_gb300.so (include/intfadv.h).  All compute runs in hand-written
CUDA kernels; there is no CPU fallback.
"""
from . import _lib
from ._build import build
from .core import (Flow, Handle, advect, advect_vof_raw, advectVOF, apply_vof, applyVOF, cVOF, get_vof_flux,
                   getVOFFlux, make_config, reconstruct_interface, reconstructInterface)
from .diagnostics import metrics, sim_metrics
from .fields import cell_coords, face_coords, ffrom, fones, fzeros, is_fortran
from .levelset import LevelSet, computeL, redistaning
from .vtk import VTKWriter
from .vtk import load as load_vtk
from .simulation import (MPCFL, MPFMomStep, NoBody, TwoPhaseSimulation, poisson_stats, set_learned, set_momentum_arith, set_poisson_coef16, set_poisson_slab_rows, set_smoother, sim_info,
                         sim_step, surfTen)

__all__ = ["Flow", "Handle", "advect", "advect_vof_raw", "advectVOF", "apply_vof", "applyVOF", "cVOF",
           "get_vof_flux", "getVOFFlux", "make_config", "reconstruct_interface", "reconstructInterface", "build",
           "cell_coords", "face_coords", "ffrom", "fones", "fzeros", "is_fortran", "MPCFL", "MPFMomStep", "NoBody",
           "TwoPhaseSimulation", "sim_info", "sim_step", "surfTen", "poisson_stats", "set_learned", "set_momentum_arith", "set_poisson_coef16", "set_poisson_slab_rows", "set_smoother", "metrics", "sim_metrics", "LevelSet", "redistaning",
           "computeL", "VTKWriter", "load_vtk"]
