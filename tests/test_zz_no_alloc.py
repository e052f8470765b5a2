"""The allocation-free advect! entry point (ia_advect_vof_noalloc).

It serves callers that cannot let a library allocate device memory while they
run (a host framework that has reserved the device memory for its own pool, or
a time loop that forbids cudaMalloc/cudaFree after set-up).  This file checks,
through the C-ABI, that two calls in a row give the same fractions, c̄ and
mass fluxes as the handle-based ia_advect_vof, that the shared scratch is
cleared between calls (the second call starts from the first call's leftovers),
and that a grid above the fixed scratch size is refused.  It runs last and
also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import intfadv as ia
from intfadv import _lib, workloads
from intfadv.fields import ptr

pytestmark = pytest.mark.gpu
TOL = 1e-10


def npf(t):
    return np.asfortranarray(t.detach().cpu().numpy())


def test_noalloc_matches_handle_path_twice(cuda, lib):
    N = 32
    sdf = workloads.sphere_sdf((0.35, 0.35, 0.35), 0.15, N)
    ref = ia.cVOF((N, N, N), InterfaceSDF=sdf)                 # handle-based path
    f = ref.f.clone()
    cbar = torch.zeros_like(ref.cbar)
    rhouf = torch.zeros_like(ref.rhouf)
    cfg = ia.make_config((N, N, N), lrho=ref.lrho)
    U = workloads.deformation_field(N)
    dt = 1.0 / (4 * N)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for step in (1, 2):
        u1 = U * workloads.deformation_time_factor((step - 1) * dt)
        u2 = U * workloads.deformation_time_factor(step * dt)
        st_ref = ia.advect_vof_raw(ref, ref.f, u1, u2, dt, step)
        st = _lib.Status()
        rc = lib.ia_advect_vof_noalloc(C.byref(cfg), stream, ptr(f), ptr(u1), ptr(u2), C.c_double(dt),
                                       C.c_int64(step), ptr(cbar), ptr(rhouf), C.byref(st))
        torch.cuda.synchronize()
        assert rc == st_ref.code == 0
        assert st.flags == st_ref.flags
        assert np.abs(npf(f) - npf(ref.f)).max() < TOL
        assert (npf(cbar) == npf(ref.cbar)).all()
        scale = max(1.0, float(ref.rhouf.abs().max()))
        assert np.abs(npf(rhouf) - npf(ref.rhouf)).max() < TOL * scale


def test_noalloc_rejects_grid_beyond_scratch(cuda, lib):
    cfg = ia.make_config((128, 128, 128))                      # 130^3 cells > IA_NOALLOC_MAX_CELLS
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    d8 = torch.zeros(8, dtype=torch.int8, device="cuda")
    st = _lib.Status()
    rc = lib.ia_advect_vof_noalloc(C.byref(cfg), None, C.c_void_p(dummy.data_ptr()), C.c_void_p(dummy.data_ptr()),
                                   C.c_void_p(dummy.data_ptr()), C.c_double(0.1), C.c_int64(1),
                                   C.c_void_p(d8.data_ptr()), None, C.byref(st))
    assert rc == _lib.IA_ERR_TOO_LARGE
