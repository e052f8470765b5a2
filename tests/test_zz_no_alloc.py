"""The allocation-free advect! entry point (ia_advect_vof_noalloc).

It serves callers that cannot let a library allocate device memory while they
run (a host framework that has reserved the device memory for its own pool, or
a time loop that forbids cudaMalloc/cudaFree after set-up).  This file checks,
through the C-ABI, that two calls in a row give the same fractions, c̄, mass
fluxes and fill status as the handle-based ia_advect_vof (3D and 2D, and with a
time step large enough to over- and under-fill cells), that the shared scratch
is cleared between calls (the second call starts from the first call's
leftovers), that a call after the first takes no device memory, and that a grid
above the fixed scratch size or an exitBC configuration is refused.  It runs
last and also passes on its own in a fresh process.
"""
import ctypes as C
import math

import numpy as np
import pytest
import torch

import intfadv as ia
from intfadv import _lib, workloads
from intfadv.fields import fzeros, ptr

pytestmark = pytest.mark.gpu
TOL = 1e-10


def npf(t):
    return np.asfortranarray(t.detach().cpu().numpy())


def vortex_2d(N):
    """Discretely divergence-free 2D single vortex on the faces of an N² grid (grid units):
    the differences of the node stream function ψ = sin²(πx) sin²(πy)/π."""
    h, ng = 1.0 / N, N + 2
    xf = (torch.arange(ng + 1, device="cuda", dtype=torch.float64) - 1) * h
    S = torch.sin(math.pi * xf) ** 2
    psi = S[:, None] * S[None, :] / math.pi          # [x node, y node]
    U = fzeros((ng, ng, 2))
    U[..., 0].copy_((psi[:ng, 1:] - psi[:ng, :ng]) / (h * h))
    U[..., 1].copy_(-(psi[1:, :ng] - psi[:ng, :ng]) / (h * h))
    return U


def noalloc_call(lib, cfg, f, u1, u2, dt, n_dt, cbar, rhouf):
    st = _lib.Status()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.ia_advect_vof_noalloc(C.byref(cfg), stream, ptr(f), ptr(u1), ptr(u2), C.c_double(dt),
                                   C.c_int64(n_dt), ptr(cbar), ptr(rhouf), C.byref(st))
    torch.cuda.synchronize()
    return rc, st


def check_same(rc, st, st_ref, f, cbar, rhouf, ref):
    assert rc == st_ref.code
    assert st.flags == st_ref.flags and st.code == st_ref.code
    if st.flags & _lib.FLAG_OVERFILL:
        assert st.maxf == st_ref.maxf and st.maxid == st_ref.maxid and st.fill_dir == st_ref.fill_dir
    if st.flags & _lib.FLAG_UNDERFILL:
        assert st.minf == st_ref.minf and st.minid == st_ref.minid and st.fill_dir == st_ref.fill_dir
    close(npf(f), npf(ref.f), TOL)
    assert (npf(cbar) == npf(ref.cbar)).all()
    close(npf(rhouf), npf(ref.rhouf), TOL * max(1.0, float(np.nanmax(np.abs(npf(ref.rhouf))))))


def close(a, b, tol):
    # NaNs (an over-driven step may produce them) must sit at the same places on both paths
    assert (np.isnan(a) == np.isnan(b)).all()
    m = ~np.isnan(a)
    assert not m.any() or np.abs(a[m] - b[m]).max() < tol


def run_pair(lib, dims, sdf, U, dt):
    ref = ia.cVOF(dims, InterfaceSDF=sdf)                       # handle-based path
    f = ref.f.clone()
    cbar = torch.zeros_like(ref.cbar)
    rhouf = torch.zeros_like(ref.rhouf)
    cfg = ia.make_config(dims, lrho=ref.lrho)
    codes = []
    for step in (1, 2):
        st_ref = ia.advect_vof_raw(ref, ref.f, U, U, dt, step)
        rc, st = noalloc_call(lib, cfg, f, U, U, dt, step, cbar, rhouf)
        check_same(rc, st, st_ref, f, cbar, rhouf, ref)
        codes.append(rc)
    return codes


def test_noalloc_matches_handle_path_twice(cuda, lib):
    N = 32
    sdf = workloads.sphere_sdf((0.35, 0.35, 0.35), 0.15, N)
    ref = ia.cVOF((N, N, N), InterfaceSDF=sdf)
    f = ref.f.clone()
    cbar = torch.zeros_like(ref.cbar)
    rhouf = torch.zeros_like(ref.rhouf)
    cfg = ia.make_config((N, N, N), lrho=ref.lrho)
    U = workloads.deformation_field(N)
    dt = 1.0 / (4 * N)
    for step in (1, 2):
        u1 = U * workloads.deformation_time_factor((step - 1) * dt)
        u2 = U * workloads.deformation_time_factor(step * dt)
        st_ref = ia.advect_vof_raw(ref, ref.f, u1, u2, dt, step)
        rc, st = noalloc_call(lib, cfg, f, u1, u2, dt, step, cbar, rhouf)
        assert rc == 0
        check_same(rc, st, st_ref, f, cbar, rhouf, ref)


def test_noalloc_2d_matches_handle_path_twice(cuda, lib):
    N = 48
    sdf = lambda x: torch.sqrt((x[0] - 0.5 * N) ** 2 + (x[1] - 0.75 * N) ** 2) - 0.15 * N
    codes = run_pair(lib, (N, N), sdf, vortex_2d(N), 1.0 / (2 * N))
    assert codes == [0, 0]


def test_noalloc_fill_status_matches_handle_path(cuda, lib):
    # a time step far above the CFL limit over- and under-fills cells; both paths must report the same
    # extremes, cells and direction (the status translation is shared, the device status is the array's)
    N = 24
    sdf = workloads.sphere_sdf((0.5, 0.5, 0.5), 0.25, N)
    U = workloads.deformation_field(N)
    codes = run_pair(lib, (N, N, N), sdf, U, 0.75 / N)           # sweeps of up to 1.5 cells
    assert _lib.IA_WARN_FILL in codes or _lib.IA_ERR_NAN in codes


def test_noalloc_call_takes_no_device_memory(cuda, lib):
    N = 32
    ref = ia.cVOF((N, N, N), InterfaceSDF=workloads.sphere_sdf((0.35, 0.35, 0.35), 0.15, N))
    f, cbar, rhouf = ref.f.clone(), torch.zeros_like(ref.cbar), torch.zeros_like(ref.rhouf)
    cfg = ia.make_config((N, N, N), lrho=ref.lrho)
    U = workloads.deformation_field(N)
    dt = 1.0 / (4 * N)
    noalloc_call(lib, cfg, f, U, U, dt, 1, cbar, rhouf)          # first call: kernels load, address lookup
    free0 = torch.cuda.mem_get_info()[0]
    for step in (2, 3):
        rc, _ = noalloc_call(lib, cfg, f, U, U, dt, step, cbar, rhouf)
        assert rc == 0
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_grid_beyond_scratch_and_exit_bc(cuda, lib):
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    d8 = torch.zeros(8, dtype=torch.int8, device="cuda")
    p = C.c_void_p(dummy.data_ptr())
    for cfg, want in ((ia.make_config((128, 128, 128)), _lib.IA_ERR_TOO_LARGE),   # 130^3 > IA_NOALLOC_MAX_CELLS
                      (ia.make_config((16, 16, 16), exitBC=True), _lib.IA_ERR_UNSUPPORTED)):
        st = _lib.Status()
        rc = lib.ia_advect_vof_noalloc(C.byref(cfg), None, p, p, p, C.c_double(0.1), C.c_int64(1),
                                       C.c_void_p(d8.data_ptr()), None, C.byref(st))
        assert rc == want
