"""GPU parity of the VOF path (advect!, reconstructInterface!, getVOFFlux!, applyVOF!)
against the CPU oracle, through the C-ABI.

Tolerance: fractions and mass fluxes within 1e-10 (absolute on f ∈ [0,1],
relative to max|ρuf| for the mass flux), c̄ exact.
"""
import math

import numpy as np
import pytest
import torch

import intfadv as ia
from intfadv import _lib, workloads
from intfadv.fields import ffrom, fzeros
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-10
SCHEMES = ["WH", "WY", "MYC", "Y", "Column", "PCD", "SLIC", "CD"]


def npf(t):
    return np.asfortranarray(t.detach().cpu().numpy())


def sphere(N, c=(0.35, 0.35, 0.35), r=0.15):
    return workloads.sphere_sdf(c, r, N)


def circle2d(N, c=(0.5, 0.5), r=0.25):
    cN, rN = [x * N for x in c], r * N
    return lambda x: torch.sqrt((x[0] - cN[0]) ** 2 + (x[1] - cN[1]) ** 2) - rN


def random_velocity(shape_ng, D, cfl, seed, device="cuda"):
    """Smooth random face velocity with max|u| * 1 = cfl (grid units, dt = 1)."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    Nv = tuple(shape_ng) + (D,)
    u = fzeros(Nv, torch.float64, device)
    coords = [torch.arange(n, dtype=torch.float64) for n in shape_ng]
    grids = torch.meshgrid(*coords, indexing="ij")
    for d in range(D):
        acc = torch.zeros(shape_ng, dtype=torch.float64)
        for _ in range(3):
            k = torch.randint(1, 3, (D,), generator=g).double()
            ph = torch.rand(D, generator=g).double() * 2 * math.pi
            term = torch.ones(shape_ng, dtype=torch.float64)
            for e in range(D):
                term = term * torch.sin(2 * math.pi * k[e] * grids[e] / shape_ng[e] + ph[e])
            acc += term
        acc = acc / acc.abs().max() * cfl
        u[..., d].copy_(acc)
    return u


def oracle_grid_state(intf):
    return npf(intf.f)


# ------------------------------------------------------------------------------------- applyVOF!
def test_apply_vof_plane_reference_values(cuda):
    # maintests.jl:237-240: cVOF((2,2); InterfaceSDF) with Neumann ghosts
    sdf = lambda x: (-x[0] - 3 * x[1] + 4.5) / math.sqrt(10)
    intf = ia.cVOF((2, 2), InterfaceSDF=sdf)
    fref = np.array([[0, 0, 2 / 3, 2 / 3], [0, 0, 2 / 3, 2 / 3], [1 / 24, 1 / 24, 23 / 24, 23 / 24],
                     [1 / 24, 1 / 24, 23 / 24, 23 / 24]])
    assert np.allclose(npf(intf.f), fref, rtol=1e-8, atol=1e-12)


def test_cvof_defaults(cuda):
    # maintests.jl:221-233
    intf = ia.cVOF((4, 4))
    assert (npf(intf.f) == 1).all() and (npf(intf.alpha) == 0).all() and (npf(intf.nhat) == 0).all()
    assert intf.perdir == ()
    i0 = ia.cVOF((4, 4), mu=0.0, eta=0.0)
    assert i0.mu is None and i0.eta is None
    i1 = ia.cVOF((4, 4), mu=0.5, lmu=0.2, lrho=0.3, eta=1.5)
    assert (i1.mu, i1.lmu, i1.lrho, i1.eta) == (0.5, 0.2, 0.3, 1.5)


@pytest.mark.parametrize("D", [2, 3])
def test_apply_vof_matches_oracle(cuda, D):
    from test_oracle_golden import apply_vof as oracle_apply
    N = (20,) * D
    sdf = sphere(20) if D == 3 else circle2d(20)
    intf = ia.cVOF(N, InterfaceSDF=sdf)

    def sdf_np(x):
        return sdf([torch.as_tensor(v) for v in x]).numpy()

    f, al, nh = oracle_apply(tuple(n + 2 for n in N), sdf_np)
    inner = tuple(slice(1, -1) for _ in range(D))
    assert np.abs(npf(intf.f) - f).max() < TOL
    assert np.abs(npf(intf.alpha)[inner] - al[inner]).max() < TOL
    assert np.abs(npf(intf.nhat)[inner] - nh[inner]).max() < TOL


# ---------------------------------------------------------------------------- reconstruction
def perturbed_field(N, D, seed=0, steps=2):
    """A generic interface field: a sphere/circle advected a few steps by the oracle."""
    sdf = sphere(N) if D == 3 else circle2d(N)
    intf = ia.cVOF((N,) * D, InterfaceSDF=sdf)
    f = npf(intf.f)
    u = npf(random_velocity(intf.Ng, D, 0.4, seed))
    for s in range(steps):
        O.advect_vof(f, u, u, 1.0, O.dir_order(s + 1, D))
    return f


@pytest.mark.parametrize("scheme", SCHEMES + ["XYLIC"])
@pytest.mark.parametrize("D", [2, 3])
def test_reconstruct_matches_oracle(cuda, scheme, D):
    f = perturbed_field(18, D)
    al_o, nh_o = O.reconstruct(f.copy(order="F"), scheme)
    intf = ia.cVOF((18,) * D, normalScheme=scheme)
    fd = ffrom(f)
    al = fzeros(fd.shape)
    nh = fzeros(tuple(fd.shape) + (D,))
    ia.reconstruct_interface(intf, fd, al, nh)
    assert np.abs(npf(al) - al_o).max() < TOL
    assert np.abs(npf(nh) - nh_o).max() < TOL


@pytest.mark.parametrize("D", [2, 3])
def test_vof_flux_matches_oracle(cuda, D):
    f = perturbed_field(16, D, seed=3)
    al, nh = O.reconstruct(f.copy(order="F"), "WH")
    u = random_velocity(f.shape, D, 0.45, 7)
    un = npf(u)
    intf = ia.cVOF((16,) * D)
    for d in range(D):
        fF_o = O.zeros(f.shape)
        ruf_o = O.zeros(f.shape + (D,))
        O.lib().orc_vof_flux(O.C.byref(O.grid(f.shape)), O.ptr(fF_o), O.ptr(f), O.ptr(al), O.ptr(nh), O.ptr(un),
                             O.ptr(un), 0.9, d, O.ptr(ruf_o), 1e-3)
        fF = fzeros(f.shape)
        ruf = fzeros(f.shape + (D,))
        ia.get_vof_flux(intf, fF, ffrom(f), ffrom(al), ffrom(nh), u, u, 0.9, d, ruf)
        assert np.abs(npf(fF) - fF_o).max() < TOL
        assert np.abs(npf(ruf) - ruf_o).max() < TOL


# --------------------------------------------------------------------------------- advect!
def run_pair(intf, f0, u1, u2, dt, steps, D, per=(), scheme="WH", lrho=1e-3, scale=None):
    """Advance GPU and oracle side by side; returns max errors per quantity."""
    fo = npf(f0)
    errs = {"f": 0.0, "rhouf": 0.0, "cbar": 0}
    for s in range(1, steps + 1):
        a = 1.0 if scale is None else scale(s)
        b = 1.0 if scale is None else scale(s + 1)
        v1 = u1 * a
        v2 = u2 * b
        st = ia.advect_vof_raw(intf, intf.f, v1, v2, dt, s)
        ost, cbar, rhouf, *_ = O.advect_vof(fo, npf(v1), npf(v2), dt, O.dir_order(s, D), lrho=lrho,
                                            scheme=scheme, per=per)
        assert (st.flags & 7) == ((1 if ost.nan else 0) | (2 if ost.over else 0) | (4 if ost.under else 0))
        errs["f"] = max(errs["f"], float(np.abs(npf(intf.f) - fo).max()))
        scale_r = max(1.0, float(np.abs(rhouf).max()))
        errs["rhouf"] = max(errs["rhouf"], float(np.abs(npf(intf.rhouf) - rhouf).max()) / scale_r)
        errs["cbar"] = max(errs["cbar"], int(np.abs(npf(intf.cbar).astype(int) - cbar.astype(int)).max()))
    return errs


@pytest.mark.parametrize("scheme", SCHEMES)
def test_advect_sphere_deformation_matches_oracle(cuda, scheme):
    N = 32
    intf = ia.cVOF((N, N, N), InterfaceSDF=sphere(N), normalScheme=scheme)
    U = workloads.deformation_field(N)
    dt = 1.0 / (4 * N)
    errs = run_pair(intf, intf.f, U, U, dt, 4, 3, scheme=scheme,
                    scale=lambda s: workloads.deformation_time_factor((s - 1) * dt))
    assert errs["f"] < TOL and errs["rhouf"] < TOL and errs["cbar"] == 0, errs


@pytest.mark.parametrize("per", [(0, 1), (0,), (1,)])
def test_advect_2d_periodicity_matches_oracle(cuda, per):
    N = 32
    intf = ia.cVOF((N, N), InterfaceSDF=circle2d(N, c=(0.3, 0.6)), perdir=per)
    u = random_velocity(intf.Ng, 2, 0.45, 11)
    errs = run_pair(intf, intf.f, u, u, 1.0, 5, 2, per=per)
    assert errs["f"] < TOL and errs["rhouf"] < TOL and errs["cbar"] == 0, errs


def test_advect_3d_mixed_periodicity_matches_oracle(cuda):
    N = 24
    per = (0, 2)
    intf = ia.cVOF((N, N, N), InterfaceSDF=sphere(N, c=(0.1, 0.5, 0.9), r=0.2), perdir=per)
    u = random_velocity(intf.Ng, 3, 0.4, 5)
    u2 = random_velocity(intf.Ng, 3, 0.4, 6)
    errs = run_pair(intf, intf.f, u, u2, 1.0, 4, 3, per=per)
    assert errs["f"] < TOL and errs["rhouf"] < TOL and errs["cbar"] == 0, errs


def test_advect_beyond_fast_path_bound_matches_oracle(cuda):
    # |u| dt up to 0.9 > 1/2: bulk cells leave the integer fast path and take the list pass
    N = 20
    intf = ia.cVOF((N, N, N), InterfaceSDF=sphere(N, c=(0.5, 0.5, 0.5), r=0.3))
    u = random_velocity(intf.Ng, 3, 0.9, 21)
    errs = run_pair(intf, intf.f, u, u, 1.0, 2, 3)
    assert errs["f"] < TOL and errs["rhouf"] < TOL, errs


def test_full_domain_stays_full(cuda):
    # all dark, c̄ = 1, arbitrary velocity: the fraction stays exactly 1 (fast path)
    intf = ia.cVOF((16, 16, 16))
    u = random_velocity(intf.Ng, 3, 0.45, 2)
    st = ia.advect_vof_raw(intf, intf.f, u, u, 1.0, 1)
    assert st.code == 0
    assert (npf(intf.f) == 1.0).all()


def test_mass_conservation_and_bounds(cuda):
    N = 48
    intf = ia.cVOF((N, N, N), InterfaceSDF=sphere(N))
    U = workloads.deformation_field(N)
    dt = 1.0 / (4 * N)
    m0 = intf.mass()
    f0 = npf(intf.f)
    assert abs(m0 - f0[1:-1, 1:-1, 1:-1].sum()) < 1e-9 * m0
    v_prev = U * workloads.deformation_time_factor(0.0)
    for s in range(1, 41):
        v_next = U * workloads.deformation_time_factor(s * dt)
        st = ia.advect_vof_raw(intf, intf.f, v_prev, v_next, dt, s)
        assert st.code in (0, _lib.IA_WARN_FILL)
        v_prev = v_next
    f = npf(intf.f)
    assert f.min() >= 0.0 and f.max() <= 1.0
    assert abs(intf.mass() - m0) / m0 < 1e-12


def test_nan_is_reported(cuda):
    intf = ia.cVOF((12, 12, 12), InterfaceSDF=sphere(12, c=(0.5, 0.5, 0.5), r=0.3))
    f = intf.f.clone()
    f_np = npf(intf.f)
    f_np[6, 6, 6] = np.nan
    intf.f.copy_(torch.as_tensor(f_np))
    u = random_velocity(intf.Ng, 3, 0.3, 1)
    with pytest.raises(FloatingPointError, match="NaN"):
        ia.advect(ia.Flow((12, 12, 12), (0, 0, 0)), intf, u1=u, u2=u, dt=1.0)
    del f


def test_overfill_status_matches_oracle(cuda):
    # a converging (non-solenoidal) field over-fills dark cells; status flags agree with the oracle
    N = 16
    intf = ia.cVOF((N, N, N), InterfaceSDF=sphere(N, c=(0.5, 0.5, 0.5), r=0.25))
    ng = intf.Ng
    u = fzeros(ng + (3,))
    for d in range(3):
        x = torch.arange(ng[d], dtype=torch.float64, device="cuda") - 1 - N / 2
        shape = [1, 1, 1]
        shape[d] = ng[d]
        u[..., d].copy_((-0.04 * x).view(*shape).expand(*ng))
    fo = npf(intf.f)
    st = ia.advect_vof_raw(intf, intf.f, u, u, 1.0, 1)
    ost, *_ = O.advect_vof(fo, npf(u), npf(u), 1.0, O.dir_order(1, 3))
    assert bool(st.flags & _lib.FLAG_OVERFILL) == bool(ost.over)
    assert bool(st.flags & _lib.FLAG_UNDERFILL) == bool(ost.under)
    assert np.abs(npf(intf.f) - fo).max() < TOL
