"""Pin the oracle against the known answers of the reference's own test suite.

Every assertion here transcribes one in InterfaceAdvection.jl's
test/maintests.jl (line numbers cited per test).  Julia indices are 1-based;
the oracle's are 0-based, so Julia ``CartesianIndex(a, b)`` is ``(a-1, b-1)``.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as O

F64 = np.float64
F32 = np.float32


def approx(a, b, T=F64):
    # Julia's default isapprox: rtol = sqrt(eps(T))
    rt = np.sqrt(np.finfo(T).eps)
    return abs(a - b) <= rt * max(abs(a), abs(b)) + (1e-30 if T == F64 else 1e-20)


# ---------------------------------------------------------------- util.jl (maintests.jl:5-23)
def test_util_helpers():
    L = O.lib()
    v = (C.c_double * 3)(1 / 2, -2 / 3, 1 / 3)
    assert L.orc_argabsmax(3, v) == 1            # myArgAbsMax(SA[1/2,-2/3,1/3]) == 2 (1-based)
    assert L.orc_get_xdir(2) == 1
    assert L.orc_get_xdir(-1) == 2
    assert L.orc_get_xdir(-2) == -1
    assert L.orc_get_xdir(1) == -2
    ix, iy = C.c_int(), C.c_int()
    for i, exp in ((3, (1, 2)), (-3, (-1, 2)), (-1, (-2, 3)), (1, (2, 3))):
        L.orc_get_xydir(i, C.byref(ix), C.byref(iy))
        assert (ix.value, iy.value) == exp


# ---------------------------------------------------------------- PLIC.jl (maintests.jl:25-51)
@pytest.mark.parametrize("T", [F32, F64])
def test_plic_intercept(T):
    gi = lambda *a: O.get_intercept(*[T(x) for x in a], dtype=T)
    assert approx(gi(2 / 3, 4 / 3, 0, 5 / 12), gi(2 / 3, 4 / 3, 5 / 12), T) and approx(gi(2 / 3, 4 / 3, 5 / 12), 8 / 9, T)
    assert approx(gi(2 / 3, 0, 4 / 3, 5 / 12), gi(2 / 3, 4 / 3, 5 / 12), T) and approx(gi(2 / 3, 0, 4 / 3, 5 / 12), 8 / 9, T)
    assert approx(gi(2 / 3, -4 / 3, 0, 5 / 12), gi(2 / 3, -4 / 3, 5 / 12), T) and approx(gi(2 / 3, -4 / 3, 5 / 12), -4 / 9, T)
    assert approx(gi(3, -4, 0, 5 / 6), gi(3, -4, 5 / 6), T) and approx(gi(3, -4, 5 / 6), 1, T)
    assert approx(gi(1 / 2, 1 / 3, 1, 7 / 12), 1, T)
    assert approx(gi(1, 1, -1, 1 - 1 / 48), 3 / 2, T)
    assert approx(gi(-7 / 6, 4 / 9, 7 / 23), gi(-7 / 6, 4 / 9, 0, 7 / 23), T)
    assert approx(gi(7 / 6, 4 / 9, -29 / 97, 7 / 23), gi(7 / 6, 4 / 9, -29 / 97, 7 / 23), T)


@pytest.mark.parametrize("T", [F32, F64])
def test_plic_volume_fraction(T):
    gv = lambda *a: O.get_volume_fraction(*[T(x) for x in a], dtype=T)
    assert approx(gv(2 / 3, 4 / 3, 0, 8 / 9), gv(2 / 3, 4 / 3, 8 / 9), T) and approx(gv(2 / 3, 4 / 3, 8 / 9), 5 / 12, T)
    assert approx(gv(2 / 3, 0, 4 / 3, 8 / 9), 5 / 12, T)
    assert approx(gv(2 / 3, -4 / 3, 0, -4 / 9), gv(2 / 3, -4 / 3, -4 / 9), T) and approx(gv(2 / 3, -4 / 3, -4 / 9), 5 / 12, T)
    assert approx(gv(3, -4, 0, 1), gv(3, -4, 1), T) and approx(gv(3, -4, 1), 5 / 6, T)
    assert approx(gv(1 / 2, 1 / 3, 1, 1), 7 / 12, T)
    assert approx(gv(1, 1, -1, 3 / 2), 1 - 1 / 48, T)
    assert approx(gv(-7 / 6, 4 / 9, 7 / 23), gv(-7 / 6, 4 / 9, 0, 7 / 23), T)


def test_plic_roundtrip_dense():
    """Forward(inverse(g)) == g over a grid of normals and fractions (FP64, tight)."""
    rng = np.random.default_rng(0)
    for _ in range(4000):
        n = rng.normal(size=3)
        g = rng.uniform(1e-6, 1 - 1e-6)
        a = O.get_intercept(*n, g)
        assert abs(O.get_volume_fraction(*n, a) - g) < 1e-11
        a2 = O.get_intercept(n[0], n[1], g)
        assert abs(O.get_volume_fraction(n[0], n[1], a2) - g) < 1e-12


# ---------------------------------------------------------------- VOFutil.jl (maintests.jl:53-137)
def test_vofutil_heights_rho_mu():
    L = O.lib()
    f = O.zeros((3, 3))
    f[1, 1] = 0.32
    f[1, 2] = 0.64
    g = O.grid(f.shape)
    Ic = O.lin(f.shape, (1, 1))
    assert 0 < f[1, 1] < 1                                                     # containInterface
    assert approx(L.orc_get3cellheight(C.byref(g), O.ptr(f), Ic, 1), 0.96)    # get3CellHeight(f,Ic,2)
    assert approx(L.orc_getrho_cell(f[1, 1], 0.7), 0.796)                     # getρ(Ic,f,0.7)
    assert approx(L.orc_getrho_face(C.byref(g), 1, Ic, O.ptr(f), 0.7), 0.748)  # getρ(2,Ic,f,0.7)

    ff = O.zeros((3, 3, 2))
    ff[2, 1, 0] = 0.1
    ff[2, 2, 0] = 0.2
    ff[1, 2, 1] = 0.3
    ff[2, 2, 1] = 0.4
    Iur = O.lin((3, 3), (2, 2))
    assert approx(L.orc_getmu(C.byref(g), 0, 0, Iur, O.ptr(ff), 0.1, 0.2, 1.0), 0.02)
    m12 = L.orc_getmu(C.byref(g), 0, 1, Iur, O.ptr(ff), 0.1, 0.2, 0.2)
    m21 = L.orc_getmu(C.byref(g), 1, 0, Iur, O.ptr(ff), 0.1, 0.2, 0.2)
    assert m12 == m21 and approx(m12, 0.028)


def test_f2face():
    fc = O.zeros((4, 4))
    fc[1:3, 1:3] = [[0.2, 0.6], [0.4, 0.8]]
    ff = O.zeros((4, 4, 2))
    O.lib().orc_f2face(C.byref(O.grid(fc.shape)), O.ptr(ff), O.ptr(fc))
    assert approx(ff[2, 2, 0], (fc[1, 2] + fc[2, 2]) / 2) and approx(ff[2, 2, 0], 0.7)
    assert approx(ff[2, 2, 1], (fc[2, 1] + fc[2, 2]) / 2) and approx(ff[2, 2, 1], 0.6)


def test_boundary_conditions():
    L = O.lib()
    rng = np.random.default_rng(1)
    g0 = np.asfortranarray(rng.random((6, 6)))
    gN = g0.copy(order="F")
    L.orc_bcf(C.byref(O.grid(gN.shape)), O.ptr(gN))
    assert (gN[0, :] == gN[1, :]).all() and (gN[-1, :] == gN[-2, :]).all()
    assert (gN[:, 0] == gN[:, 1]).all() and (gN[:, -1] == gN[:, -2]).all()
    gP = g0.copy(order="F")
    L.orc_bcf(C.byref(O.grid(gP.shape, per=(0, 1))), O.ptr(gP))
    assert (gP[0, :] == gP[-2, :]).all() and (gP[-1, :] == gP[1, :]).all()
    assert (gP[:, 0] == gP[:, -2]).all() and (gP[:, -1] == gP[:, 1]).all()

    g1 = g0.copy(order="F")
    L.orc_bcf_d(C.byref(O.grid(g1.shape)), 0, O.ptr(g1))
    assert (g1[0, 1:-1] == g0[2, 1:-1]).all()
    assert (g1[-1, 1:-1] == g0[-1, 1:-1]).all()
    assert (g1[:, 0] == g1[:, 1]).all() and (g1[:, -1] == g1[:, -2]).all()
    g1p = g0.copy(order="F")
    L.orc_bcf_d(C.byref(O.grid(g1p.shape, per=(0,))), 0, O.ptr(g1p))
    assert (g1p[0, :] == g1p[-2, :]).all() and (g1p[-1, :] == g1p[1, :]).all()

    u = np.asfortranarray(rng.random((6, 6, 2)))
    uN = u.copy(order="F")
    L.orc_bcv(C.byref(O.grid((6, 6))), O.ptr(uN))
    assert (uN[0, 1:-1, 0] == u[2, 1:-1, 0]).all()
    assert (uN[-1, 1:-1, 0] == u[-1, 1:-1, 0]).all()
    assert (uN[:, 0, 0] == uN[:, 1, 0]).all() and (uN[:, -1, 0] == uN[:, -2, 0]).all()
    assert (uN[1:-1, 0, 1] == u[1:-1, 2, 1]).all()
    assert (uN[1:-1, -1, 1] == u[1:-1, -1, 1]).all()
    assert (uN[0, :, 1] == uN[1, :, 1]).all() and (uN[-1, :, 1] == uN[-2, :, 1]).all()
    u1 = np.asfortranarray(u[:, :, 0].copy())
    L.orc_bcf_d(C.byref(O.grid((6, 6))), 0, O.ptr(u1))                         # BCv1D!(view(u,:,:,1),1)
    assert (u1 == uN[:, :, 0]).all()

    f = np.asfortranarray(rng.random((6, 6)))
    a = np.asfortranarray(rng.random((6, 6)))
    n = np.asfortranarray(rng.random((6, 6, 2)))
    a0, n0 = a.copy(), n.copy()
    L.orc_bcvof(C.byref(O.grid((6, 6))), O.ptr(f), O.ptr(a), O.ptr(n))
    assert (f[0, :] == f[1, :]).all() and (f[-1, :] == f[-2, :]).all()
    assert (a[0, :] == a0[0, :]).all() and (n[0, :, :] == n0[0, :, :]).all()
    f = np.asfortranarray(rng.random((6, 6)))
    a = np.asfortranarray(rng.random((6, 6)))
    n = np.asfortranarray(rng.random((6, 6, 2)))
    L.orc_bcvof(C.byref(O.grid((6, 6), per=(0, 1))), O.ptr(f), O.ptr(a), O.ptr(n))
    assert (f[0, :] == f[-2, :]).all() and (a[0, :] == a[-2, :]).all() and (n[0, :, :] == n[-2, :, :]).all()


def sdf_samples(shape, sdf, h=0.01):
    """SDF at cell centres (WaterLily loc(0,I) = I - 1.5, 1-based) and at ±0.01 e_d (applyVOF!)."""
    D = len(shape)
    idx = np.meshgrid(*[np.arange(n, dtype=F64) for n in shape], indexing="ij")
    xc = [c + 1 - 1.5 for c in idx]                     # 0-based index -> 1-based - 1.5
    out = [np.asfortranarray(sdf(xc))]
    for d in range(D):
        for s in (+h, -h):
            x = [xc[e] + (s if e == d else 0.0) for e in range(D)]
            out.append(np.asfortranarray(sdf(x)))
    return out


def apply_vof(shape, sdf, per=(), bc=True):
    f = np.asfortranarray(np.ones(shape))
    al = O.zeros(shape)
    nh = O.zeros(shape + (len(shape),))
    samples = sdf_samples(shape, sdf)
    arr = (C.c_void_p * len(samples))(*[s.ctypes.data for s in samples])
    g = O.grid(shape, per)
    O.lib().orc_apply_vof(C.byref(g), O.ptr(f), O.ptr(al), O.ptr(nh), arr)
    if bc:
        O.lib().orc_bcf(C.byref(g), O.ptr(f))
    return f, al, nh


def test_apply_vof_plane():
    # maintests.jl:131-136 (applyVOF! on a 2x2 interior, ghosts untouched = 0)
    shape = (4, 4)
    f = O.zeros(shape)
    al = O.zeros(shape)
    nh = O.zeros(shape + (2,))
    sdf = lambda x: (-x[0] - 3 * x[1] + 4.5) / np.sqrt(10)
    samples = sdf_samples(shape, sdf)
    arr = (C.c_void_p * len(samples))(*[s.ctypes.data for s in samples])
    O.lib().orc_apply_vof(C.byref(O.grid(shape)), O.ptr(f), O.ptr(al), O.ptr(nh), arr)
    fref = np.array([[0, 0, 0, 0], [0, 0, 2 / 3, 0], [0, 1 / 24, 23 / 24, 0], [0, 0, 0, 0]])
    assert np.allclose(f, fref, rtol=1e-8, atol=1e-12)
    # cVOF with SDF then BCf! (maintests.jl:237-240)
    f2, _, _ = apply_vof(shape, sdf)
    fref2 = np.array([[0, 0, 2 / 3, 2 / 3], [0, 0, 2 / 3, 2 / 3], [1 / 24, 1 / 24, 23 / 24, 23 / 24],
                      [1 / 24, 1 / 24, 23 / 24, 23 / 24]])
    assert np.allclose(f2, fref2, rtol=1e-8, atol=1e-12)


# ---------------------------------------------------------------- normalEstimation.jl (maintests.jl:139-156)
def test_normals_wy_myc():
    f = np.array([[5 / 12, 1, 2 / 3], [1 / 4, 11 / 12, 1 / 12], [1 / 12, 1 / 3, 0]])
    n = O.normal(f, (1, 1), "WY")
    assert approx(n[0], 1.0) and approx(n[1] + 0.5, 0.5)
    f = np.array([[0, 1 / 3, 1], [1 / 12, 11 / 12, 1], [1, 1, 1]], dtype=F64)
    n = O.normal(f, (1, 1), "WY")
    assert approx(n[0], -2 / 3) and approx(n[1], -1.0)
    f = np.array([[0, 0, 0], [0, 0.1, 0], [0, 0, 0]], dtype=F64)
    n = O.normal(f, (1, 1), "WY")
    assert n[0] == 1 and n[1] == 0
    n = O.normal(f, (1, 1), "MYC")
    assert n[0] == 0.5 and n[1] == 0.5


# ---------------------------------------------------------------- advection.jl (maintests.jl:158-180)
def test_vof_face_flux():
    L = O.lib()
    shape = (3, 3)
    f = O.zeros(shape)
    f[1, 1] = 0.32
    al = O.zeros(shape)
    al[1, 1] = -0.2
    nh = O.zeros(shape + (2,))
    nh[1, 1, :] = [1, -1]
    rhouf = O.zeros(shape + (2,))
    fF = O.zeros(shape)
    g = O.grid(shape)
    Ic = O.lin(shape, (1, 1))
    args = lambda dl, d, IF: (C.byref(g), O.ptr(fF), O.ptr(f), O.ptr(al), O.ptr(nh), dl, d, IF, O.ptr(rhouf), 0.1)
    d = 0
    L.orc_vof_flux_face(*args(-0.4, d, Ic))
    L.orc_vof_flux_face(*args(0.4, d, Ic + 1))
    assert approx(fF[1, 1], -0.24) and approx(fF[2, 1], 0.02)
    assert approx(rhouf[1, 1, 0], -0.256) and approx(rhouf[2, 1, 0], 0.058)
    d = 1
    L.orc_vof_flux_face(*args(-0.4, d, Ic))
    L.orc_vof_flux_face(*args(0.4, d, Ic + 3))
    assert approx(fF[1, 1], -0.02) and approx(fF[1, 2], 0.24)
    assert approx(rhouf[1, 1, 1], -0.058) and approx(rhouf[1, 2, 1], 0.256)


# ---------------------------------------------------------------- surfaceTension.jl (maintests.jl:182-191)
def test_popinet_heights_and_curvature():
    L = O.lib()
    f = np.asfortranarray(np.array([[0.3, 0.2, 0.1, 0.1, 0.2, 0.3, 0.0, 0.0],
                                    [1.0, 1.0, 0.6, 0.5, 0.3, 0.2, 0.0, 0.0],
                                    [0.0, 0.0, 0.0, 0.1, 0.0, 0.0, 0.0, 0.0]]))
    g = O.grid(f.shape)
    h = lambda a, b: L.orc_popinet_height(C.byref(g), O.ptr(f), O.lin(f.shape, (a - 1, b - 1)), 2)
    assert h(1, 5) == -0.3
    assert h(2, 5) == -0.9
    assert h(3, 5) == -1.4
    k = L.orc_curvature(C.byref(g), O.ptr(f), O.lin(f.shape, (1, 4)), 2)
    assert approx(k, 0.0672718547928328)
