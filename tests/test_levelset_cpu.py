"""Level-set reinitialisation oracle pinned on the reference's own tests
(test/maintests.jl:264-319, redistaning.jl testset)."""
import numpy as np

from oracle import pyoracle as O


def F(a):
    return np.asfortranarray(a, dtype=np.float64)


def test_rhs_vanishes_on_a_distance_ramp():
    # maintests.jl:267-279: ϕ = i - 2.5 - 8 (1-based i) on 18x18, Neumann and periodic in y
    phi = F(np.fromfunction(lambda i, j: (i + 1) - 2.5 - 8, (18, 18)))
    for per in ((), (1,)):
        L = O.levelset_rhs(phi, phi.copy(order="F"), per=per)
        assert np.abs(L[1:-1, 1:-1]).max() < 1e-12


def test_rk_stages_on_a_diagonal_plane():
    # maintests.jl:281-295: three stages on ϕ = i + j (6x6) with ϕ_ini aliasing ϕ
    phid = F(np.fromfunction(lambda i, j: (i + 1) + (j + 1), (6, 6)))
    phi0 = phid.copy(order="F")
    L = F(np.zeros((6, 6)))
    dtau = 0.01
    for a in (0.0, 0.75, 1 / 3):
        O.levelset_stage(phid, phi0, phid, L, dtau, a)
    assert np.abs(phid[1:-1, 1:-1] - (phi0[1:-1, 1:-1] + dtau * (1 - np.sqrt(2)))).max() < 0.05


def planar_f(n=16, x_if=8.0):
    # cVOF of InterfaceSDF x - 8 on 16x16 (dark fluid x < 8): the interface is a cell face,
    # cells with centre c - 0.5 < 8 are full; ghosts by BCf! (Neumann in x, periodic in y)
    f = np.zeros((n + 2, n + 2))
    for c in range(1, n + 1):
        f[c, 1:-1] = 1.0 if c - 0.5 < x_if else 0.0
    f = F(f)
    O.lib().orc_bcf(O.C.byref(O.grid(f.shape, (1,))), O.ptr(f))
    return f


def test_planar_interface_reinitialises_to_distance():
    # maintests.jl:305-317
    phi = O.redistance(planar_f(), d=4.0, dtau=0.05, per=(1,))
    assert np.isfinite(phi).all()
    col = phi[1:-1, 8]
    assert np.all(np.diff(col) <= 0)
    assert np.array_equal(phi[:, 0], phi[:, -2]) and np.array_equal(phi[:, -1], phi[:, 1])
    for ix in range(8, 12):                 # 1-based ix of the reference
        assert abs(phi[ix - 1, 8] - (-(ix - 1.5 - 8))) <= 0.01
