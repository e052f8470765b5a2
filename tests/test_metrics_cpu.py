"""Diagnostics of src/metrics.jl: the oracle's per-cell functions pinned on the reference's own
known answers (test/maintests.jl:321-347)."""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as O


def zeros(*shape):
    return np.zeros(shape, order="F")


@pytest.fixture(scope="module")
def case2d():
    # test/maintests.jl:324-328 (1-based indices there, 0-based here)
    u = zeros(4, 4, 2)
    u[1, 1, 0] = 1
    u[2, 1, 0] = 2
    u[1, 1, 1] = 3
    u[1, 2, 1] = 4
    f = zeros(4, 4)
    f[1, 1] = 0.5
    return u, f, O.grid((4, 4)), 1 + 4 * 1


def vec(*v):
    a = np.zeros(3)
    a[:len(v)] = v
    return a.ctypes.data, a


def test_rhoke_rhou_rhogh_known_answers(case2d):
    u, f, g, I = case2d
    L = O.lib()
    z, _z = vec(0.0, 0.0)
    one, _o = vec(1.0, 1.0)
    assert L.orc_rhoke(C.byref(g), I, O.ptr(u), O.ptr(f), 0.2, z) == pytest.approx(4.5)
    assert L.orc_rhoke(C.byref(g), I, O.ptr(u), O.ptr(f), 0.2, one) == pytest.approx(2.1)
    assert L.orc_rhou(C.byref(g), 0, I, O.ptr(u), O.ptr(f), 0.2, z) == pytest.approx(0.9)
    assert L.orc_rhou(C.byref(g), 1, I, O.ptr(u), O.ptr(f), 0.2, z) == pytest.approx(2.1)
    assert L.orc_rhou(C.byref(g), 0, I, O.ptr(u), O.ptr(f), 0.2, one) == pytest.approx(0.3)
    gv, _g = vec(0.0, -1.0)
    assert L.orc_rhogh(C.byref(g), I, gv, O.ptr(f), 0.2, z) == pytest.approx(0.3)


def test_enstrophy_known_answers():
    L = O.lib()
    w = zeros(4, 4)
    w[1, 1], w[2, 1], w[1, 2], w[2, 2] = 1, 2, 3, 4
    assert L.orc_ens(C.byref(O.grid((4, 4))), 1 + 4, O.ptr(w)) == pytest.approx(3.75)
    w3 = zeros(4, 4, 4, 3)
    for (x, y, z, i), v in {(1, 1, 1, 0): 1, (1, 2, 1, 0): 2, (1, 1, 2, 0): 3, (1, 2, 2, 0): 4,
                            (1, 1, 1, 1): 1, (1, 1, 2, 1): 2, (2, 1, 1, 1): 3, (2, 1, 2, 1): 4,
                            (1, 1, 1, 2): 1, (2, 1, 1, 2): 2, (1, 2, 1, 2): 3, (2, 2, 1, 2): 4}.items():
        w3[x, y, z, i] = v
    assert L.orc_ens(C.byref(O.grid((4, 4, 4))), 1 + 4 + 16, O.ptr(w3)) == pytest.approx(11.25)


def test_domain_sums_add_the_cells():
    rng = np.random.default_rng(0)
    u = np.asfortranarray(rng.standard_normal((6, 5, 2)))
    f = np.asfortranarray(rng.uniform(0, 1, (6, 5)))
    m = O.metrics(u, f, 0.1, U=(0.2, -0.1), g=(0.0, -1.0), statwl=(0.0, 1.5), omega=np.asfortranarray(f * 2))
    g = O.grid((6, 5))
    L = O.lib()
    U, _U = vec(0.2, -0.1)
    ke = sum(L.orc_rhoke(C.byref(g), x + 6 * y, O.ptr(u), O.ptr(f), 0.1, U) for x in range(1, 5) for y in range(1, 4))
    assert m["ke"] == pytest.approx(ke, rel=1e-14)
