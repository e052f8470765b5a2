"""VTK collection output and restart (load!(sim, Val(:pvd)), ext/IntfAdvReadVTKExt.jl:29-50)."""
import numpy as np
import pytest
import torch

from intfadv import vtk


def test_vti_round_trip_cpu(tmp_path):
    rng = np.random.default_rng(0)
    shape = (6, 5, 4)
    p = np.asfortranarray(rng.standard_normal(shape))
    u = np.asfortranarray(rng.standard_normal(shape + (3,)))
    path = str(tmp_path / "a.vti")
    vtk.write_vti(path, {"p": (p, 1), "u": (u, 3)}, shape)
    dims, arrs = vtk.read_vti(path)
    assert dims == shape
    assert np.array_equal(arrs["p"][0].reshape(shape, order="F"), p)
    uv, nc = arrs["u"]
    assert nc == 3
    # VTK tuple order: the 3 components of point 0 first
    assert np.array_equal(uv[:3], u[0, 0, 0, :])
    assert np.array_equal(uv.reshape((-1, 3)).reshape(shape + (3,), order="F"), u)


@pytest.mark.gpu
def test_restart_continues_the_run(cuda, tmp_path, monkeypatch):
    import intfadv as ia
    monkeypatch.chdir(tmp_path)
    N = 16

    def make():
        sdf = lambda x: torch.sqrt((x[0] - 8) ** 2 + (x[1] - 7) ** 2) - 4
        return ia.TwoPhaseSimulation((N, N), (0.0, 0.0), float(N), U=1.0, InterfaceSDF=sdf, g=(0.0, -0.01),
                                     ν=0.01, λρ=1e-2, perdir=(0,), poisson_tol=1e-12, poisson_itmx=500)

    a = make()
    for _ in range(3):
        ia.sim_step(a)
    w = ia.VTKWriter("run", "vtk_data")
    w.save(a)
    b = make()
    w2 = ia.load_vtk(b, "run.pvd")
    assert torch.equal(a.flow.u, b.flow.u) and torch.equal(a.intf.f, b.intf.f) and torch.equal(a.flow.p, b.flow.p)
    assert abs(b.sim_time() - a.sim_time()) < 1e-12 * a.sim_time()
    # the restarted run continues (the split-direction order follows len(Δt), as in the reference,
    # so it is not the continuous run's sequence)
    m0 = b.intf.mass()
    for _ in range(2):
        st = ia.sim_step(b)
        assert st.code == 0
    assert bool(torch.isfinite(b.flow.u).all()) and abs(b.intf.mass() - m0) <= 1e-12 * m0
    w2.save(b)
    assert w2.k == 2 and len(vtk.read_pvd("run.pvd")) == 2
