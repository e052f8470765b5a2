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


class _Fake:
    """The fields a writer reads from a TwoPhaseSimulation, on the host."""

    def __init__(self, shape, t, rng):
        D = len(shape)
        self.flow = type("F", (), {})()
        self.intf = type("I", (), {})()
        self.flow.p = torch.as_tensor(np.asfortranarray(rng.standard_normal(shape)))
        self.flow.u = torch.as_tensor(np.asfortranarray(rng.standard_normal(shape + (D,))))
        self.intf.f = torch.as_tensor(np.asfortranarray(rng.uniform(0, 1, shape)))
        self.t = t

    def sim_time(self):
        return self.t


def _load_like_reference(pvd):
    """load!(a, Val(:pvd); fname) (ext/IntfAdvReadVTKExt.jl:29-50) restated with the published ReadVTK
    conventions and nothing of this package: PVDFile(fname).vtk_filenames[end] (paths relative to the
    .pvd's directory) and .timesteps[end]; get_whole_extent(vtk)[2:2:end] with the zero extents dropped,
    +1 = the array sizes; get_data_reshaped of a point array = (ncomp, nx, ny, nz) in column-major
    order over the interleaved tuples; components_last; squeeze."""
    import os
    import xml.etree.ElementTree as ET
    root = ET.parse(pvd).getroot()
    sets = list(root.iter("DataSet"))
    t = float(sets[-1].get("timestep"))
    path = os.path.join(os.path.dirname(os.path.abspath(pvd)), sets[-1].get("file"))
    data = open(path, "rb").read()
    start = data.index(b"<AppendedData")
    head = ET.fromstring(data[:start].decode() + "</VTKFile>")
    assert head.get("type") == "ImageData" and head.get("byte_order") == "LittleEndian"
    hsz = 8 if head.get("header_type") == "UInt64" else 4
    img = head.find("ImageData")
    ext = [int(v) for v in img.get("WholeExtent").split()]
    sizes = [e + 1 for e in ext[1::2] if e != 0]
    blob = data[data.index(b"_", data.index(b">", start)) + 1:]
    out = {}
    for da in img.find("Piece").find("PointData").iter("DataArray"):
        off = int(da.get("offset"))
        n = int.from_bytes(blob[off:off + hsz], "little")
        vals = np.frombuffer(blob[off + hsz:off + hsz + n], dtype={"Float64": "<f8", "Float32": "<f4"}[da.get("type")])
        nc = int(da.get("NumberOfComponents", "1"))
        full = [n + 1 for n in ext[1::2]]                       # (nx, ny, nz) of the grid, 2D with nz = 1
        a = vals.reshape([nc] + full, order="F")                # get_data_reshaped: components first
        a = np.moveaxis(a, 0, -1)                               # components_last
        out[da.get("Name")] = np.squeeze(a, axis=tuple(k for k in range(a.ndim) if a.shape[k] == 1))
    return t, sizes, out


@pytest.mark.parametrize("shape", [(7, 5), (6, 5, 4)])
def test_collection_follows_the_reference_reader_conventions(tmp_path, monkeypatch, shape):
    # the writer's files read back exactly by the steps of the reference's load!; the collection sits
    # in a subdirectory of the working directory, so the DataSet paths must be relative to it
    monkeypatch.chdir(tmp_path)
    rng = np.random.default_rng(len(shape))
    w = vtk.VTKWriter("out/run", "out/vtk_data")
    sims = [_Fake(shape, 0.25 * (k + 1), rng) for k in range(2)]
    for s in sims:
        w.save(s)
    t, sizes, arrs = _load_like_reference("out/run.pvd")
    last = sims[-1]
    assert t == last.sim_time()
    assert sizes == list(shape)                                   # @assert extent.+1 == size(a.flow.p)
    assert set(arrs) == {"p", "f", "u"}
    assert np.array_equal(arrs["p"], last.flow.p.numpy())
    assert np.array_equal(arrs["f"], last.intf.f.numpy())
    assert arrs["u"].shape == shape + (len(shape),)
    assert np.array_equal(arrs["u"], last.flow.u.numpy())
