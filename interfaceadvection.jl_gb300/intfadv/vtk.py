"""VTK output and restart — host mirror of the reference's checkpoint path: WaterLily's vtkWriter
collection (a .pvd file listing .vti ImageData files) and ``load!(sim, Val(:pvd); fname)``
(ext/IntfAdvReadVTKExt.jl:29-50).

Each .vti holds point data over the whole ghost-inclusive grid, as the reference writes it: the
pressure ``p``, the fraction ``f`` and the velocity ``u`` (components first), FP64, in appended raw
binary with UInt64 block headers.  ``load`` reads the last file of a collection back into a
TwoPhaseSimulation and resets the time step like the reference (Δt[end] = t·L/U, then a new CFL
entry).  This is host I/O around the device fields; no kernel is involved.
"""
from __future__ import annotations

import os
import xml.etree.ElementTree as ET

import numpy as np
import torch

from .fields import ffrom

_VTK_TYPES = {"Float64": np.float64, "Float32": np.float32, "Int32": np.int32, "Int64": np.int64,
              "UInt8": np.uint8}


def _host(t: torch.Tensor) -> np.ndarray:
    return np.asfortranarray(t.detach().cpu().numpy())


def write_vti(path: str, arrays: dict, shape) -> None:
    """ImageData file with point arrays (name -> (array in Fortran order, components))."""
    ext = " ".join(f"0 {n - 1}" for n in shape) + (" 0 0" if len(shape) == 2 else "")
    header, blobs, offset = [], [], 0
    for name, (a, ncomp) in arrays.items():
        # VTK tuples: the components of a point together, points x fastest
        flat = a.reshape((-1, ncomp), order="F").reshape(-1)
        raw = np.ascontiguousarray(flat, dtype=np.float64).tobytes()
        header.append(f'        <DataArray type="Float64" Name="{name}" NumberOfComponents="{ncomp}" '
                      f'format="appended" offset="{offset}"/>')
        blob = np.uint64(len(raw)).tobytes() + raw
        blobs.append(blob)
        offset += len(blob)
    xml = ('<?xml version="1.0" encoding="utf-8"?>\n'
           '<VTKFile type="ImageData" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n'
           f'  <ImageData WholeExtent="{ext}" Origin="0 0 0" Spacing="1 1 1">\n'
           f'    <Piece Extent="{ext}">\n      <PointData>\n' + "\n".join(header) +
           '\n      </PointData>\n    </Piece>\n  </ImageData>\n  <AppendedData encoding="raw">\n   _')
    with open(path, "wb") as fh:
        fh.write(xml.encode())
        for b in blobs:
            fh.write(b)
        fh.write(b"\n  </AppendedData>\n</VTKFile>\n")


def read_vti(path: str):
    """Point arrays of an ImageData file written with appended raw data -> (dims, {name: array})."""
    data = open(path, "rb").read()
    start = data.index(b"<AppendedData")
    us = data.index(b"_", data.index(b">", start)) + 1
    root = ET.fromstring(data[:start].decode() + "</VTKFile>")
    img = root.find("ImageData")
    ext = [int(v) for v in img.get("WholeExtent").split()]
    dims = tuple(ext[2 * k + 1] - ext[2 * k] + 1 for k in range(3))
    htype = np.uint64 if root.get("header_type", "UInt32") == "UInt64" else np.uint32
    out = {}
    for da in img.iter("DataArray"):
        off = int(da.get("offset"))
        hsz = np.dtype(htype).itemsize
        nbytes = int(np.frombuffer(data[us + off:us + off + hsz], dtype=htype)[0])
        dt = _VTK_TYPES[da.get("type")]
        vals = np.frombuffer(data[us + off + hsz:us + off + hsz + nbytes], dtype=dt)
        out[da.get("Name")] = (vals, int(da.get("NumberOfComponents", "1")))
    return dims, out


class VTKWriter:
    """vtkWriter(fname; dir) collection: ``save(sim)`` writes <dir>/<name>_<k>.vti (name: the base name
    of fname) and rewrites <fname>.pvd with every file, relative to the .pvd's directory, and its
    simulation time (sim_time)."""

    def __init__(self, fname: str = "WaterLily", dir: str = "vtk_data", k: int = 0, entries=None):
        self.fname, self.dir, self.k = fname, dir, k
        self.entries = list(entries or [])
        os.makedirs(dir, exist_ok=True)

    def save(self, sim) -> str:
        shape = tuple(sim.flow.p.shape)
        arrays = {"p": (_host(sim.flow.p), 1), "f": (_host(sim.intf.f), 1), "u": (_host(sim.flow.u), len(shape))}
        path = os.path.join(self.dir, f"{os.path.basename(self.fname)}_{self.k:06d}.vti")
        write_vti(path, arrays, shape)
        self.entries.append((sim.sim_time(), path))
        self.k += 1
        # DataSet paths are relative to the collection file's directory, where ReadVTK's PVDFile
        # resolves them
        pvd = self.fname + ".pvd"
        base = os.path.dirname(os.path.abspath(pvd))
        rows = "\n".join(f'    <DataSet timestep="{t!r}" part="0" file="{os.path.relpath(os.path.abspath(p), base)}"/>'
                         for t, p in self.entries)
        with open(pvd, "w") as fh:
            fh.write('<?xml version="1.0" encoding="utf-8"?>\n<VTKFile type="Collection" version="1.0">\n'
                     f'  <Collection>\n{rows}\n  </Collection>\n</VTKFile>\n')
        return path


def read_pvd(fname: str):
    """(timestep, file) of every DataSet, the files resolved against the collection's directory."""
    root = ET.parse(fname).getroot()
    base = os.path.dirname(os.path.abspath(fname))
    return [(float(ds.get("timestep")), os.path.join(base, ds.get("file"))) for ds in root.iter("DataSet")]


def load(sim, fname: str = "WaterLily.pvd") -> VTKWriter:
    """load!(sim, Val(:pvd); fname) (ext/IntfAdvReadVTKExt.jl:29-50): restore p, f and u from the last
    file of the collection, set Δt[end] = t·L/U, push a new CFL entry, and return a writer that
    appends to the same collection."""
    from .simulation import MPCFL
    entries = read_pvd(fname)
    t, path = entries[-1]
    dims, arrs = read_vti(path)
    shape = tuple(sim.flow.p.shape)
    if tuple(d for d in dims if d != 1) != tuple(n for n in shape if n != 1):
        raise ValueError("The dimensions of the simulation do not match the dimensions of the vtk file.")
    dev = sim.flow.p.device
    if "p" in arrs:
        sim.flow.p.copy_(ffrom(arrs["p"][0].reshape(shape, order="F"), device=dev))
    if "f" in arrs:
        sim.intf.f.copy_(ffrom(arrs["f"][0].reshape(shape, order="F"), device=dev))
    uv, nc = arrs["u"]
    u = uv.reshape((-1, nc)).reshape(shape + (nc,), order="F")
    sim.flow.u.copy_(ffrom(np.asfortranarray(u), device=dev))
    sim.flow.Δt[-1] = t * sim.L / sim.U
    sim.flow.Δt.append(MPCFL(sim))
    base = fname[:-4] if fname.endswith(".pvd") else fname
    return VTKWriter(base, os.path.dirname(path) or ".", k=len(entries),
                     entries=[(tt, os.path.relpath(pp)) for tt, pp in entries])
