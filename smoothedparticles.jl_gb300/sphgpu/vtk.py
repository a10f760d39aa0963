"""ParaView frames: the device-side exporter (save_frame!, src/IO.jl:55-75)
and a reader of the files it writes (the host side of import_particles!,
src/IO.jl:90-130)."""
from __future__ import annotations

import ctypes as C
import os
import xml.etree.ElementTree as ET

import numpy as np

from . import _lib as L

_FIELD_BITS = {"x": L.SPH_FIELD_X, "v": L.SPH_FIELD_V, "a": L.SPH_FIELD_A,
               "xsph": L.SPH_FIELD_XSPH, "rho": L.SPH_FIELD_RHO, "rho_ref": L.SPH_FIELD_RHO_REF,
               "P": L.SPH_FIELD_P, "type": L.SPH_FIELD_TYPE, "oid": L.SPH_FIELD_OID,
               "key": L.SPH_FIELD_KEY}


class VtkSeries:
    """new_pvd_file(path): frames <path>/frame<k>.vtp and <path>/result.pvd.

    ``save_frame(*fields)`` returns as soon as the gather is queued on the
    system's stream; copies and file writes overlap the following steps."""

    def __init__(self, system, path: str):
        from . import SphError
        self._lib = L.load()
        self.system = system
        self.path = path
        h = C.c_void_p()
        rc = self._lib.sph_vtk_open(system._h, path.encode(), C.byref(h))
        if rc != 0:
            raise SphError(rc, f"sph_vtk_open({path}) failed")
        self._h = h
        self._frame = 0

    def save_frame(self, *fields: str, time: float | None = None) -> int:
        from . import SphError
        bits = 0
        for f in fields:
            bits |= 1 << _FIELD_BITS[f]
        k = C.c_int32()
        t = float(self._frame if time is None else time)
        rc = self._lib.sph_vtk_save_frame(self._h, bits, t, C.byref(k))
        if rc != 0:
            raise SphError(rc, "sph_vtk_save_frame failed")
        self._frame = k.value + 1
        return k.value

    def close(self):
        from . import SphError
        if getattr(self, "_h", None):
            rc = self._lib.sph_vtk_close(self._h)
            self._h = None
            if rc != 0:
                raise SphError(rc, "sph_vtk_close: a frame or the collection could not be written")

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def new_pvd_file(system, path: str) -> VtkSeries:
    """new_pvd_file(path) (src/IO.jl:22-27) bound to a system."""
    return VtkSeries(system, path)


def save_frame(data: VtkSeries, *vars: str, time: float | None = None) -> int:
    """save_frame!(data, sys, vars...) (src/IO.jl:55-75)."""
    return data.save_frame(*vars, time=time)


def save_pvd_file(data: VtkSeries):
    """save_pvd_file(data) (src/IO.jl:34-36): waits for the frames, writes
    the collection."""
    data.close()


_DT = {"Float64": np.float64, "Float32": np.float32, "Int32": np.int32, "Int64": np.int64,
       "UInt8": np.uint8}


def read_vtp(path: str) -> dict:
    """Points, vertex cells and point data of a PolyData file with raw
    appended data (UInt64 block headers)."""
    raw = open(path, "rb").read()
    start = raw.index(b"<AppendedData")
    us = raw.index(b"_", start) + 1
    xml = raw[:start].decode() + "</VTKFile>"
    root = ET.fromstring(xml)
    assert root.get("header_type") == "UInt64" and root.get("byte_order") == "LittleEndian"
    piece = root.find("PolyData/Piece")
    n = int(piece.get("NumberOfPoints"))

    def block(da):
        off = us + int(da.get("offset"))
        nb = int(np.frombuffer(raw, dtype="<u8", count=1, offset=off)[0])
        a = np.frombuffer(raw, dtype=_DT[da.get("type")], count=nb // np.dtype(_DT[da.get("type")]).itemsize,
                          offset=off + 8)
        comps = int(da.get("NumberOfComponents", "1"))
        return a.reshape(-1, comps) if comps > 1 else a

    out = {"n": n, "points": block(piece.find("Points/DataArray"))}
    for da in piece.find("Verts").findall("DataArray"):
        out[da.get("Name")] = block(da)
    out["point_data"] = {da.get("Name"): block(da) for da in piece.find("PointData").findall("DataArray")}
    return out


# import_particles! reads these point-data arrays by the particle's field
# names; the others stay at the constructor's values (zero here).
_IMPORTED = ("v", "rho", "rho_ref", "type")


def import_particles(system, path: str) -> int:
    """import_particles!(sys, path, constructor) (IO.jl:83-118): the points of
    the .vtp file at `path` are appended to the system's particles, in file
    order, with every field the file holds under the system's field names
    (v, rho, rho_ref, type); the others start at zero.  The particles already
    in the system keep their reference order and fields (x, v, rho, rho_ref,
    type; a later init_state or step recomputes the rest).  Returns the
    number of particles added."""
    d = read_vtp(path)
    n_new = d["n"]
    pts = np.asarray(d["points"], dtype=np.float64).reshape(n_new, 3)
    pd = d["point_data"]
    add = {"x": pts}
    for f in _IMPORTED:
        if f in pd:
            a = np.asarray(pd[f])
            add[f] = a.reshape(n_new, 3) if f == "v" else a.reshape(n_new)
    n0 = system.n
    old = {f: system.get(f) for f in ("x", "v", "rho", "rho_ref", "type")} if n0 else {}

    def cat(f, shape, dtype):
        a = old.get(f, np.zeros((0,) + shape, dtype))
        b = add.get(f, np.zeros((n_new,) + shape, dtype)).astype(dtype)
        return np.concatenate([a.reshape((-1,) + shape), b])

    system.upload(cat("x", (3,), np.float64), cat("v", (3,), np.float64),
                  rho=cat("rho", (), np.float64), rho_ref=cat("rho_ref", (), np.float64),
                  type=cat("type", (), np.int32))
    return n_new


def read_pvd(path: str) -> list:
    """(time, file) of every frame of a collection."""
    root = ET.parse(path).getroot()
    return [(float(d.get("timestep")), os.path.join(os.path.dirname(path), d.get("file")))
            for d in root.find("Collection").findall("DataSet")]
