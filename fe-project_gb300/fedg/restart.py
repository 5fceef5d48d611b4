"""Restart files of the dynamics state, host side (numpy): the same flat little-endian format the
library's fedg_restart_write / fedg_restart_read use (layout in fe-project_gb300/csrc/fedg_restart.cu),
the content FElib writes through NetCDF (FElib/src/file/scale_file_restart_meshfield.F90:136-186).
Fields are (Ne, Np) float64 arrays in C order, the memory of FElib's column-major (Np, Ne)."""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

MAGIC = b"FEDGRST1"
HEADER = 112
NAMES = ("DDENS", "MOMX", "MOMY", "MOMZ", "DRHOT", "DENS_hyd", "PRES_hyd", "THERM_hyd")


@dataclass
class Restart:
    porder: int
    NeX: int
    NeY: int
    NeZ: int
    step: int = 0
    time: float = 0.0
    dt: float = 0.0
    scheme: str = ""
    ref_wind: tuple | None = None  # (U, V) of the fast update paths, or None
    fields: dict = field(default_factory=dict)  # NAMES -> (Ne, Np) arrays

    @property
    def Np(self):
        return (self.porder + 1) ** 3

    @property
    def Ne(self):
        return self.NeX * self.NeY * self.NeZ


def write(path, r: Restart):
    head = bytearray(HEADER)
    head[0:8] = MAGIC
    wind = r.ref_wind is not None
    struct.pack_into("<8i", head, 8, r.porder, r.NeX, r.NeY, r.NeZ, r.Np, len(NAMES), int(wind), 0)
    struct.pack_into("<q", head, 40, int(r.step))
    u, v = r.ref_wind if wind else (0.0, 0.0)
    struct.pack_into("<4d", head, 48, float(r.time), float(r.dt), float(u), float(v))
    name = r.scheme.encode()[:31]
    head[80:80 + len(name)] = name
    with open(path, "wb") as f:
        f.write(bytes(head))
        for nm in NAMES:
            a = np.ascontiguousarray(r.fields[nm], dtype="<f8")
            assert a.shape == (r.Ne, r.Np), (nm, a.shape)
            f.write(a.tobytes())


def read(path) -> Restart:
    with open(path, "rb") as f:
        head = f.read(HEADER)
        if len(head) != HEADER or head[:8] != MAGIC:
            raise ValueError(f"{path}: not a restart file of this library")
        porder, nex, ney, nez, np_, nf, wind, _ = struct.unpack_from("<8i", head, 8)
        (step,) = struct.unpack_from("<q", head, 40)
        time, dt, u, v = struct.unpack_from("<4d", head, 48)
        scheme = head[80:112].split(b"\0", 1)[0].decode()
        r = Restart(porder, nex, ney, nez, step, time, dt, scheme, (u, v) if wind else None)
        if np_ != r.Np or nf != len(NAMES):
            raise ValueError(f"{path}: inconsistent header")
        for nm in NAMES:
            a = np.frombuffer(f.read(8 * r.Ne * r.Np), dtype="<f8")
            if a.size != r.Ne * r.Np:
                raise ValueError(f"{path}: file too short")
            r.fields[nm] = a.reshape(r.Ne, r.Np).astype(np.float64)
    return r
