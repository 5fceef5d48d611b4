"""Decomposition of the cube domain into parts along x and y, and the halo exchange between them.

FElib runs one local mesh per MPI rank and exchanges the face values of the prognostic fields and
of DPRES before each tendency evaluation (PROG_VARS / AUXDYNVAR3D_manager %MeshFieldComm_Exchange,
FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_driver_nonhydro3d.F90:768-787; MPI_Isend/Irecv and
waitall in MeshFieldCommBase_exchange_core / _wait_core, FElib/src/data/scale_meshfieldcomm_base.F90:
340-470).  Here the domain is split into a px x py grid of parts with full-height columns, rank
r = rx + px * ry holding element columns [rx NeX_p, (rx+1) NeX_p) x [ry NeY_p, (ry+1) NeY_p),
periodic across the grid.  A part's context (``fedg.lib.Context(..., periodic_x=HALO)`` in a split
direction) packs its boundary face layers and calls the exchange below, which moves them between
neighbouring ranks with ``torch.distributed`` point-to-point operations: NCCL on device buffers
between GPUs, gloo on host buffers (the CPU tests).  A direction with one part stays periodic.
Sides: 0 x-, 1 x+, 2 y-, 3 y+.
"""
from __future__ import annotations

import dataclasses


def _dims(nranks, dims):
    return (nranks, 1) if dims is None else tuple(dims)


def coords(rank: int, dims):
    """(rx, ry) of rank in a px x py grid"""
    px, _ = dims
    return rank % px, rank // px


def slab_case(case, rank: int, nranks: int, weak: bool = True, dims=None):
    """The Case of rank's part.  dims = (px, py), px * py = nranks (default (nranks, 1): slabs along
    x).  weak: every rank holds a whole copy of ``case``'s mesh and the domain is px x py times as
    large; strong: ``case`` is the whole domain and each rank holds an NeX/px x NeY/py part of it."""
    px, py = _dims(nranks, dims)
    if px * py != nranks:
        raise ValueError(f"dims {px} x {py} do not make {nranks} ranks")
    rx, ry = coords(rank, (px, py))
    xmin, xmax, ymin, ymax, zmin, zmax = case.dom
    if weak:
        lx, ly = xmax - xmin, ymax - ymin
        dom = (xmin + rx * lx, xmin + (rx + 1) * lx, ymin + ry * ly, ymin + (ry + 1) * ly, zmin, zmax)
        return dataclasses.replace(case, dom=dom)
    if case.NeX % px or case.NeY % py:
        raise ValueError(f"{case.NeX} x {case.NeY} elements do not split into {px} x {py} parts")
    nx, ny = case.NeX // px, case.NeY // py
    dx, dy = (xmax - xmin) / case.NeX, (ymax - ymin) / case.NeY
    dom = (xmin + rx * nx * dx, xmin + (rx + 1) * nx * dx, ymin + ry * ny * dy, ymin + (ry + 1) * ny * dy, zmin, zmax)
    return dataclasses.replace(case, NeX=nx, NeY=ny, dom=dom)


def slab_of(field, case, rank: int, nranks: int, dims=None):
    """rank's part of a field (Ne, Np) of the whole domain ``case`` (element order ex + NeX ey +
    NeX NeY ez)."""
    import numpy as np

    px, py = _dims(nranks, dims)
    rx, ry = coords(rank, (px, py))
    nx, ny = case.NeX // px, case.NeY // py
    a = np.asarray(field).reshape(case.NeZ, case.NeY, case.NeX, -1)
    part = a[:, ry * ny:(ry + 1) * ny, rx * nx:(rx + 1) * nx]
    return np.ascontiguousarray(part).reshape(case.NeZ * ny * nx, -1)


def assemble(parts, case, dims):
    """The whole-domain field (Ne, Np) from the ranks' parts (inverse of slab_of)."""
    import numpy as np

    px, py = dims
    nx, ny = case.NeX // px, case.NeY // py
    out = np.empty((case.NeZ, case.NeY, case.NeX, case.Np))
    for r, p in enumerate(parts):
        rx, ry = coords(r, dims)
        out[:, ry * ny:(ry + 1) * ny, rx * nx:(rx + 1) * nx] = np.asarray(p).reshape(case.NeZ, ny, nx, -1)
    return out.reshape(case.Ne, -1)


def periodic_flags(nranks: int, dims=None, halo: int = 2):
    """(periodic_x, periodic_y) of the parts' meshes: FEDG_HALO in a split direction, else 1"""
    px, py = _dims(nranks, dims)
    return (halo if px > 1 else 1), (halo if py > 1 else 1)


class HaloExchange:
    """The exchange of one part: send/recv are this rank's four buffers (torch tensors, device
    tensors with NCCL, host tensors with gloo; None on sides of an unsplit direction).  Calling it
    moves send[1] to the x+ neighbour's recv[0], send[0] to the x- neighbour's recv[1], send[3] to the
    y+ neighbour's recv[2] and send[2] to the y- neighbour's recv[3] (tags 0..3), and returns once all
    of this rank's receives are complete (and, for device buffers, visible to every stream)."""

    def __init__(self, send, recv, rank: int, nranks: int, group=None, dims=None):
        self.send, self.recv = send, recv
        self.dims = _dims(nranks, dims)
        self.rank, self.nranks, self.group = rank, nranks, group
        px, py = self.dims
        rx, ry = coords(rank, self.dims)
        self.peers = [((rx - 1) % px) + px * ry, ((rx + 1) % px) + px * ry,  # x-, x+
                      rx + px * ((ry - 1) % py), rx + px * ((ry + 1) % py)]  # y-, y+
        self.calls = 0

    def __call__(self, stage: int = 0, send=None, recv=None):
        import torch

        send = self.send if send is None else send
        recv = self.recv if recv is None else recv
        self.calls += 1
        ops = []
        # (this side's send, the neighbour across it, the neighbour's side it lands on)
        for sd, opp in ((1, 0), (0, 1), (3, 2), (2, 3)):
            if send[sd] is None:
                continue
            peer = self.peers[sd]
            if peer == self.rank:  # one part in this direction: its own faces are its neighbours'
                recv[opp].copy_(send[sd])
                continue
            import torch.distributed as dist

            # send across side sd (tag sd); receive on side opp from the neighbour across it
            ops.append(dist.P2POp(dist.isend, send[sd], peer, self.group, sd))
            ops.append(dist.P2POp(dist.irecv, recv[opp], self.peers[opp], self.group, sd))
        if ops:
            import torch.distributed as dist

            for req in dist.batch_isend_irecv(ops):
                req.wait()
        dev = next((t for t in recv if t is not None), None)
        if dev is not None and dev.is_cuda:
            torch.cuda.synchronize(dev.device)
