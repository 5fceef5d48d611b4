"""Slab decomposition of the cube domain along x, and the halo exchange between slabs.

FElib runs one local mesh per MPI rank and exchanges the face values of the prognostic fields and
of DPRES before each tendency evaluation (PROG_VARS / AUXDYNVAR3D_manager %MeshFieldComm_Exchange,
FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_driver_nonhydro3d.F90:768-787; MPI_Isend/Irecv and
waitall in MeshFieldCommBase_exchange_core / _wait_core, FElib/src/data/scale_meshfieldcomm_base.F90:
340-470).  Here the domain is split along x into ``nranks`` slabs of full y extent with
full-height columns, rank r holding the element columns ex in [r NeX_s, (r+1) NeX_s), periodic
in x across the ring of slabs.  A slab context (``fedg.lib.Context(..., periodic_x=HALO)``) packs
its two boundary face layers and calls the exchange below, which moves them between neighbouring
ranks with ``torch.distributed`` point-to-point operations: NCCL on device buffers between GPUs,
gloo on host buffers (the CPU tests).  A single rank is its own neighbour on both sides.
"""
from __future__ import annotations

import dataclasses


def slab_case(case, rank: int, nranks: int, weak: bool = True):
    """The Case of rank's slab.  weak: every rank holds a whole copy of ``case``'s mesh (NeX elements)
    and the domain is nranks times as long in x; strong: ``case`` is the whole domain and each rank
    holds NeX/nranks element columns of it."""
    xmin, xmax, ymin, ymax, zmin, zmax = case.dom
    if weak:
        lx = xmax - xmin
        dom = (xmin + rank * lx, xmin + (rank + 1) * lx, ymin, ymax, zmin, zmax)
        return dataclasses.replace(case, dom=dom)
    if case.NeX % nranks:
        raise ValueError(f"NeX = {case.NeX} is not a multiple of {nranks} slabs")
    nx = case.NeX // nranks
    dx = (xmax - xmin) / case.NeX
    dom = (xmin + rank * nx * dx, xmin + (rank + 1) * nx * dx, ymin, ymax, zmin, zmax)
    return dataclasses.replace(case, NeX=nx, dom=dom)


def slab_of(field, case, rank: int, nranks: int):
    """rank's part of a field (Ne, Np) of the whole domain ``case`` (element order ex + NeX ey +
    NeX NeY ez): the element columns ex in [rank NeX/nranks, (rank+1) NeX/nranks)."""
    import numpy as np

    nx = case.NeX // nranks
    a = np.asarray(field).reshape(case.NeZ, case.NeY, case.NeX, -1)
    return np.ascontiguousarray(a[:, :, rank * nx:(rank + 1) * nx]).reshape(case.NeZ * case.NeY * nx, -1)


class HaloExchange:
    """The exchange of one slab: send/recv are this rank's two buffers each (torch tensors, device
    tensors with NCCL, host tensors with gloo).  Calling it moves send[1] to the x+ neighbour's recv[0]
    and send[0] to the x- neighbour's recv[1] (tags 0 and 1), and returns once both of this rank's
    receives are complete (and, for device buffers, visible to every stream of the device)."""

    def __init__(self, send, recv, rank: int, nranks: int, group=None):
        self.send, self.recv = send, recv
        self.rank, self.nranks, self.group = rank, nranks, group
        self.right = (rank + 1) % nranks
        self.left = (rank - 1) % nranks
        self.calls = 0

    def __call__(self, stage: int = 0, send=None, recv=None):
        import torch

        send = self.send if send is None else send
        recv = self.recv if recv is None else recv
        self.calls += 1
        if self.nranks == 1:  # periodic in x through one slab: its own faces are its neighbours'
            recv[0].copy_(send[1])
            recv[1].copy_(send[0])
        else:
            import torch.distributed as dist

            ops = [dist.P2POp(dist.isend, send[1], self.right, self.group, 0),
                   dist.P2POp(dist.irecv, recv[0], self.left, self.group, 0),
                   dist.P2POp(dist.isend, send[0], self.left, self.group, 1),
                   dist.P2POp(dist.irecv, recv[1], self.right, self.group, 1)]
            for req in dist.batch_isend_irecv(ops):
                req.wait()
        if recv[0].is_cuda:
            torch.cuda.synchronize(recv[0].device)
