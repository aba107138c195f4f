"""Field output (the reference's VIS path): nodal values of an adof field on
the device (fem_gpu_nodal_field) and an Exodus II file of the interpolation
mesh with nodal fields (fem_vis_write_exodus)."""
import ctypes as C

import numpy as np

from . import FemGpuError, _dev_ptr, lib

ELEM_TYPES = {(2, 4): "QUAD4", (3, 8): "HEX8"}


def nodal_field(model, u):
    """[dim][num_nodes] nodal values of the adof vector u (CUDA tensors)"""
    import torch
    out = torch.empty(model.dim * model.num_nodes, dtype=torch.float64, device="cuda")
    model._check(lib().fem_gpu_nodal_field(model.h, _dev_ptr(u), _dev_ptr(out)), "nodal_field")
    return out.view(model.dim, model.num_nodes)


def write_exodus(path, coords, cells, fields, time=0.0):
    """coords [n][dim], cells [ncells][nodes per cell] (0-based), fields
    {name: [n] values}; one element block, one time step"""
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    cells = np.ascontiguousarray(cells, dtype=np.int32)
    n, dim = coords.shape
    nc, npc = cells.shape
    names = list(fields)
    vals = np.ascontiguousarray(np.stack([np.asarray(fields[k], dtype=np.float64) for k in names])
                                if names else np.zeros((0, n)))
    cnames = (C.c_char_p * max(1, len(names)))(*[k.encode() for k in names])
    st = lib().fem_vis_write_exodus(str(path).encode(), dim, n, coords.ctypes.data_as(C.c_void_p), nc, npc,
                                    cells.ctypes.data_as(C.c_void_p), ELEM_TYPES.get((dim, npc), "HEX8").encode(),
                                    len(names), C.cast(cnames, C.c_void_p), vals.ctypes.data_as(C.c_void_p),
                                    float(time))
    if st:
        raise FemGpuError(st, "fem_vis_write_exodus")
