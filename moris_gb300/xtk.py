"""XFEM input over the C ABI (fem_xtk_*): decomposition of a uniform level-0
HEX8 mesh by a nodal level set into TET4 integration cells, Heaviside
enrichment, interface and ghost facets, on the host or on the GPU; returns
numpy arrays."""
import ctypes as C

import numpy as np

from . import FemGpuError, _np_ptr, lib
from ._lib import XtkSizes


def decompose(num_elements, lengths, order, node_phi, device=False):
    """node_phi: level set at the (n0+1)(n1+1)(n2+1) grid nodes (i fastest);
    phase 1 where phi < 0.  device=True computes the same decomposition on
    the GPU (fem_xtk_decompose_device).  Returns a dict of arrays (see fem_xtk_*
    in include/fem_gpu.h)."""
    L = lib()
    ne = np.ascontiguousarray(num_elements, dtype=np.int32)
    ln = np.ascontiguousarray(lengths, dtype=np.float64)
    phi = np.ascontiguousarray(node_phi, dtype=np.float64)
    h = C.c_void_p()
    fn = L.fem_xtk_decompose_device if device else L.fem_xtk_decompose
    st = fn(_np_ptr(ne), _np_ptr(ln), order, _np_ptr(phi), C.byref(h))
    if st:
        raise FemGpuError(st, "fem_xtk_decompose_device" if device else "fem_xtk_decompose")
    try:
        s = XtkSizes()
        L.fem_xtk_get_sizes(h, C.byref(s))
        out = dict(sizes=s)
        nn, nc, tn = s.num_nodes, s.num_cells, s.t_nnz
        coords = np.zeros(nn * 3)
        cells = np.zeros(nc * 8, dtype=np.int32)
        t_off = np.zeros(nn + 1, dtype=np.int64)
        t_b = np.zeros(tn, dtype=np.int32)
        t_w = np.zeros(tn)
        bgc = np.zeros(nc, dtype=np.int32)
        ph = np.zeros(nc, dtype=np.int32)
        L.fem_xtk_get_ip_mesh(h, _np_ptr(coords), _np_ptr(cells), _np_ptr(t_off), _np_ptr(t_b), _np_ptr(t_w),
                              _np_ptr(bgc), _np_ptr(ph))
        out["mesh"] = dict(coords=coords.reshape(nn, 3), cells=cells.reshape(nc, 8), t_off=t_off, t_bases=t_b,
                           t_w=t_w, num_bases=s.num_bases)
        out["cell_background"], out["cell_phase"] = bgc, ph
        for p in (0, 1):
            unc = np.zeros(s.num_uncut[p], dtype=np.int32)
            cut = np.zeros(s.num_cut[p], dtype=np.int32)
            off = np.zeros(s.num_cut[p] + 1, dtype=np.int64)
            nig = s.num_ig_cells[p]
            igx = np.zeros(nig * 12)
            igp = np.zeros(nig * 12)
            igv = np.zeros(nig * 4, dtype=np.int32)
            L.fem_xtk_get_bulk(h, p, _np_ptr(unc), _np_ptr(cut), _np_ptr(off), _np_ptr(igx), _np_ptr(igp),
                               _np_ptr(igv))
            out["uncut%d" % p] = unc
            out["cut%d" % p] = dict(cells=cut, ig_offsets=off, ig_coords=igx, ig_param=igp,
                                    ig_vertices=igv.reshape(-1, 4))
            ng = s.num_ghost[p]
            gl = np.zeros(ng, dtype=np.int32)
            gf = np.zeros(ng, dtype=np.int32)
            gx = np.zeros(ng * 12)
            gpl = np.zeros(ng * 12)
            gpf = np.zeros(ng * 12)
            L.fem_xtk_get_ghost(h, p, _np_ptr(gl), _np_ptr(gf), _np_ptr(gx), _np_ptr(gpl), _np_ptr(gpf))
            out["ghost%d" % p] = dict(leader=gl, follower=gf, offsets=np.arange(ng + 1, dtype=np.int64), coords=gx,
                                      leader_param=gpl, follower_param=gpf)
        ni, nf = s.num_interface, s.num_interface_facets
        il = np.zeros(ni, dtype=np.int32)
        iff = np.zeros(ni, dtype=np.int32)
        ioff = np.zeros(ni + 1, dtype=np.int64)
        ix = np.zeros(nf * 9)
        ip = np.zeros(nf * 9)
        iv = np.zeros(nf * 3, dtype=np.int32)
        L.fem_xtk_get_interface(h, _np_ptr(il), _np_ptr(iff), _np_ptr(ioff), _np_ptr(ix), _np_ptr(ip), _np_ptr(iv))
        out["interface"] = dict(leader=il, follower=iff, offsets=ioff, coords=ix, param=ip, vertices=iv.reshape(-1, 3))
        nv = s.num_ig_vertices
        kind = np.zeros(nv, dtype=np.int32)
        par = np.zeros(nv * 8, dtype=np.int32)
        vx = np.zeros(nv * 3)
        val = np.zeros(nv)
        L.fem_xtk_get_vertices(h, _np_ptr(kind), _np_ptr(par), _np_ptr(vx), _np_ptr(val))
        out["vertices"] = dict(kind=kind, parents=par.reshape(nv, 8), coords=vx.reshape(nv, 3), value=val)
        return out
    finally:
        L.fem_xtk_free(h)
