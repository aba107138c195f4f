"""moris_gb300 -- GB300 (sm_103a) element hot path of MORIS behind a C ABI.

Python here is glue for tests and benchmarks: every compute entry point is
a call into libfem_gpu.so (include/fem_gpu.h).  The classes mirror the
reference's solver-interface vocabulary: sets of equation objects, element
topology (adof ids), element operators, fill_matrix_and_RHS.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import BulkSetDesc, DoubleSideSetDesc, MeshDesc, PcgOpts, PcgReport, SideSetDesc

# enums (identical values in include/fem_gpu.h)
CELL_QUAD4, CELL_HEX8, CELL_TRI3, CELL_TET4, CELL_LINE2 = 0, 1, 2, 3, 4
RULE_BAR_1, RULE_BAR_3, RULE_QUAD_2x2, RULE_HEX_2x2x2, RULE_HEX_3x3x3 = 0, 1, 2, 3, 4
RULE_TRI_7, RULE_TET_4, RULE_TET_11, RULE_TRI_3 = 5, 6, 7, 8
RULE_AUTO = -1
SET_BULK, SET_SIDESET, SET_DOUBLE_SIDESET = 0, 1, 2
MODEL_PLANE_STRAIN, MODEL_PLANE_STRESS, MODEL_3D = 0, 1, 2
SHAPE_RECTANGULAR, SHAPE_GENERAL = 0, 1
IWG_STRUC_LINEAR_BULK = 0
IWG_STRUC_LINEAR_NEUMANN = 1
IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE = 2
IWG_STRUC_LINEAR_DIRICHLET_UNSYMMETRIC_NITSCHE = 3
IWG_STRUC_LINEAR_INTERFACE_SYMMETRIC_NITSCHE = 4
IWG_STRUC_LINEAR_INTERFACE_UNSYMMETRIC_NITSCHE = 5
IWG_STRUC_LINEAR_VW_GHOST = 6
IWG_GHOST_NORMAL_FIELD = 7
HOST_BUFFERS, NO_JACOBIAN, NO_RESIDUAL, ACCUMULATE, ASYNC = 1, 2, 4, 8, 16


class FemGpuError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("fem_gpu status %d (%s): %s" % (status, _status_text(status), msg))
        self.status = status


def _status_text(s):
    t = _lib.load().fem_gpu_status_string(s)
    return t.decode() if t else "?"


def _np_ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _dev_ptr(t):
    """Device pointer of a CUDA tensor (or None)."""
    if t is None:
        return None
    assert t.is_cuda and t.is_contiguous()
    return C.c_void_p(t.data_ptr())


_default_stream = None


def set_default_stream(fn):
    """Stream for models created from now on: fn() returns a cudaStream_t as an
    int (torch: ``lambda: torch.cuda.current_stream().cuda_stream``), or fn is
    None for the library's own stream.  A model whose inputs come from another
    stream's kernels must run on that stream (or the caller synchronises)."""
    global _default_stream
    _default_stream = fn


def lib():
    return _lib.load()


def device_count():
    return lib().fem_gpu_device_count()


def bspline_tmatrix(num_coefs, lengths, order, points):
    """(cols, vals) [n_points][(order+1)^3] of a uniform tensor B-spline field."""
    nc = np.ascontiguousarray(num_coefs, dtype=np.int32)
    ln = np.ascontiguousarray(lengths, dtype=np.float64)
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    w = (order + 1) ** 3
    cols = np.zeros((len(pts), w), dtype=np.int32)
    vals = np.zeros((len(pts), w))
    st = lib().fem_gen_bspline_tmatrix(_np_ptr(nc), _np_ptr(ln), order, len(pts), _np_ptr(pts), _np_ptr(cols),
                                       _np_ptr(vals))
    if st:
        raise FemGpuError(st, "fem_gen_bspline_tmatrix")
    return cols, vals


def auto_integration_rule(set_kind, cell, interpolation_order=1):
    """The reference's automatic integration rule (Set::get_auto_integration_order)."""
    r = C.c_int32()
    st = lib().fem_gpu_auto_integration_rule(set_kind, cell, interpolation_order, C.byref(r))
    if st:
        raise FemGpuError(st, "fem_gpu_auto_integration_rule")
    return r.value


def probe_fp64_tflops(iters=20000):
    """Measured FP64 FMA throughput of the current GPU (TFLOP/s)."""
    t = C.c_double()
    st = lib().fem_gpu_probe_fp64_tflops(iters, C.byref(t))
    if st:
        raise FemGpuError(st, "probe_fp64_tflops")
    return t.value


def probe_dmma_tflops(iters=300, mixed=False):
    """Measured FP64 tensor-core (DMMA) throughput, optionally mixed with DFMA."""
    t = C.c_double()
    st = lib().fem_gpu_probe_dmma_tflops(iters, 1 if mixed else 0, C.byref(t))
    if st:
        raise FemGpuError(st, "probe_dmma_tflops")
    return t.value


def hmr_uniform_mesh(dim, num_elements, lengths, bspline_order):
    """Uniform level-0 HMR-equivalent mesh: dict of numpy arrays."""
    L = lib()
    ne = np.asarray(list(num_elements) + [1] * (3 - len(num_elements)), dtype=np.int32)
    ln = np.asarray(list(lengths) + [1.0] * (3 - len(lengths)), dtype=np.float64)
    h = C.c_void_p()
    st = L.fem_hmr_uniform_mesh(dim, _np_ptr(ne), _np_ptr(ln), bspline_order, C.byref(h))
    if st:
        raise FemGpuError(st, "fem_hmr_uniform_mesh")
    nn, nc, nb, nz = (C.c_int64() for _ in range(4))
    L.fem_hmr_mesh_sizes(h, C.byref(nn), C.byref(nc), C.byref(nb), C.byref(nz))
    npe = 4 if dim == 2 else 8
    coords = np.zeros(nn.value * dim)
    cells = np.zeros(nc.value * npe, dtype=np.int32)
    t_off = np.zeros(nn.value + 1, dtype=np.int64)
    t_b = np.zeros(nz.value, dtype=np.int32)
    t_w = np.zeros(nz.value)
    L.fem_hmr_mesh_arrays(h, _np_ptr(coords), _np_ptr(cells), _np_ptr(t_off), _np_ptr(t_b), _np_ptr(t_w))
    L.fem_hmr_mesh_free(h)
    return dict(coords=coords.reshape(-1, dim), cells=cells.reshape(-1, npe), num_bases=nb.value, t_off=t_off,
                t_bases=t_b, t_w=t_w)


def _mesh_dict(L, h, dim):
    nn, nc, nb, nz = (C.c_int64() for _ in range(4))
    L.fem_hmr_mesh_sizes(h, C.byref(nn), C.byref(nc), C.byref(nb), C.byref(nz))
    npe = 4 if dim == 2 else 8
    coords = np.zeros(nn.value * dim)
    cells = np.zeros(nc.value * npe, dtype=np.int32)
    t_off = np.zeros(nn.value + 1, dtype=np.int64)
    t_b = np.zeros(nz.value, dtype=np.int32)
    t_w = np.zeros(nz.value)
    L.fem_hmr_mesh_arrays(h, _np_ptr(coords), _np_ptr(cells), _np_ptr(t_off), _np_ptr(t_b), _np_ptr(t_w))
    L.fem_hmr_mesh_free(h)
    return dict(coords=coords.reshape(-1, dim), cells=cells.reshape(-1, npe), num_bases=nb.value, t_off=t_off,
                t_bases=t_b, t_w=t_w)


class RefinedHmr:
    """A refined (hierarchical) HMR B-spline mesh (fem_hmr_refined_*):
    refine active domain elements level by level, query element T matrices,
    and produce the Lagrange mesh with node extraction rows for FemModel."""

    def __init__(self, dim, num_elements, lengths, order, staircase_buffer=None, padding_refinement=None):
        self.L = lib()
        self.dim, self.order = dim, order
        buf = order if staircase_buffer is None else staircase_buffer
        pr = (order + 1) // 2 if padding_refinement is None else padding_refinement
        ne = np.ascontiguousarray(num_elements, dtype=np.int32)
        ln = np.ascontiguousarray(lengths, dtype=np.float64)
        h = C.c_void_p()
        st = self.L.fem_hmr_refined_create(dim, _np_ptr(ne), _np_ptr(ln), order, buf, pr, C.byref(h))
        if st:
            raise FemGpuError(st, "fem_hmr_refined_create")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            self.L.fem_hmr_refined_free(self.h)
            self.h = None

    def refine(self, elements):
        """elements: [(level, ijk)] of active domain elements (domain-relative ijk)"""
        lv = np.ascontiguousarray([l for l, _ in elements], dtype=np.int32)
        ijk = np.ascontiguousarray([list(e) for _, e in elements], dtype=np.int32).ravel()
        st = self.L.fem_hmr_refined_refine(self.h, len(lv), _np_ptr(lv), _np_ptr(ijk))
        if st:
            raise FemGpuError(st, "fem_hmr_refined_refine")

    def active_elements(self):
        n = C.c_int64()
        self.L.fem_hmr_refined_active_elements(self.h, C.byref(n), None, None)
        lv = np.zeros(n.value, dtype=np.int32)
        ijk = np.zeros(n.value * self.dim, dtype=np.int32)
        self.L.fem_hmr_refined_active_elements(self.h, C.byref(n), _np_ptr(lv), _np_ptr(ijk))
        return lv, ijk.reshape(-1, self.dim)

    def element_t_matrix(self, level, ijk, truncate):
        """(T [(order+1)^dim, ndof], dof levels [ndof], dof ijk [ndof, dim])"""
        e = np.ascontiguousarray(ijk, dtype=np.int32)
        nd = C.c_int32()
        st = self.L.fem_hmr_refined_element_t_matrix(self.h, level, _np_ptr(e), int(truncate), 0, C.byref(nd), None,
                                                    None, None)
        if st:
            raise FemGpuError(st, "fem_hmr_refined_element_t_matrix")
        n, B = nd.value, (self.order + 1) ** self.dim
        T = np.zeros(B * max(n, 1))
        dl = np.zeros(max(n, 1), dtype=np.int32)
        di = np.zeros(max(n, 1) * self.dim, dtype=np.int32)
        st = self.L.fem_hmr_refined_element_t_matrix(self.h, level, _np_ptr(e), int(truncate), n, C.byref(nd),
                                                    _np_ptr(T), _np_ptr(dl), _np_ptr(di))
        if st:
            raise FemGpuError(st, "fem_hmr_refined_element_t_matrix")
        return T[:B * n].reshape(B, n), dl[:n], di[:n * self.dim].reshape(n, self.dim)

    def mesh(self, truncate=True, device=False):
        """The Lagrange mesh of the active elements with its node rows; with
        device=True the element T matrices and node rows are evaluated on the GPU."""
        h = C.c_void_p()
        fn = self.L.fem_hmr_refined_mesh_device if device else self.L.fem_hmr_refined_mesh
        st = fn(self.h, int(truncate), C.byref(h))
        if st:
            raise FemGpuError(st, "fem_hmr_refined_mesh" + ("_device" if device else ""))
        return _mesh_dict(self.L, h, self.dim)

    def element_t_matrices_device(self, levels, ijk, truncate):
        """T matrices of several elements computed on the GPU: a list of
        (T [(order+1)^dim, ndof], dof levels [ndof], dof ijk [ndof, dim])"""
        lv = np.ascontiguousarray(levels, dtype=np.int32)
        e = np.ascontiguousarray(ijk, dtype=np.int32).reshape(len(lv), self.dim)
        n = len(lv)
        nd = np.zeros(max(n, 1), dtype=np.int32)
        st = self.L.fem_hmr_refined_element_t_matrices_device(self.h, int(truncate), n, _np_ptr(lv), _np_ptr(e), 0,
                                                              _np_ptr(nd), None, None, None)
        if st:
            raise FemGpuError(st, "fem_hmr_refined_element_t_matrices_device")
        cap, B = max(int(nd[:n].max()) if n else 1, 1), (self.order + 1) ** self.dim
        T = np.zeros(n * B * cap)
        dl = np.zeros(n * cap, dtype=np.int32)
        di = np.zeros(n * cap * self.dim, dtype=np.int32)
        st = self.L.fem_hmr_refined_element_t_matrices_device(self.h, int(truncate), n, _np_ptr(lv), _np_ptr(e), cap,
                                                              _np_ptr(nd), _np_ptr(T), _np_ptr(dl), _np_ptr(di))
        if st:
            raise FemGpuError(st, "fem_hmr_refined_element_t_matrices_device")
        T = T.reshape(n, B, cap)
        dl = dl.reshape(n, cap)
        di = di.reshape(n, cap, self.dim)
        return [(T[i, :, :nd[i]], dl[i, :nd[i]], di[i, :nd[i]]) for i in range(n)]


class FemModel:
    """A context of libfem_gpu: one interpolation mesh, its sets, the CSR graph."""

    def __init__(self, dim, mesh, shape=SHAPE_RECTANGULAR):
        self.L = lib()
        self.dim = dim
        self._keep = {}
        coords = np.ascontiguousarray(mesh["coords"], dtype=np.float64).ravel()
        cells = np.ascontiguousarray(mesh["cells"], dtype=np.int32).ravel()
        t_off = np.ascontiguousarray(mesh["t_off"], dtype=np.int64)
        t_b = np.ascontiguousarray(mesh["t_bases"], dtype=np.int32)
        t_w = np.ascontiguousarray(mesh["t_w"], dtype=np.float64)
        d = MeshDesc(dim, CELL_QUAD4 if dim == 2 else CELL_HEX8, shape, 0, len(coords) // dim, _np_ptr(coords),
                     len(mesh["cells"]), _np_ptr(cells), int(mesh["num_bases"]), _np_ptr(t_off), _np_ptr(t_b),
                     _np_ptr(t_w))
        h = C.c_void_p()
        self._check(self.L.fem_gpu_create(C.byref(d), C.byref(h)), "create", ctx=False)
        self.h = h
        self.num_sets = 0
        self.num_nodes = len(coords) // dim
        if _default_stream is not None:
            self.set_stream(_default_stream())

    def __del__(self):
        if getattr(self, "h", None):
            self.L.fem_gpu_destroy(self.h)
            self.h = None

    def _check(self, st, what, ctx=True):
        if st:
            msg = what
            if ctx and getattr(self, "h", None):
                e = self.L.fem_gpu_last_error(self.h)
                msg += ": " + (e.decode() if e else "")
            raise FemGpuError(st, msg)

    def set_stream(self, stream_ptr):
        self._check(self.L.fem_gpu_set_stream(self.h, C.c_void_p(stream_ptr)), "set_stream")

    def add_bulk_set(self, ip_cells, youngs, poisson, rule, model, ig_cell=None, ig_offsets=None, ig_coords=None,
                     ig_param=None, node_density=None, density_exponent=3.0, ig_vertex_ids=None, thickness=0.0):
        ipc = np.ascontiguousarray(ip_cells, dtype=np.int32)
        rho = None if node_density is None else np.ascontiguousarray(node_density, dtype=np.float64)
        E = np.ascontiguousarray(youngs, dtype=np.float64)
        off = None if ig_offsets is None else np.ascontiguousarray(ig_offsets, dtype=np.int64)
        xc = None if ig_coords is None else np.ascontiguousarray(ig_coords, dtype=np.float64)
        xp = None if ig_param is None else np.ascontiguousarray(ig_param, dtype=np.float64)
        if ig_cell is None:
            ig_cell = CELL_QUAD4 if self.dim == 2 else CELL_HEX8
        vid = None if ig_vertex_ids is None else np.ascontiguousarray(ig_vertex_ids, dtype=np.int32)
        d = BulkSetDesc(IWG_STRUC_LINEAR_BULK, ig_cell, rule, model, len(ipc), _np_ptr(ipc), _np_ptr(off),
                        _np_ptr(xc), _np_ptr(xp), _np_ptr(E), poisson, _np_ptr(rho), density_exponent, _np_ptr(vid),
                        thickness)
        idx = C.c_int32()
        self._check(self.L.fem_gpu_add_bulk_set(self.h, C.byref(d), C.byref(idx)), "add_bulk_set")
        self.num_sets += 1
        return idx.value

    def add_side_set(self, iwg, ip_cells, ordinals, youngs, poisson, rule, model, alpha=0.0, value=(0, 0, 0),
                     thickness=0.0, select=None):
        """thickness: the IWG's Thickness property (0 = none); select: the
        Dirichlet IWG's Select matrix (dim x dim, None = identity)"""
        ipc = np.ascontiguousarray(ip_cells, dtype=np.int32)
        ords = np.ascontiguousarray(ordinals, dtype=np.int32)
        E = np.ascontiguousarray(youngs, dtype=np.float64)
        v = (C.c_double * 3)(*(list(value) + [0.0] * (3 - len(value))))
        sel = None if select is None else np.ascontiguousarray(select, dtype=np.float64).reshape(self.dim, self.dim)
        d = SideSetDesc(iwg, rule, model, 0, len(ipc), _np_ptr(ipc), _np_ptr(ords), _np_ptr(E), poisson, alpha, v,
                        thickness, _np_ptr(sel))
        idx = C.c_int32()
        self._check(self.L.fem_gpu_add_side_set(self.h, C.byref(d), C.byref(idx)), "add_side_set")
        self.num_sets += 1
        return idx.value

    def add_double_side_set(self, iwg, leader, follower, facet_offsets, facet_coords, leader_param, follower_param,
                            leader_youngs, follower_youngs, poisson, rule, facet_cell, alpha, model=MODEL_3D,
                            facet_vertex_ids=None):
        """Interface (Nitsche) or ghost clusters: facets given by vertex coords and
        their parametric coords in the leader / follower IP cells."""
        L_ = np.ascontiguousarray(leader, dtype=np.int32)
        F_ = np.ascontiguousarray(follower, dtype=np.int32)
        off = np.ascontiguousarray(facet_offsets, dtype=np.int64)
        fx = np.ascontiguousarray(facet_coords, dtype=np.float64)
        fl = np.ascontiguousarray(leader_param, dtype=np.float64)
        ff = np.ascontiguousarray(follower_param, dtype=np.float64)
        EL = np.ascontiguousarray(leader_youngs, dtype=np.float64)
        EF = np.ascontiguousarray(follower_youngs, dtype=np.float64)
        vid = None if facet_vertex_ids is None else np.ascontiguousarray(facet_vertex_ids, dtype=np.int32)
        d = DoubleSideSetDesc(iwg, facet_cell, rule, model, len(L_), _np_ptr(L_), _np_ptr(F_), _np_ptr(off),
                              _np_ptr(fx), _np_ptr(fl), _np_ptr(ff), _np_ptr(EL), _np_ptr(EF), poisson, alpha,
                              _np_ptr(vid))
        idx = C.c_int32()
        self._check(self.L.fem_gpu_add_double_side_set(self.h, C.byref(d), C.byref(idx)), "add_double_side_set")
        self.num_sets += 1
        return idx.value

    def assemble_batched(self, u, vals, rhs, flags=0):
        """All bulk and double-sided clusters in one persistent graph-captured launch
        (device tensors)."""
        self._check(self.L.fem_gpu_assemble_batched(self.h, _dev_ptr(u), _dev_ptr(vals), _dev_ptr(rhs), flags),
                    "assemble_batched")

    # ---- shape sensitivities -------------------------------------------------
    def set_ig_vertices(self, kind, parents, coords, value):
        k = np.ascontiguousarray(kind, dtype=np.int32)
        p = np.ascontiguousarray(parents, dtype=np.int32)
        x = np.ascontiguousarray(coords, dtype=np.float64)
        v = np.ascontiguousarray(value, dtype=np.float64)
        self._check(self.L.fem_gpu_set_ig_vertices(self.h, len(k), _np_ptr(k), _np_ptr(p), _np_ptr(x), _np_ptr(v)),
                    "set_ig_vertices")

    def update_ig_vertices(self, t):
        t = np.ascontiguousarray(t, dtype=np.float64)
        self._check(self.L.fem_gpu_update_ig_vertices(self.h, _np_ptr(t)), "update_ig_vertices")

    def strain_energy(self, u, dqdu):
        q = C.c_double()
        self._check(self.L.fem_gpu_strain_energy(self.h, _dev_ptr(u), _dev_ptr(dqdu), C.byref(q)), "strain_energy")
        return q.value

    def drdp_adjoint(self, u, lam, G):
        self._check(self.L.fem_gpu_drdp_adjoint(self.h, _dev_ptr(u), _dev_ptr(lam), _dev_ptr(G)), "drdp_adjoint")

    def set_level_set_field(self, cols, tmat, num_coefs):
        """Stores the level-set field on the device (fem_gpu_set_level_set_field)."""
        cols = np.ascontiguousarray(cols, dtype=np.int32)
        tmat = np.ascontiguousarray(tmat, dtype=np.float64)
        if cols.shape != tmat.shape or cols.ndim != 2:
            raise ValueError("cols and tmat: [nodes][width] of one shape")
        self._check(self.L.fem_gpu_set_level_set_field(self.h, cols.shape[0], cols.shape[1], _np_ptr(cols),
                                                       _np_ptr(tmat), num_coefs), "set_level_set_field")
        self._ls_shape = cols.shape

    def gen_dqdp(self, G, cols, tmat, num_coefs, dqdp):
        """dQ/dp through the level-set field; cols = tmat = None uses the field
        stored by set_level_set_field."""
        if cols is None and tmat is None:
            nbn, width = getattr(self, "_ls_shape", (0, 0))
            if nbn == 0:
                raise ValueError("no stored level-set field")
            self._check(self.L.fem_gen_dqdp(self.h, _dev_ptr(G), nbn, width, None, None, num_coefs,
                                            _dev_ptr(dqdp)), "gen_dqdp")
            return
        cols = np.ascontiguousarray(cols, dtype=np.int32)
        tmat = np.ascontiguousarray(tmat, dtype=np.float64)
        self._check(self.L.fem_gen_dqdp(self.h, _dev_ptr(G), cols.shape[0], cols.shape[1], _np_ptr(cols),
                                        _np_ptr(tmat), num_coefs, _dev_ptr(dqdp)), "gen_dqdp")

    def check_status(self):
        self._check(self.L.fem_gpu_check_status(self.h), "check_status")

    def autotune_batched(self):
        w, sp, ms = C.c_int32(), C.c_int32(), C.c_double()
        self._check(self.L.fem_gpu_autotune_batched(self.h, C.byref(w), C.byref(sp), C.byref(ms)), "autotune_batched")
        return w.value, sp.value, ms.value

    def set_batched_config(self, warps, split):
        self._check(self.L.fem_gpu_set_batched_config(self.h, warps, split), "set_batched_config")

    def finalize(self, host_only=False):
        f = self.L.fem_gpu_finalize_host if host_only else self.L.fem_gpu_finalize
        self._check(f(self.h), "finalize")
        nad, nnz, ns = C.c_int64(), C.c_int64(), C.c_int32()
        self._check(self.L.fem_gpu_get_sizes(self.h, C.byref(nad), C.byref(nnz), C.byref(ns)), "get_sizes")
        self.num_adofs, self.nnz = nad.value, nnz.value

    def num_eq(self, s):
        n = C.c_int64()
        self._check(self.L.fem_gpu_get_num_equation_objects(self.h, s, C.byref(n)), "num_eq")
        return n.value

    def max_element_adofs(self, s):
        n = C.c_int32()
        self._check(self.L.fem_gpu_get_max_element_adofs(self.h, s, C.byref(n)), "max_element_adofs")
        return n.value

    def graph(self):
        rp = np.zeros(self.num_adofs + 1, dtype=np.int32)
        ci = np.zeros(self.nnz, dtype=np.int32)
        self._check(self.L.fem_gpu_build_graph(self.h, _np_ptr(rp), _np_ptr(ci), HOST_BUFFERS), "build_graph")
        return rp, ci

    def graph_device(self, rowptr_t, colidx_t):
        self._check(self.L.fem_gpu_build_graph(self.h, _dev_ptr(rowptr_t), _dev_ptr(colidx_t), 0), "build_graph")

    def element_topology(self, s, eq):
        ids = np.zeros(max(self.max_element_adofs(s), 1), dtype=np.int32)
        n = C.c_int32()
        self._check(self.L.fem_gpu_get_element_topology(self.h, s, eq, _np_ptr(ids), C.byref(n)), "topology")
        return ids[:n.value].copy()

    def element_matrices(self, s, first, count, u=None):
        """Host path: returns K (count, n, n) with K[e, i, j] and R (count, n)."""
        n = self.max_element_adofs(s)
        K = np.zeros(count * n * n)
        R = np.zeros(count * n)
        uu = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
        st = self.L.fem_gpu_element_matrices(self.h, s, first, count, _np_ptr(uu), _np_ptr(K), _np_ptr(R),
                                             HOST_BUFFERS)
        self._check(st, "element_matrices")
        return K.reshape(count, n, n).transpose(0, 2, 1).copy(), R.reshape(count, n)

    def assemble(self, u, vals, rhs, flags=0):
        """Device path: u, vals, rhs are CUDA tensors (vals/rhs may be None)."""
        self._check(self.L.fem_gpu_assemble(self.h, _dev_ptr(u), _dev_ptr(vals), _dev_ptr(rhs), flags), "assemble")

    def assemble_host(self, u, flags=0):
        vals = np.zeros(self.nnz)
        rhs = np.zeros(self.num_adofs)
        uu = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
        st = self.L.fem_gpu_assemble(self.h, _np_ptr(uu), _np_ptr(vals), _np_ptr(rhs), flags | HOST_BUFFERS)
        self._check(st, "assemble")
        return vals, rhs

    def assemble_raw(self, u_ptr, vals_ptr, rhs_ptr, flags):
        """Raw-pointer form (e.g. pinned host memory with HOST_BUFFERS)."""
        st = self.L.fem_gpu_assemble(self.h, C.c_void_p(u_ptr), C.c_void_p(vals_ptr), C.c_void_p(rhs_ptr), flags)
        self._check(st, "assemble")

    def apply(self, x, y, flags=0):
        self._check(self.L.fem_gpu_apply(self.h, _dev_ptr(x), _dev_ptr(y), flags), "apply")

    def pcg(self, rowptr, colidx, vals, b, x, rel_tol=1e-10, max_iter=100000, jacobi=True):
        o = PcgOpts(rel_tol, max_iter, 1 if jacobi else 0)
        r = PcgReport()
        st = self.L.fem_gpu_pcg(self.h, _dev_ptr(rowptr), _dev_ptr(colidx), _dev_ptr(vals), _dev_ptr(b), _dev_ptr(x),
                                C.byref(o), C.byref(r), 0)
        self._check(st, "pcg")
        return dict(iterations=r.iterations, converged=bool(r.converged), rel_residual=r.rel_residual,
                    seconds=r.seconds)

    def pcg_noalloc(self, rowptr, colidx, vals, b, x, rel_tol=1e-10, max_iter=100000, jacobi=True):
        """fem_gpu_pcg_noalloc: PCG in the library's fixed device array (no
        device allocation; at most 131072 rows)."""
        o = PcgOpts(rel_tol, max_iter, 1 if jacobi else 0)
        r = PcgReport()
        st = self.L.fem_gpu_pcg_noalloc(self.h, _dev_ptr(rowptr), _dev_ptr(colidx), _dev_ptr(vals), _dev_ptr(b),
                                        _dev_ptr(x), C.byref(o), C.byref(r), 0)
        self._check(st, "pcg_noalloc")
        return dict(iterations=r.iterations, converged=bool(r.converged), rel_residual=r.rel_residual,
                    seconds=r.seconds)

    def element_flux(self, s, eq, xi, u):
        """Voigt stress of bulk set s at IP-parametric points: eq (n,) equation
        objects, xi (n, dim), u a CUDA tensor of adof values; returns (n, ncomp)"""
        eqa = np.ascontiguousarray(eq, dtype=np.int64)
        xia = np.ascontiguousarray(xi, dtype=np.float64).reshape(len(eqa), self.dim)
        out = np.zeros(len(eqa) * 6)
        nc = C.c_int32()
        uu = _dev_ptr(u) if not isinstance(u, np.ndarray) else _np_ptr(np.ascontiguousarray(u, dtype=np.float64))
        flags = HOST_BUFFERS
        if not isinstance(u, np.ndarray):
            # u on the device, the result staged back through a host array
            import torch
            o = torch.empty(len(eqa) * 6, dtype=torch.float64, device=u.device)
            self._check(self.L.fem_gpu_element_flux(self.h, s, len(eqa), _np_ptr(eqa), _np_ptr(xia), uu, _dev_ptr(o),
                                                    C.byref(nc), 0), "element_flux")
            return o[:len(eqa) * nc.value].cpu().numpy().reshape(len(eqa), nc.value)
        self._check(self.L.fem_gpu_element_flux(self.h, s, len(eqa), _np_ptr(eqa), _np_ptr(xia), uu, _np_ptr(out),
                                                C.byref(nc), flags), "element_flux")
        return out[:len(eqa) * nc.value].reshape(len(eqa), nc.value)

    def autotune(self, max_elements=0):
        self._check(self.L.fem_gpu_autotune(self.h, max_elements), "autotune")

    def variant(self, s):
        v, ms, name = C.c_int32(), C.c_double(), C.c_char_p()
        self._check(self.L.fem_gpu_get_variant(self.h, s, C.byref(v), C.byref(ms), C.byref(name)), "get_variant")
        return v.value, ms.value, (name.value or b"").decode()

    def set_variant(self, s, v):
        self._check(self.L.fem_gpu_set_variant(self.h, s, v), "set_variant")

    def launch_count(self):
        return self.L.fem_gpu_launch_count(self.h)
