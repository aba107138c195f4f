"""ctypes wrapper of the C++ oracle (test infrastructure only)."""
import ctypes as C
import os

import numpy as np

from . import build as _build

_P = C.c_void_p
_I = C.c_int
_L = C.c_int64
_D = C.c_double

_LIB = None


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


def load():
    """Build (if needed) and load the oracle shared library."""
    global _LIB
    if _LIB is None:
        path = _build.build()
        lib = C.CDLL(path)
        sig = {
            "orc_auto_rule": (_I, [_I, _I]),
            "orc_rule_size": (_I, [_I, _P, _P]),
            "orc_rule": (_I, [_I, _P, _P]),
            "orc_cell_num_nodes": (_I, [_I]),
            "orc_cell_param_dim": (_I, [_I]),
            "orc_shape": (_I, [_I, _P, _P, _P]),
            "orc_bspline_shape": (_D, [_I, _I, _D]),
            "orc_hmr_uniform": (_P, [_I, _P, _P, _I]),
            "orc_mesh_sizes": (None, [_P, _P, _P, _P, _P]),
            "orc_mesh_arrays": (None, [_P, _P, _P, _P, _P, _P]),
            "orc_mesh_free": (None, [_P]),
            "orc_model_create": (_P, [_I, _I, _I, _L, _P, _L, _P, _L, _P, _P, _P]),
            "orc_model_free": (None, [_P]),
            "orc_model_add_bulk_set": (_I, [_P, _I, _I, _I, _L, _P, _P, _P, _P, _P, _D]),
            "orc_model_add_side_set": (_I, [_P, _I, _I, _I, _L, _P, _P, _P, _D, _D, _P]),
            "orc_model_set_density": (_I, [_P, _I, _P, _D]),
            "orc_model_add_double_side_set": (_I, [_P, _I, _I, _I, _I, _L, _P, _P, _P, _P, _P, _P, _P, _P, _D,
                                                   _D]),
            "orc_model_set_bulk_thickness": (_I, [_P, _I, _D]),
            "orc_model_set_side_options": (_I, [_P, _I, _D, _P]),
            "orc_element_flux": (_I, [_P, _I, _L, _P, _P, _P, _P]),
            "orc_model_finalize": (_I, [_P]),
            "orc_model_update_ig": (_I, [_P, _I, _L, _P, _P]),
            "orc_model_update_facets": (_I, [_P, _I, _L, _P, _P, _P]),
            "orc_model_num_adofs": (_L, [_P]),
            "orc_model_nnz": (_L, [_P]),
            "orc_model_num_sets": (_I, [_P]),
            "orc_model_num_eq": (_L, [_P, _I]),
            "orc_graph": (_I, [_P, _P, _P]),
            "orc_element_topology": (_I, [_P, _I, _L, _P, _P]),
            "orc_element_matrices": (_I, [_P, _I, _L, _P, _P, _P]),
            "orc_element_pdof_matrices": (_I, [_P, _I, _L, _P, _P, _P, _P]),
            "orc_assemble": (_I, [_P, _P, _P, _P, _I, _L, _I]),
            "orc_pcg": (_I, [_L, _P, _P, _P, _P, _P, _D, _I, _I, _P, _P]),
            "orc_pcg_mt": (_I, [_L, _P, _P, _P, _P, _P, _D, _I, _I, _P, _P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _LIB = lib
    return _LIB


class OracleLib:
    """Reference-element tables and shape functions."""

    def __init__(self):
        self.lib = load()

    def auto_rule(self, kind, cell):
        """the reference's automatic integration rule (kind 0 bulk, 1 side, 2 double)"""
        return self.lib.orc_auto_rule(kind, cell)

    def rule(self, rule):
        dim, n = C.c_int(), C.c_int()
        assert self.lib.orc_rule_size(rule, C.byref(dim), C.byref(n)) == 0
        pts = np.zeros(dim.value * n.value)
        w = np.zeros(n.value)
        self.lib.orc_rule(rule, _ptr(pts), _ptr(w))
        return pts.reshape(n.value, dim.value).T.copy(), w

    def shape(self, cell, xi):
        n = self.lib.orc_cell_num_nodes(cell)
        pd = self.lib.orc_cell_param_dim(cell)
        xi = np.ascontiguousarray(xi, dtype=np.float64)
        N = np.zeros(n)
        dN = np.zeros(pd * n)
        self.lib.orc_shape(cell, _ptr(xi), _ptr(N), _ptr(dN))
        return N, dN.reshape(n, pd).T.copy()

    def bspline_shape(self, order, basis, xi):
        return self.lib.orc_bspline_shape(order, basis, xi)

    def hmr_uniform(self, dim, nelem, length, order):
        """Uniform level-0 HMR mesh: (coords, cells, num_bases, t_off, t_bases, t_w)."""
        ne = np.asarray(list(nelem) + [1] * (3 - len(nelem)), dtype=np.int32)
        ln = np.asarray(list(length) + [1.0] * (3 - len(length)), dtype=np.float64)
        h = self.lib.orc_hmr_uniform(dim, _ptr(ne), _ptr(ln), order)
        assert h
        nn, nc, nb, nz = (C.c_int64() for _ in range(4))
        self.lib.orc_mesh_sizes(h, C.byref(nn), C.byref(nc), C.byref(nb), C.byref(nz))
        npe = 4 if dim == 2 else 8
        coords = np.zeros(nn.value * dim)
        cells = np.zeros(nc.value * npe, dtype=np.int32)
        t_off = np.zeros(nn.value + 1, dtype=np.int64)
        t_b = np.zeros(nz.value, dtype=np.int32)
        t_w = np.zeros(nz.value)
        self.lib.orc_mesh_arrays(h, _ptr(coords), _ptr(cells), _ptr(t_off), _ptr(t_b), _ptr(t_w))
        self.lib.orc_mesh_free(h)
        return dict(coords=coords.reshape(-1, dim), cells=cells.reshape(-1, npe), num_bases=nb.value,
                    t_off=t_off, t_bases=t_b, t_w=t_w)


class OracleModel:
    """Restated Solver_Interface path over one mesh (see fem_oracle.h)."""

    def __init__(self, dim, ip_cell, shape, mesh):
        self.lib = load()
        self.dim = dim
        self._keep = []
        coords = np.ascontiguousarray(mesh["coords"], dtype=np.float64).ravel()
        cells = np.ascontiguousarray(mesh["cells"], dtype=np.int32).ravel()
        t_off = np.ascontiguousarray(mesh["t_off"], dtype=np.int64)
        t_b = np.ascontiguousarray(mesh["t_bases"], dtype=np.int32)
        t_w = np.ascontiguousarray(mesh["t_w"], dtype=np.float64)
        self.h = self.lib.orc_model_create(dim, ip_cell, shape, len(coords) // dim, _ptr(coords),
                                           len(mesh["cells"]), _ptr(cells), int(mesh["num_bases"]),
                                           _ptr(t_off), _ptr(t_b), _ptr(t_w))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_model_free(self.h)
            self.h = None

    def add_bulk_set(self, ig_cell, rule, model, ip_cells, E, nu, ig_offsets=None, ig_coords=None,
                     ig_param=None):
        ipc = np.ascontiguousarray(ip_cells, dtype=np.int32)
        E = np.ascontiguousarray(E, dtype=np.float64)
        off = None if ig_offsets is None else np.ascontiguousarray(ig_offsets, dtype=np.int64)
        xc = None if ig_coords is None else np.ascontiguousarray(ig_coords, dtype=np.float64)
        xp = None if ig_param is None else np.ascontiguousarray(ig_param, dtype=np.float64)
        r = self.lib.orc_model_add_bulk_set(self.h, ig_cell, rule, model, len(ipc), _ptr(ipc), _ptr(off),
                                            _ptr(xc), _ptr(xp), _ptr(E), nu)
        assert r == 0

    def add_double_side_set(self, iwg, facet_cell, rule, model, leader, follower, offsets, coords, leader_param,
                            follower_param, EL, EF, nu, alpha):
        arrs = [np.ascontiguousarray(leader, dtype=np.int32), np.ascontiguousarray(follower, dtype=np.int32),
                np.ascontiguousarray(offsets, dtype=np.int64)]
        arrs += [np.ascontiguousarray(a, dtype=np.float64) for a in (coords, leader_param, follower_param, EL, EF)]
        r = self.lib.orc_model_add_double_side_set(self.h, iwg, facet_cell, rule, model, len(arrs[0]),
                                                   *[_ptr(a) for a in arrs], nu, alpha)
        assert r == 0

    def update_ig(self, s, eq, coords, param):
        c = np.ascontiguousarray(coords, dtype=np.float64)
        p = np.ascontiguousarray(param, dtype=np.float64)
        assert self.lib.orc_model_update_ig(self.h, s, eq, _ptr(c), _ptr(p)) == 0

    def update_facets(self, s, eq, coords, lparam, fparam):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (coords, lparam, fparam)]
        assert self.lib.orc_model_update_facets(self.h, s, eq, *[_ptr(a) for a in arrs]) == 0

    def set_density(self, s, node_rho, beta=3.0):
        rho = np.ascontiguousarray(node_rho, dtype=np.float64)
        self._keep.append(rho)
        assert self.lib.orc_model_set_density(self.h, s, _ptr(rho), beta) == 0

    def add_side_set(self, iwg, rule, model, ip_cells, ordinals, E, nu, alpha, value):
        ipc = np.ascontiguousarray(ip_cells, dtype=np.int32)
        ords = np.ascontiguousarray(ordinals, dtype=np.int32)
        E = np.ascontiguousarray(E, dtype=np.float64)
        v = np.zeros(3)
        v[:len(value)] = value
        r = self.lib.orc_model_add_side_set(self.h, iwg, rule, model, len(ipc), _ptr(ipc), _ptr(ords),
                                            _ptr(E), nu, alpha, _ptr(v))
        assert r == 0

    def set_bulk_thickness(self, bulk_set, thickness):
        assert self.lib.orc_model_set_bulk_thickness(self.h, bulk_set, thickness) == 0

    def set_side_options(self, side_set, thickness=1.0, select=None):
        """Thickness and Select properties of the side_set-th side set"""
        sel = None if select is None else np.ascontiguousarray(select, dtype=np.float64).ravel()
        assert self.lib.orc_model_set_side_options(self.h, side_set, thickness, _ptr(sel)) == 0

    def element_flux(self, s, eq, xi, u_adof):
        """Voigt stress of a bulk equation object at IP-parametric point xi"""
        out = np.zeros(6)
        n = C.c_int32()
        x = np.ascontiguousarray(xi, dtype=np.float64)
        u = np.ascontiguousarray(u_adof, dtype=np.float64)
        assert self.lib.orc_element_flux(self.h, s, eq, _ptr(x), _ptr(u), _ptr(out), C.byref(n)) == 0
        return out[:n.value].copy()

    def finalize(self):
        assert self.lib.orc_model_finalize(self.h) == 0
        self.num_adofs = self.lib.orc_model_num_adofs(self.h)
        self.nnz = self.lib.orc_model_nnz(self.h)

    def graph(self):
        rp = np.zeros(self.num_adofs + 1, dtype=np.int32)
        ci = np.zeros(self.nnz, dtype=np.int32)
        assert self.lib.orc_graph(self.h, _ptr(rp), _ptr(ci)) == 0
        return rp, ci

    def num_sets(self):
        return self.lib.orc_model_num_sets(self.h)

    def num_eq(self, s):
        return self.lib.orc_model_num_eq(self.h, s)

    def element_topology(self, s, eq):
        ids = np.zeros(512, dtype=np.int32)
        n = C.c_int32()
        assert self.lib.orc_element_topology(self.h, s, eq, _ptr(ids), C.byref(n)) == 0
        return ids[:n.value].copy()

    def element_matrices(self, s, eq, u_adof=None):
        n = len(self.element_topology(s, eq))
        K = np.zeros(n * n)
        R = np.zeros(n)
        u = None if u_adof is None else np.ascontiguousarray(u_adof, dtype=np.float64)
        assert self.lib.orc_element_matrices(self.h, s, eq, _ptr(u), _ptr(K), _ptr(R)) == 0
        return K.reshape(n, n).T.copy(), R  # column-major -> K[i, j]

    def element_pdof_matrices(self, s, eq, u_pdof=None):
        K = np.zeros(512 * 512)
        R = np.zeros(512)
        n = C.c_int32()
        u = None if u_pdof is None else np.ascontiguousarray(u_pdof, dtype=np.float64)
        assert self.lib.orc_element_pdof_matrices(self.h, s, eq, _ptr(u), _ptr(K), _ptr(R), C.byref(n)) == 0
        m = n.value
        return K[:m * m].reshape(m, m).T.copy(), R[:m].copy()

    def assemble(self, u_adof=None, nthreads=1, eq_stride=1, out=None):
        """Assemble into fresh arrays, or accumulate into out=(vals, rhs)."""
        if out is None:
            vals = np.zeros(self.nnz)
            rhs = np.zeros(self.num_adofs)
        else:
            vals, rhs = out
        u = None if u_adof is None else np.ascontiguousarray(u_adof, dtype=np.float64)
        assert self.lib.orc_assemble(self.h, _ptr(u), _ptr(vals), _ptr(rhs), nthreads, eq_stride, 0) == 0
        return vals, rhs


def pcg(rowptr, colidx, vals, b, rtol=1e-10, max_iter=100000, jacobi=True, x0=None):
    lib = load()
    n = len(b)
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    it = C.c_int()
    rr = C.c_double()
    rc = lib.orc_pcg(n, _ptr(np.ascontiguousarray(rowptr, dtype=np.int32)),
                     _ptr(np.ascontiguousarray(colidx, dtype=np.int32)),
                     _ptr(np.ascontiguousarray(vals, dtype=np.float64)),
                     _ptr(np.ascontiguousarray(b, dtype=np.float64)), _ptr(x), rtol, max_iter,
                     1 if jacobi else 0, C.byref(it), C.byref(rr))
    return x, it.value, rr.value, rc


def pcg_mt(rowptr, colidx, vals, b, rtol=1e-10, max_iter=100000, nthreads=1, x0=None):
    """Jacobi-PCG with its loops on nthreads host threads; (x, iterations, rel_res, rc)"""
    lib = load()
    n = len(b)
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    it = C.c_int()
    rr = C.c_double()
    rc = lib.orc_pcg_mt(n, _ptr(np.ascontiguousarray(rowptr, dtype=np.int32)),
                        _ptr(np.ascontiguousarray(colidx, dtype=np.int32)),
                        _ptr(np.ascontiguousarray(vals, dtype=np.float64)),
                        _ptr(np.ascontiguousarray(b, dtype=np.float64)), _ptr(x), rtol, max_iter, nthreads,
                        C.byref(it), C.byref(rr))
    return x, it.value, rr.value, rc
