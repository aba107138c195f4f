"""Hierarchical (refined) HMR B-spline meshes restated in numpy -- TEST
INFRASTRUCTURE ONLY (the checker of moris_gb300's fem_hmr_refined_* entry
points; pinned on the reference's T-Matrix_test_values.hdf5 fixture).

What it restates, by reference file:
* the background mesh: a domain of ne elements per direction surrounded by
  `padding` elements (HMR/src/cl_HMR_Parameters.cpp:418-423), children by
  bisection; padding elements are never active and carry the refined flag on
  every pattern, but have children only where they were refined
  (Background_Element_Base::set_padding_flag, cl_HMR_Background_Element_Base.
  hpp:225-249; their owner is no processor);
* perform_refinement (cl_HMR_Background_Mesh_Base.cpp:648-737): the queued
  elements, the padding test of every queued element owned by the processor
  (cl_HMR_Background_Mesh.hpp:1101-1145: an element within `padding_refinement`
  of the domain boundary queues its padding neighbours within that distance),
  the staircase buffer (cl_HMR_Background_Mesh_Base.cpp:1383-1495: the active
  coarser neighbours, within half the buffer, of a queued element's parent are
  queued when their nearest child is within `buffer` elements), repeated
  until the queue stops growing;
* the B-spline basis states of BSpline_Mesh::determine_basis_state
  (cl_HMR_BSpline_Mesh.hpp:738-807): deactivated unless all (p+1)^d elements of
  its support exist and are active or refined; active if any is active,
  refined otherwise;
* T_Matrix_Base::calculate_untruncated_t_matrix / calculate_truncated_t_matrix
  (cl_HMR_T_Matrix_Base.cpp:58-248) with the child matrices of the uniform
  B-spline two-scale relation (children 2m-p+j, weights 2^-p C(p+1, j)) and
  the element-local basis order of the B-spline elements
  (cl_HMR_BSpline_Element_{Quad4,Quad9,Quad16,Hex8,Hex27,Hex64}.hpp,
  get_ijk_of_basis);
* the node extraction rows of T_Matrix_Base::evaluate (cl_HMR_T_Matrix_Base.
  cpp:306-457): the element T evaluated at the Lagrange (corner) nodes,
  entries with |t| <= 1e-12 dropped, the first element that visits a node
  sets its row.

Indices: element and basis ijk are counted from the first padding element, a
level-l basis m has the support elements m-p .. m per direction.
"""
import itertools
import math

import numpy as np

# element-local basis order of HMR's B-spline elements, ijk offsets per local index
_LOCAL = {
    (2, 1): "00 10 11 01",
    (2, 2): "00 20 22 02 10 21 12 01 11",
    (2, 3): "00 30 33 03 10 20 31 32 23 13 02 01 11 21 22 12",
    (3, 1): "000 100 110 010 001 101 111 011",
    (3, 2): "000 200 220 020 002 202 222 022 100 210 120 010 001 201 221 021 102 212 122 012 111 110 112 011 211 "
            "101 121",
    (3, 3): "000 300 330 030 003 303 333 033 100 200 010 020 001 002 310 320 301 302 230 130 331 332 031 032 103 "
            "203 013 023 313 323 233 133 110 120 220 210 101 201 202 102 011 012 022 021 311 321 322 312 231 131 "
            "132 232 113 213 223 123 111 211 221 121 112 212 222 122",
}


def local_order(dim, p):
    return [tuple(int(c) for c in w) for w in _LOCAL[(dim, p)].split()]


class RefinedMesh:
    def __init__(self, dim, ne, lengths, p, buffer=None, padding_refinement=None, padding=None):
        self.d, self.p = dim, p
        self.ne = tuple(ne)
        self.len = tuple(lengths)
        self.buf = p if buffer is None else buffer
        self.pad = max(self.buf, p) if padding is None else padding
        self.pr = math.ceil(0.5 * p) if padding_refinement is None else padding_refinement
        self.hb = math.ceil(0.5 * self.buf)
        self.refined = [set() for _ in range(16)]
        self.local = local_order(dim, p)

    # ---- background mesh ----------------------------------------------------
    def count(self, l, k):
        return (self.ne[k] + 2 * self.pad) * 2 ** l

    def exists(self, l, e):
        if any(c < 0 or c >= self.count(l, k) for k, c in enumerate(e)):
            return False
        return l == 0 or tuple(c // 2 for c in e) in self.refined[l - 1]

    def padding(self, l, e):
        return any(c < self.pad * 2 ** l or c >= (self.pad + self.ne[k]) * 2 ** l for k, c in enumerate(e))

    def active(self, l, e):
        return self.exists(l, e) and e not in self.refined[l] and not self.padding(l, e)

    def neighbours(self, l, e, r):
        for off in itertools.product(range(-r, r + 1), repeat=self.d):
            if any(off):
                f = tuple(c + o for c, o in zip(e, off))
                if self.exists(l, f):
                    yield f

    def refine(self, elements):
        """one perform_refinement over the queued (level, ijk) elements"""
        q = set((l, tuple(e)) for l, e in elements)

        def padding_test():
            new = set()
            for l, e in q:
                if self.padding(l, e):
                    continue  # padding elements belong to no processor
                lo = [self.pad * 2 ** l] * self.d
                hi = [(self.pad + self.ne[k]) * 2 ** l - 1 for k in range(self.d)]
                if any(e[k] < lo[k] + self.pr or e[k] > hi[k] - self.pr for k in range(self.d)):
                    for f in self.neighbours(l, e, self.pr):
                        if self.padding(l, f) and (l, f) not in q:
                            new.add((l, f))
            return new

        def staircase(l, e):
            if l == 0:
                return
            par = tuple(c // 2 for c in e)
            for f in self.neighbours(l - 1, par, self.hb):
                if self.active(l - 1, f) and (l - 1, f) not in q:
                    dist = max((2 * f[k] - e[k]) if 2 * f[k] >= e[k] else (e[k] - 2 * f[k] - 1)
                               for k in range(self.d))
                    if dist <= self.buf:
                        q.add((l - 1, f))
                        staircase(l - 1, f)

        q |= padding_test()
        while True:
            n = len(q)
            for l, e in list(q):
                staircase(l, e)
            q |= padding_test()
            if len(q) == n:
                break
        for l, e in q:
            self.refined[l].add(e)

    def max_level(self):
        return max([l + 1 for l in range(16) if self.refined[l]], default=0)

    # ---- B-spline bases ----------------------------------------------------------
    def basis_state(self, l, m):
        els = [tuple(c - o for c, o in zip(m, off)) for off in itertools.product(range(self.p + 1), repeat=self.d)]
        if not all(self.exists(l, e) for e in els):
            return "deactivated"
        return "active" if any(self.active(l, e) for e in els) else "refined"

    def element_bases(self, l, e):
        return [tuple(c + o for c, o in zip(e, off)) for off in self.local]

    def children(self, m):
        out = []
        for js in itertools.product(range(self.p + 2), repeat=self.d):
            w = 1.0
            for j in js:
                w *= math.comb(self.p + 1, j) / 2.0 ** self.p
            out.append((tuple(2 * mi - self.p + j for mi, j in zip(m, js)), w))
        return out

    def child_matrix(self, l, e):
        """C[i][k]: the child element's local basis i in the parent's local basis k"""
        par = tuple(c // 2 for c in e)
        idx = {b: i for i, b in enumerate(self.element_bases(l, e))}
        pb = self.element_bases(l - 1, par)
        C = np.zeros((len(idx), len(pb)))
        for k, m in enumerate(pb):
            for c, w in self.children(m):
                if c in idx:
                    C[idx[c], k] += w
        return C

    def element_t_matrix(self, l, e, truncate):
        """(T [local bases x dofs], [(level, basis ijk)] of the dofs)"""
        B = len(self.local)
        cols, dofs = [], []
        if not truncate:
            T = np.eye(B)
            el = tuple(e)
            for lev in range(l, -1, -1):
                for k, m in enumerate(self.element_bases(lev, el)):
                    if self.basis_state(lev, m) == "active":
                        cols.append(T[:, k].copy())
                        dofs.append((lev, m))
                if lev > 0:
                    T = T @ self.child_matrix(lev, el)
                    el = tuple(c // 2 for c in el)
        else:
            mine = self.element_bases(l, e)
            for k, m in enumerate(mine):
                if self.basis_state(l, m) == "active":
                    c = np.zeros(B)
                    c[k] = 1.0
                    cols.append(c)
                    dofs.append((l, m))
            if l > 0:
                idx = {b: i for i, b in enumerate(mine)}
                for m in self.element_bases(l - 1, tuple(c // 2 for c in e)):
                    if self.basis_state(l - 1, m) != "active":
                        continue
                    c = np.zeros(B)
                    for ch, w in self.children(m):
                        if ch in idx and self.basis_state(l, ch) == "deactivated":
                            c[idx[ch]] += w
                    if c.min() < -1e-12 or c.max() > 1e-12:
                        cols.append(c)
                        dofs.append((l - 1, m))
        T = np.array(cols).T if cols else np.zeros((B, 0))
        return T, dofs

    # ---- Lagrange mesh with node extraction rows ------------------------------------
    def leaves(self):
        """active domain elements: coarsest domain elements in lexicographic order
        (x fastest), each followed by its active descendants, children in child
        order (x fastest)"""
        out = []

        def visit(l, e):
            if e in self.refined[l]:
                for off in itertools.product(range(2), repeat=self.d):
                    off = off[::-1]
                    visit(l + 1, tuple(2 * c + o for c, o in zip(e, off)))
            else:
                out.append((l, e))

        for ijk in itertools.product(*[range(self.pad, self.pad + n) for n in self.ne[::-1]]):
            visit(0, tuple(ijk[::-1]))
        return out

    def bspline_value(self, lev, m, x):
        """value of the level-lev basis m at the physical point x"""
        v = 1.0
        for k in range(self.d):
            h = self.len[k] / self.ne[k] / 2 ** lev
            t = (x[k] + self.pad * self.len[k] / self.ne[k]) / h - (m[k] - self.p)
            v *= _cardinal(self.p, t)
        return v

    def lagrange_mesh(self, truncate):
        """dict(coords, cells, num_bases, t_off, t_bases, t_w) of the active domain
        elements as QUAD4 / HEX8 cells; basis ids by (level, ijk x fastest) over
        the active bases; nodes numbered by first visit"""
        L = max(self.max_level(), 0)
        corners = [(0, 0), (1, 0), (1, 1), (0, 1)] if self.d == 2 else \
            [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
        leaves = self.leaves()
        node_id, coords, rows, cells = {}, [], [], []
        used = set()
        elem_t = []
        for l, e in leaves:
            T, dofs = self.element_t_matrix(l, e, truncate)
            elem_t.append((T, dofs))
            used.update(dofs)
        order = sorted(used, key=lambda b: (b[0],) + tuple(b[1][::-1]))
        bid = {b: i for i, b in enumerate(order)}
        for (l, e), (T, dofs) in zip(leaves, elem_t):
            cell = []
            for c in corners:
                key = tuple((ei + ci) * 2 ** (L - l) for ei, ci in zip(e, c))
                if key not in node_id:
                    h = [self.len[k] / self.ne[k] / 2 ** L for k in range(self.d)]
                    x = [(key[k] - self.pad * 2 ** L) * h[k] for k in range(self.d)]
                    node_id[key] = len(coords)
                    coords.append(x)
                    # element local B-splines at the node (the Lagrange matrix row), times T
                    lb = self.element_bases(l, e)
                    lag = np.array([self.bspline_value(l, m, x) for m in lb])
                    t = lag @ T
                    rows.append([(bid[dofs[j]], t[j]) for j in range(len(dofs)) if abs(t[j]) > 1e-12])
                cell.append(node_id[key])
            cells.append(cell)
        t_off = np.zeros(len(rows) + 1, dtype=np.int64)
        t_off[1:] = np.cumsum([len(r) for r in rows])
        return dict(coords=np.array(coords), cells=np.array(cells, dtype=np.int32), num_bases=len(order),
                    t_off=t_off, t_bases=np.array([b for r in rows for b, _ in r], dtype=np.int32),
                    t_w=np.array([w for r in rows for _, w in r]))


def _cardinal(p, t):
    """uniform cardinal B-spline of degree p on [0, p + 1] (Cox-de Boor)"""
    if p == 0:
        return 1.0 if 0.0 <= t < 1.0 else 0.0
    return (t * _cardinal(p - 1, t) + (p + 1 - t) * _cardinal(p - 1, t - 1)) / p
