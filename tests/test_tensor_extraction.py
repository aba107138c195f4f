"""The tensor-product structure that the bulk kernel's fast path relies on,
checked on the host (no GPU): on a uniform quadratic B-spline mesh every
element's extraction T (8 corner nodes x 27 bases) is P / 8, P the 0/1 pattern
of the node sets (x left / both / right) x (y) x (z); and the kernel's staged
sums reproduce T^T K T: K T / 8 = (K / 64) P summed axis by axis (8 node
values -> 12 -> 18 -> 27) and T^T K T = P^T ((K / 64) P)."""
import numpy as np

import moris_gb300 as mg

# HEX8 corner nodes: x left {0,3,4,7}, right {1,2,5,6}; y left {0,1,4,5}, right
# {2,3,6,7}; z left {0..3}, right {4..7}
LEFT = [0x99, 0x33, 0x0F]
RIGHT = [0x66, 0xCC, 0xF0]


def element_t(mesh, cell):
    """8 x nb extraction of one cell from the node rows, bases in first-seen order."""
    off, bases, w = mesh["t_off"], mesh["t_bases"], mesh["t_w"]
    nodes = mesh["cells"][cell]
    cols = []
    for a in nodes:
        for b in bases[off[a]:off[a + 1]]:
            if b not in cols:
                cols.append(int(b))
    T = np.zeros((8, len(cols)))
    for k, a in enumerate(nodes):
        for b, t in zip(bases[off[a]:off[a + 1]], w[off[a]:off[a + 1]]):
            T[k, cols.index(int(b))] = t
    return T


def tensor_codes(T):
    """natural code jx + 3 jy + 9 jz of every column, or None when T is not P/8"""
    if T.shape[1] != 27:
        return None
    codes = []
    for j in range(27):
        mask = sum(1 << a for a in range(8) if T[a, j] != 0.0)
        if mask == 0 or np.any((T[:, j] != 0.0) & (T[:, j] != 0.125)):
            return None
        expect, nat = 0xFF, 0
        for d, mul in zip(range(3), (1, 3, 9)):
            c = (1 if mask & RIGHT[d] else 0) if mask & LEFT[d] else 2
            expect &= LEFT[d] if c == 0 else RIGHT[d] if c == 2 else 0xFF
            nat += c * mul
        if mask != expect:
            return None
        codes.append(nat)
    return codes if sorted(codes) == list(range(27)) else None


def test_every_element_of_a_uniform_quadratic_mesh_is_a_tensor_product():
    ne = (7, 6, 5)
    mesh = mg.hmr_uniform_mesh(3, ne, [1.0, 1.0, 1.0], 2)
    for cell in range(len(mesh["cells"])):
        assert tensor_codes(element_t(mesh, cell)) is not None, cell


def test_linear_and_cubic_extractions_are_not():
    for p in (1, 3):
        mesh = mg.hmr_uniform_mesh(3, (3, 3, 3), [1.0, 1.0, 1.0], p)
        assert tensor_codes(element_t(mesh, 13)) is None


def staged_kt(K64, codes):
    """(K / 64) P column by column as the kernel forms it: y stage for each jy,
    then x, then z; K64 is 24 x 24 with rows / columns (field, node)."""
    KT = np.zeros((24, 81))
    slot = {nat: j for j, nat in enumerate(codes)}
    for r in range(24):
        for g in range(3):
            v = K64[r, g * 8:(g + 1) * 8]
            for jy in range(3):
                w = np.zeros((2, 2))
                for bz in range(2):
                    for bx in range(2):
                        v0 = v[4 * bz + (1 if bx else 0)]   # by = 0
                        v1 = v[4 * bz + (2 if bx else 3)]   # by = 1
                        w[bx, bz] = v0 if jy == 0 else v1 if jy == 2 else v0 + v1
                for jx in range(3):
                    u0 = w[0, 0] if jx == 0 else w[1, 0] if jx == 2 else w[0, 0] + w[1, 0]
                    u1 = w[0, 1] if jx == 0 else w[1, 1] if jx == 2 else w[0, 1] + w[1, 1]
                    for jz, val in ((0, u0), (1, u0 + u1), (2, u1)):
                        KT[r, slot[jx + 3 * jy + 9 * jz] * 3 + g] = val
    return KT


def test_staged_sums_reproduce_the_element_matrix():
    mesh = mg.hmr_uniform_mesh(3, (4, 4, 4), [1.0, 1.0, 1.0], 2)
    T = element_t(mesh, 21)
    codes = tensor_codes(T)
    rng = np.random.default_rng(4)
    A = rng.standard_normal((24, 24))
    K = A + A.T                                  # rows / columns (field f, node a): f * 8 + a
    Tf = np.zeros((24, 81))                      # T per field: adof (basis j, field g) = j * 3 + g
    for g in range(3):
        Tf[g * 8:(g + 1) * 8, g::3] = T
    ref = Tf.T @ K @ Tf
    KT = staged_kt(K / 64.0, codes)              # = K T / 8
    # T^T K T = P^T ((K/64) P): a plain sum over each column's nodes
    P = (T != 0.0).astype(float)
    Pf = np.zeros((24, 81))
    for g in range(3):
        Pf[g * 8:(g + 1) * 8, g::3] = P
    assert np.allclose(KT, (K @ Tf) / 8.0, rtol=0, atol=1e-14 * np.abs(K).max())
    KA = Pf.T @ KT
    assert np.allclose(KA, ref, rtol=0, atol=1e-14 * np.abs(ref).max())
