"""CPU restatement of the geometric multigrid V-cycle (test infrastructure:
only tests and the benchmark's CPU leg use it, as the checker).

It follows the reference's PCMG preconditioner (SOL/DLA/src/
cl_DLA_Preconditioner_PETSc.cpp:77-345): a multiplicative V-cycle with
Galerkin coarse operators A_(l+1) = P^T A_l P (PC_MG_GALERKIN_BOTH) and the
prolongation of the B-spline two-scale relation (Geometric_Multigrid,
SOL/DLA/src/cl_DLA_Geometric_Multigrid.cpp:47-121), which for linear
B-splines on nested uniform grids is trilinear interpolation with weights
1 / 1/2 per direction.  Smoother and coarsest solve are the product's
(Chebyshev-accelerated point Jacobi, dense inverse) so that both compute the
same operator V; the reference's own SOR smoother and LU coarse solve differ
from them by design.

Vectors are type-major like the adof vector: v[g * n^3 + x + n (y + n z)].
"""
import numpy as np
import scipy.sparse as sp

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)


def splitmix_uniform(seed, m):
    """element t: splitmix64 of seed + (t+1) * golden, top 53 bits in [0, 1), minus 1/2"""
    with np.errstate(over="ignore"):
        i = np.arange(1, m + 1, dtype=np.uint64)
        z = np.uint64(seed) + i * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0) - 0.5


def prolongation_1d(nf):
    nc = (nf - 1) // 2 + 1
    rows, cols, vals = [], [], []
    for i in range(nf):
        if i % 2 == 0:
            rows.append(i)
            cols.append(i // 2)
            vals.append(1.0)
        else:
            rows += [i, i]
            cols += [(i - 1) // 2, (i + 1) // 2]
            vals += [0.5, 0.5]
    return sp.csr_matrix((vals, (rows, cols)), shape=(nf, nc))


def prolongation(nf):
    """P for the 3-component type-major vector of an nf^3 node grid"""
    p = prolongation_1d(nf)
    return sp.kron(sp.identity(3), sp.kron(p, sp.kron(p, p))).tocsr()


def grid_levels(nf, coarse_max):
    ns = [nf]
    while ns[-1] > coarse_max:
        assert (ns[-1] - 1) % 2 == 0
        ns.append((ns[-1] - 1) // 2 + 1)
    return ns


def stencil(A, n):
    """[27][3][3][n^3] block stencil of a nodal operator (tap k = (dx+1) + 3 (dy+1) + 9 (dz+1))"""
    A = A.tocoo()
    N = n ** 3
    f, i = np.divmod(A.row, N)
    g, j = np.divmod(A.col, N)
    ix, iy, iz = i % n, (i // n) % n, i // (n * n)
    jx, jy, jz = j % n, (j // n) % n, j // (n * n)
    k = (jx - ix + 1) + 3 * (jy - iy + 1) + 9 * (jz - iz + 1)
    S = np.zeros((27, 3, 3, N))
    np.add.at(S, (k, f, g, i), A.data)
    return S


class Hierarchy:
    def __init__(self, A, nf, coarse_max=9, degree=2, lo_frac=0.1, hi_frac=1.1, power_iters=12):
        self.ns = grid_levels(nf, coarse_max)
        self.A = [sp.csr_matrix(A)]
        self.P = []
        for n in self.ns[:-1]:
            P = prolongation(n)
            self.P.append(P)
            self.A.append((P.T @ self.A[-1] @ P).tocsr())
        self.dinv = []
        for a in self.A:
            d = a.diagonal()
            self.dinv.append(np.where(d != 0.0, 1.0 / np.where(d != 0.0, d, 1.0), 0.0))
        self.degree, self.lo, self.hi = degree, lo_frac, hi_frac
        self.lmax = [self._power(l, power_iters) for l in range(len(self.ns) - 1)] + [0.0]
        self.ainv = np.linalg.inv(self.A[-1].toarray())

    def _power(self, l, iters):
        x = splitmix_uniform(0x5EED + l, self.A[l].shape[0])
        xn = np.linalg.norm(x)
        lam = 0.0
        for _ in range(iters):
            y = self.dinv[l] * (self.A[l] @ x)
            yn = np.linalg.norm(y)
            lam = yn / xn
            x = y / yn
            xn = 1.0
        return lam

    def _cheb(self, l):
        lo, hi = self.lo * self.lmax[l], self.hi * self.lmax[l]
        theta, delta = 0.5 * (hi + lo), 0.5 * (hi - lo)
        return theta, delta, theta / delta

    def _steps(self, l, r, d, x, sigma, delta):
        A, dinv = self.A[l], self.dinv[l]
        rho = 1.0 / sigma
        for _ in range(1, self.degree):
            rn = 1.0 / (2.0 * sigma - rho)
            r = r - A @ d
            d = rn * rho * d + (2.0 * rn / delta) * dinv * r
            x = x + d
            rho = rn
        return r, d, x

    def vcycle(self, b, l=0):
        if l == len(self.ns) - 1:
            return self.ainv @ b
        A, dinv = self.A[l], self.dinv[l]
        theta, delta, sigma = self._cheb(l)
        # pre-smoothing from x = 0, residual kept as b - A x
        r = b.copy()
        d = dinv * b / theta
        x = d.copy()
        r, d, x = self._steps(l, r, d, x, sigma, delta)
        r = r - A @ d
        e = self.P[l] @ self.vcycle(self.P[l].T @ r, l + 1)
        # post-smoothing: the first step folds in the coarse correction
        r = r - A @ e
        d = dinv * r / theta
        x = x + e + d
        r, d, x = self._steps(l, r, d, x, sigma, delta)
        return x


def pcg(A, b, apply_m, rel_tol=1e-8, max_iter=10000):
    """preconditioned CG; returns (x, iterations)"""
    x = np.zeros_like(b)
    r = b.copy()
    z = apply_m(r)
    p = z.copy()
    rz = r @ z
    bn = np.linalg.norm(b)
    for it in range(1, max_iter + 1):
        q = A @ p
        a = rz / (p @ q)
        x += a * p
        r -= a * q
        if np.linalg.norm(r) <= rel_tol * bn:
            return x, it
        z = apply_m(r)
        rz_new = r @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
    return x, max_iter
