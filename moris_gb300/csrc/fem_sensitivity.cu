// fem_sensitivity.cu -- shape sensitivities of the strain energy through the
// level-set coefficients (adjoint method).
//
//   dQ/dp = sum_v G[v] dt_v/dp,   G[v] = d/dt_v ( Q(u, t) - lambda^T R(u, t) ),
//   K^T lambda = dQ/du,
//
// where t_v is the edge coordinate of intersection vertex v
// (x_v = x_p0 + t_v (x_p1 - x_p0)).  The reference assembles dR/dp by finite
// differences of the IG vertex coordinates (IWG::select_dRdp_FD_geometry_bulk,
// FEM/INT/src/IWG/cl_FEM_IWG.cpp:2997-3154, plus the cluster-measure terms
// :3827-3924) and contracts with the adjoint in Interpolation_Element::
// compute_dQIdp_explicit_implicit (FEM/INT/src/ELEM/cl_FEM_Interpolation_
// Element.cpp:820-948).  Here the derivative is exact: every integration
// cell (TET4) and interface facet (TRI3) is evaluated once in forward-mode
// dual arithmetic with one derivative slot per vertex, and the contraction
// with u and lambda happens inside the kernel:
//
//   tet     F = sum_q w detJ (1/2 sigma(u):eps(u) - sigma(u):eps(lambda))
//   facet   -lambda^T R_interface = -( w_L A + w_F B + gamma C ),
//           A = sum_q w* (-[lambda].t_L(u) + beta t_L(lambda).[u]),  B likewise
//           with t_F, C = sum_q w* [lambda].[u]  (IWG_Isotropic_Struc_Linear_
//           Interface residual contracted with lambda), and the SP_Nitsche_
//           Interface weights / gamma differentiated through the cluster
//           volumes (the cut clusters' tets) and the interface measure.
// Rectangular IP cells: xi = -1 + 2 (x - X0) / (X6 - X0).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fem_internal.hpp"

namespace fem {
namespace {

template <int M>
struct Dual {
    double v;
    double d[M];
    __device__ Dual() {}
    __device__ explicit Dual(double x) : v(x) {
        for (int i = 0; i < M; ++i) d[i] = 0.0;
    }
};
template <int M>
__device__ __forceinline__ Dual<M> operator+(const Dual<M>& a, const Dual<M>& b) {
    Dual<M> r;
    r.v = a.v + b.v;
    for (int i = 0; i < M; ++i) r.d[i] = a.d[i] + b.d[i];
    return r;
}
template <int M>
__device__ __forceinline__ Dual<M> operator-(const Dual<M>& a, const Dual<M>& b) {
    Dual<M> r;
    r.v = a.v - b.v;
    for (int i = 0; i < M; ++i) r.d[i] = a.d[i] - b.d[i];
    return r;
}
template <int M>
__device__ __forceinline__ Dual<M> operator*(const Dual<M>& a, const Dual<M>& b) {
    Dual<M> r;
    r.v = a.v * b.v;
    for (int i = 0; i < M; ++i) r.d[i] = fma(a.d[i], b.v, a.v * b.d[i]);
    return r;
}
template <int M>
__device__ __forceinline__ Dual<M> operator*(double s, const Dual<M>& a) {
    Dual<M> r;
    r.v = s * a.v;
    for (int i = 0; i < M; ++i) r.d[i] = s * a.d[i];
    return r;
}
template <int M>
__device__ __forceinline__ Dual<M> operator+(double s, const Dual<M>& a) {
    Dual<M> r = a;
    r.v += s;
    return r;
}
template <int M>
__device__ __forceinline__ Dual<M> dsqrt(const Dual<M>& a) {
    Dual<M> r;
    r.v = sqrt(a.v);
    const double h = a.v > 0.0 ? 0.5 / r.v : 0.0;
    for (int i = 0; i < M; ++i) r.d[i] = h * a.d[i];
    return r;
}
template <int M>
__device__ __forceinline__ Dual<M> dinv(const Dual<M>& a) {
    Dual<M> r;
    r.v = 1.0 / a.v;
    const double h = -r.v * r.v;
    for (int i = 0; i < M; ++i) r.d[i] = h * a.d[i];
    return r;
}
// a += s * b (s constant)
template <int M>
__device__ __forceinline__ void axpy(double s, const Dual<M>& b, Dual<M>& a) {
    a.v = fma(s, b.v, a.v);
    for (int i = 0; i < M; ++i) a.d[i] = fma(s, b.d[i], a.d[i]);
}

// A trilinear field of a rectangular HEX8 cell (nodal values f_a, shape
// functions N_a = (1 + s_x xi)(1 + s_y eta)(1 + s_z zeta) / 8) written as a
// polynomial in the physical offsets (x, y, z) from the cell centre:
//   f = k0 + k1 x + k2 y + k3 z + k4 xy + k5 yz + k6 xz + k7 xyz,
// k_m = (1/8) sum_a f_a prod_{d in m} s_d(a) / prod_{d in m} jd_d  (jd the half
// edge lengths).  Its gradient needs only the pair products:
//   df/dx = k1 + k4 y + k6 z + k7 yz,  df/dy = k2 + k4 x + k5 z + k7 xz,
//   df/dz = k3 + k6 x + k5 y + k7 xy.
// Monomial m -> the set of coordinates it contains (bit d for coordinate d).
__device__ __forceinline__ int monomial_mask(int m) {
    return m < 4 ? (m == 0 ? 0 : 1 << (m - 1)) : (m == 4 ? 3 : m == 5 ? 6 : m == 6 ? 5 : 7);
}
// coefficient r = comp * 8 + m of the field with nodal values f[comp * 8 + a]
// on the cell X[8][3] (node 0 and node 6 opposite corners)
__device__ double monomial_coefficient(const double* f, const double* X, int r) {
    const int fl = r >> 3, mask = monomial_mask(r & 7);
    double c = 0.0;
    for (int a = 0; a < 8; ++a) {
        const int sx = ((a & 3) == 1 || (a & 3) == 2) ? 1 : -1;
        const int sy = ((a & 3) >= 2) ? 1 : -1;
        const int sz = a >= 4 ? 1 : -1;
        const int sg = ((mask & 1) ? sx : 1) * ((mask & 2) ? sy : 1) * ((mask & 4) ? sz : 1);
        c += sg > 0 ? f[fl * 8 + a] : -f[fl * 8 + a];
    }
    double den = 8.0;
    for (int d = 0; d < 3; ++d)
        if (mask & (1 << d)) den *= 0.5 * (X[18 + d] - X[d]);
    return c / den;
}

// a0 + a1 p + a2 q + a3 r (constant coefficients)
template <int M>
__device__ __forceinline__ Dual<M> lin3(double a0, double a1, const Dual<M>& p, double a2, const Dual<M>& q, double a3,
                                        const Dual<M>& r) {
    Dual<M> o;
    o.v = fma(a3, r.v, fma(a2, q.v, fma(a1, p.v, a0)));
    for (int i = 0; i < M; ++i) o.d[i] = fma(a3, r.d[i], fma(a2, q.d[i], a1 * p.d[i]));
    return o;
}

// gradient grad[comp][d] (and with VAL the value) of a field in monomial form
// k[comp * 8 + m] at the offsets x[3]; pr = {xy, yz, xz}
template <int M, bool VAL>
__device__ __forceinline__ void mono_field(const double* __restrict__ k, const Dual<M> x[3], const Dual<M> pr[3],
                                           Dual<M> val[3], Dual<M> grad[3][3]) {
    for (int fl = 0; fl < 3; ++fl) {
        const double* c = k + fl * 8;
        grad[fl][0] = lin3(c[1], c[4], x[1], c[6], x[2], c[7], pr[1]);
        grad[fl][1] = lin3(c[2], c[4], x[0], c[5], x[2], c[7], pr[2]);
        grad[fl][2] = lin3(c[3], c[6], x[0], c[5], x[1], c[7], pr[0]);
        // k0 + k2 y + k3 z + k5 yz + x df/dx
        if (VAL) val[fl] = lin3(c[0], c[2], x[1], c[3], x[2], c[5], pr[1]) + x[0] * grad[fl][0];
    }
}

// sigma = lam tr(G) I + mu (G + G^T) of a displacement gradient G[f][i] = du_f/dx_i
template <int M>
__device__ void stress(const Dual<M> G[3][3], double lam, double mu, Dual<M> S[3][3]) {
    const Dual<M> tr = G[0][0] + G[1][1] + G[2][2];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            S[i][j] = mu * (G[i][j] + G[j][i]);
            if (i == j) axpy(lam, tr, S[i][j]);
        }
}

struct AdjArgs {
    // vertex table
    const int32_t* vkind;
    const int32_t* vpar;  // [nv][8]
    const double* vx;     // [nv][3]
    double* G;            // [nv]
    // adof vectors
    const double* u;
    const double* lam;
    int64_t nu;
};

struct CutSetDev {
    int64_t neq;
    const double* xe;      // [neq][8][3]
    const double* E;
    const int32_t* nb;
    const int32_t* bases;  // [neq][W]
    const double* T;       // [neq][8][W]
    int W;
    double lam_c, mu_c;
    const int64_t* ig_off;
    const int32_t* vid;    // [ig][4]
    const double* gp;      // TET rule points [ngp][3]
    const double* gw;
    int ngp;
};

__device__ void pdof_values(const double* T, const int32_t* bases, int nb, int W, const double* ua, int64_t nu,
                            double* out /*[24]*/, int tid, int nt) {
    for (int r = tid; r < 24; r += nt) {
        const int f = r / 8, a = r % 8;
        double v = 0.0;
        if (ua)
            for (int j = 0; j < nb; ++j) {
                const double t = T[a * W + j];
                if (t != 0.0) v = fma(t, ua[f * nu + bases[j]], v);
            }
        out[r] = v;
    }
}

// vertex position as a dual in slot `slot` (intersection vertices move with t)
template <int M>
__device__ void vertex_dual(const AdjArgs& A, int32_t v, int slot, Dual<M> x[3], bool& moving) {
    moving = A.vkind[v] == 3;
    for (int d = 0; d < 3; ++d) {
        x[d] = Dual<M>(A.vx[(int64_t)v * 3 + d]);
        if (moving) {
            const int32_t p0 = A.vpar[(int64_t)v * 8], p1 = A.vpar[(int64_t)v * 8 + 1];
            const double dx = A.vx[(int64_t)p1 * 3 + d] - A.vx[(int64_t)p0 * 3 + d];
            // slot chosen at run time: a select per slot keeps the dual in registers
#pragma unroll
            for (int i = 0; i < M; ++i) x[d].d[i] = i == slot ? dx : x[d].d[i];
        }
    }
}

template <int M>
__device__ Dual<M> tet_volume(const Dual<M> X[4][3]) {
    Dual<M> a[3], b[3], c[3];
    for (int d = 0; d < 3; ++d) {
        a[d] = X[0][d] - X[2][d];
        b[d] = X[1][d] - X[2][d];
        c[d] = X[3][d] - X[2][d];
    }
    const Dual<M> det = a[0] * (b[1] * c[2] - c[1] * b[2]) - a[1] * (b[0] * c[2] - b[2] * c[0]) +
                        a[2] * (b[0] * c[1] - b[1] * c[0]);
    return (1.0 / 6.0) * det;
}

// Cut clusters: F = sum_q w detJ (1/2 sigma(u):eps(u) - sigma(u):eps(lambda))
// over every integration cell in forward-mode dual arithmetic with one slot
// per tet vertex, dF/dt added to G of the moving vertices.  One thread per
// integration cell of the whole set: the cells of a cluster (1 to about 100)
// rarely fill whole warps, and on this GPU
// an FP64 warp instruction costs the pipe the same however few of its lanes
// are active.  The cluster's pdof values u and lambda are gathered once per
// cluster first (adjoint_cluster_values), which also writes every cell's
// cluster index.
__global__ void adjoint_cluster_values(AdjArgs A, CutSetDev S, double* UL /*[neq][48]*/, int32_t* cell_cluster) {
    const int64_t e = blockIdx.x;
    if (e >= S.neq) return;
    __shared__ double nod[48];
    for (int64_t g = S.ig_off[e] + threadIdx.x; g < S.ig_off[e + 1]; g += blockDim.x) cell_cluster[g] = (int32_t)e;
    const int nb = S.nb[e];
    pdof_values(S.T + e * 8 * S.W, S.bases + e * S.W, nb, S.W, A.u, A.nu, nod, threadIdx.x, blockDim.x);
    pdof_values(S.T + e * 8 * S.W, S.bases + e * S.W, nb, S.W, A.lam, A.nu, nod + 24, threadIdx.x, blockDim.x);
    __syncthreads();
    for (int r = threadIdx.x; r < 48; r += blockDim.x)
        UL[e * 48 + r] = monomial_coefficient(nod + (r / 24) * 24, S.xe + e * 24, r % 24);
}

// Cells with exactly M moving vertices (listed in `cells`): the moving
// vertices take derivative slots 0..M-1 in vertex order; cells without a
// moving vertex contribute nothing and are not listed.
template <int M>
__global__ void adjoint_tets_flat(AdjArgs A, CutSetDev S, const double* __restrict__ UL,
                                  const int32_t* __restrict__ cell_cluster, const int32_t* __restrict__ cells,
                                  int64_t ncells) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ncells;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t g = cells[i];
        const int64_t e = cell_cluster[g];
        const double* X = S.xe + e * 24;
        const double* U = UL + e * 48;
        const double* L = U + 24;
        const double xc[3] = {0.5 * (X[18] + X[0]), 0.5 * (X[19] + X[1]), 0.5 * (X[20] + X[2])};
        const double lam = S.E[e] * S.lam_c, mu = S.E[e] * S.mu_c;
        Dual<M> Xv[4][3], xo[4][3];  // vertices, their offsets from the cell centre
        bool mv[4];
        int32_t vids[4];
        int slot[4], next = 0;
        for (int k = 0; k < 4; ++k) {
            vids[k] = S.vid[g * 4 + k];
            slot[k] = A.vkind[vids[k]] == 3 ? next++ : -1;
            vertex_dual<M>(A, vids[k], slot[k], Xv[k], mv[k]);
            for (int d = 0; d < 3; ++d) xo[k][d] = (-xc[d]) + Xv[k][d];
        }
        const Dual<M> detJ = tet_volume<M>(Xv);
        Dual<M> F(0.0);
        for (int q = 0; q < S.ngp; ++q) {
            const double z0 = S.gp[q * 3], z1 = S.gp[q * 3 + 1], z2 = S.gp[q * 3 + 2];
            const double Nt[4] = {z0, z1, 1.0 - z0 - z1 - z2, z2};
            Dual<M> xq[3];
            for (int d = 0; d < 3; ++d) {
                xq[d] = Dual<M>(0.0);
                for (int k = 0; k < 4; ++k) axpy(Nt[k], xo[k][d], xq[d]);
            }
            const Dual<M> pr[3] = {xq[0] * xq[1], xq[1] * xq[2], xq[0] * xq[2]};
            Dual<M> Gu[3][3], Gl[3][3], Su[3][3];
            mono_field<M, false>(U, xq, pr, nullptr, Gu);
            mono_field<M, false>(L, xq, pr, nullptr, Gl);
            stress<M>(Gu, lam, mu, Su);
            Dual<M> phi(0.0);
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) phi = phi + Su[i][j] * (0.5 * Gu[i][j] + (-1.0) * Gl[i][j]);
            // skipped points (detJ < -1e-6) contribute nothing (cl_FEM_Element_Bulk.cpp:164)
            if (detJ.v < -1.0e-6) continue;
            axpy(S.gw[q], detJ * phi, F);
        }
        for (int k = 0; k < 4; ++k)
            if (mv[k]) {
                double dk = 0.0;
#pragma unroll
                for (int i2 = 0; i2 < M; ++i2) dk = i2 == slot[k] ? F.d[i2] : dk;
                atomicAdd(A.G + vids[k], dk);
            }
    }
}

struct IfSetDev {
    int64_t neq;
    int beta_sym;
    double alpha, lam_c, mu_c;
    const double* xe;      // [neq][2][8][3]
    const double* E;
    const double* EF;
    const int32_t* nb;     // [neq][2]
    const int32_t* bases;  // [neq][2][W]
    const double* T;       // [neq][2][8][W]
    int W;
    const int64_t* fc_off;
    const int32_t* vid;    // [facet][3]
    const double* gp;      // TRI rule [ngp][2]
    const double* gw;
    int ngp;
    const double* vol;     // [neq][2]
    const int32_t* link;   // [neq][4]: leader (set, eq), follower (set, eq) among the cut sets
};

// The interface sum, flattened like the cut cells (a cluster has a few
// facets).  The facet integrals are formed once, in dual arithmetic:
//   iface_cluster_values   per cluster: pdof values of u and lambda of both
//                          sides, each facet's cluster index;
//   iface_facets           one thread per facet: the values A, B, C, |G| into
//                          the cluster sums, the derivatives kept per facet;
//   iface_apply            one thread per facet: dF/dt with the now known
//                          cluster sums (w_L, w_F, gamma);
//   iface_volumes          one thread per (cluster, side, cell of the linked
//                          cut cluster): dF/dV through w_L, w_F and gamma.
constexpr int kIfParts = 12;  // dA, dB, dC, d|G| for the three vertices

__global__ void iface_cluster_values(AdjArgs A, IfSetDev S, double* UL /*[neq][96]*/, int32_t* facet_cluster) {
    const int64_t e = blockIdx.x;
    if (e >= S.neq) return;
    __shared__ double nod[96];
    for (int64_t f = S.fc_off[e] + threadIdx.x; f < S.fc_off[e + 1]; f += blockDim.x) facet_cluster[f] = (int32_t)e;
    for (int s = 0; s < 2; ++s) {
        const int nb = S.nb[2 * e + s];
        pdof_values(S.T + (e * 2 + s) * 8 * S.W, S.bases + (e * 2 + s) * S.W, nb, S.W, A.u, A.nu, nod + 24 * s,
                    threadIdx.x, blockDim.x);
        pdof_values(S.T + (e * 2 + s) * 8 * S.W, S.bases + (e * 2 + s) * S.W, nb, S.W, A.lam, A.nu,
                    nod + 48 + 24 * s, threadIdx.x, blockDim.x);
    }
    __syncthreads();
    // [u side 0, u side 1, lambda side 0, lambda side 1], each on its side's cell
    for (int r = threadIdx.x; r < 96; r += blockDim.x)
        UL[e * 96 + r] = monomial_coefficient(nod + (r / 24) * 24, S.xe + e * 48 + 24 * ((r / 24) & 1), r % 24);
}

__global__ void iface_facets(AdjArgs A, IfSetDev S, const double* __restrict__ UL,
                             const int32_t* __restrict__ facet_cluster, int64_t nfacets, double* sums /*[neq][4]*/,
                             double* parts /*[nf][kIfParts]*/) {
    for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nfacets;
         f += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = facet_cluster[f];
        const double* X = S.xe + e * 48;
        const double* U = UL + e * 96;
        const double* L = U + 48;
        const double Es[2] = {S.E[e], S.EF[e]};
        const double beta = S.beta_sym ? -1.0 : 1.0;
        double* P = parts + f * kIfParts;
        Dual<3> Xv[3][3];
        bool mv[3];
        for (int k = 0; k < 3; ++k) vertex_dual<3>(A, S.vid[f * 3 + k], k, Xv[k], mv[k]);
        // facet detJ |(x0-x2) x (x1-x2)| / 2 and the unit normal
        Dual<3> a[3], b[3], cr[3];
        for (int d = 0; d < 3; ++d) {
            a[d] = Xv[0][d] - Xv[2][d];
            b[d] = Xv[1][d] - Xv[2][d];
        }
        cr[0] = a[1] * b[2] - a[2] * b[1];
        cr[1] = a[2] * b[0] - a[0] * b[2];
        cr[2] = a[0] * b[1] - a[1] * b[0];
        const Dual<3> nn = dsqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
        if (!(nn.v > 0.0)) {
            for (int k = 0; k < kIfParts; ++k) P[k] = 0.0;
            continue;
        }
        const Dual<3> inv = dinv(nn);
        const Dual<3> n[3] = {cr[0] * inv, cr[1] * inv, cr[2] * inv};
        const Dual<3> detJ = 0.5 * nn;
        double xc[2][3];  // the sides' cell centres
        for (int s = 0; s < 2; ++s)
            for (int d = 0; d < 3; ++d) xc[s][d] = 0.5 * (X[24 * s + 18 + d] + X[24 * s + d]);
        Dual<3> fa(0.0), fb(0.0), fc(0.0), fr(0.0);
        for (int q = 0; q < S.ngp; ++q) {
            const double z0 = S.gp[q * 2], z1 = S.gp[q * 2 + 1];
            const double Nf[3] = {z0, z1, 1.0 - z0 - z1};
            // per side: values and tractions t_s(.) = sigma_s(.) n, each
            // gradient turned into its traction at once
            Dual<3> uv[2][3], lv[2][3], tu[2][3], tl[2][3], xp[3];
            for (int d = 0; d < 3; ++d) {
                xp[d] = Dual<3>(0.0);
                for (int k = 0; k < 3; ++k) axpy(Nf[k], Xv[k][d], xp[d]);
            }
            for (int s = 0; s < 2; ++s) {
                Dual<3> xq[3];
                for (int d = 0; d < 3; ++d) xq[d] = (-xc[s][d]) + xp[d];
                const Dual<3> pr[3] = {xq[0] * xq[1], xq[1] * xq[2], xq[0] * xq[2]};
                for (int fld = 0; fld < 2; ++fld) {
                    Dual<3> Gf[3][3], Sf[3][3];
                    mono_field<3, true>((fld ? L : U) + 24 * s, xq, pr, fld ? lv[s] : uv[s], Gf);
                    stress<3>(Gf, Es[s] * S.lam_c, Es[s] * S.mu_c, Sf);
                    Dual<3>* t = fld ? tl[s] : tu[s];
                    for (int i2 = 0; i2 < 3; ++i2) t[i2] = Sf[i2][0] * n[0] + Sf[i2][1] * n[1] + Sf[i2][2] * n[2];
                }
            }
            Dual<3> qa(0.0), qb(0.0), qc(0.0);
            for (int i = 0; i < 3; ++i) {
                const Dual<3> ju = uv[0][i] - uv[1][i], jl = lv[0][i] - lv[1][i];
                qa = qa + beta * (tl[0][i] * ju) - jl * tu[0][i];
                qb = qb + beta * (tl[1][i] * ju) - jl * tu[1][i];
                qc = qc + jl * ju;
            }
            const Dual<3> ws = S.gw[q] * detJ;
            fa = fa + ws * qa;
            fb = fb + ws * qb;
            fc = fc + ws * qc;
            fr = fr + ws;
        }
        atomicAdd(sums + e * 4 + 0, fa.v);
        atomicAdd(sums + e * 4 + 1, fb.v);
        atomicAdd(sums + e * 4 + 2, fc.v);
        atomicAdd(sums + e * 4 + 3, fr.v);
        for (int k = 0; k < 3; ++k) {
            // a vertex that does not move has no derivative slot
            P[k] = mv[k] ? fa.d[k] : 0.0;
            P[3 + k] = mv[k] ? fb.d[k] : 0.0;
            P[6 + k] = mv[k] ? fc.d[k] : 0.0;
            P[9 + k] = mv[k] ? fr.d[k] : 0.0;
        }
    }
}

// the cluster's Nitsche weights and gamma from its sums and volumes
__device__ __forceinline__ void iface_weights(const IfSetDev& S, int64_t e, double& wl, double& wf, double& Ssum) {
    const double vl = S.vol[2 * e] / S.E[e], vf = S.vol[2 * e + 1] / S.EF[e];
    Ssum = vl + vf;
    wl = vl / Ssum;
    wf = vf / Ssum;
}

__global__ void iface_apply(AdjArgs A, IfSetDev S, const int32_t* __restrict__ facet_cluster, int64_t nfacets,
                            const double* __restrict__ sums, const double* __restrict__ parts) {
    for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nfacets;
         f += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = facet_cluster[f];
        double wl, wf, Ssum;
        iface_weights(S, e, wl, wf, Ssum);
        // F = -(wL A + wF B + gamma C), gamma = 2 alpha |G| / S
        const double gamma = 2.0 * S.alpha * sums[e * 4 + 3] / Ssum;
        const double dg_darea = 2.0 * S.alpha / Ssum;
        const double* P = parts + f * kIfParts;
        for (int k = 0; k < 3; ++k) {
            const double g = -(wl * P[k] + wf * P[3 + k] + gamma * P[6 + k] + sums[e * 4 + 2] * dg_darea * P[9 + k]);
            if (P[k] != 0.0 || P[3 + k] != 0.0 || P[6 + k] != 0.0 || P[9 + k] != 0.0)
                atomicAdd(A.G + S.vid[f * 3 + k], g);
        }
    }
}

// items: (interface cluster e, side) per cell of the linked cut cluster
__global__ void iface_volumes(AdjArgs A, IfSetDev S, const CutSetDev* cuts, int64_t nitems,
                              const int64_t* __restrict__ item_e, const int64_t* __restrict__ item_cell,
                              const double* __restrict__ sums) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nitems;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t es = item_e[t], e = es >> 1;
        const int side = (int)(es & 1);
        const CutSetDev& C = cuts[S.link[e * 4 + side * 2]];
        const int64_t g = item_cell[t];
        double wl, wf, Ssum;
        iface_weights(S, e, wl, wf, Ssum);
        const double vl = S.vol[2 * e] / S.E[e], vf = S.vol[2 * e + 1] / S.EF[e];
        const double gamma = 2.0 * S.alpha * sums[e * 4 + 3] / Ssum;
        const double dwl = side == 0 ? vf / (Ssum * Ssum) : -vl / (Ssum * Ssum);
        const double dg_dv = -gamma / Ssum;
        const double Es = side == 0 ? S.E[e] : S.EF[e];
        // dF/dvol = -((A - B) dwL/dv + C dgamma/dv) / E_side
        const double coef = -((sums[e * 4 + 0] - sums[e * 4 + 1]) * dwl + sums[e * 4 + 2] * dg_dv) / Es;
        Dual<4> Xv[4][3];
        bool mv[4];
        int32_t vids[4];
        for (int k = 0; k < 4; ++k) {
            vids[k] = C.vid[g * 4 + k];
            vertex_dual<4>(A, vids[k], k, Xv[k], mv[k]);
        }
        const Dual<4> vol = tet_volume<4>(Xv);
        for (int k = 0; k < 4; ++k)
            if (mv[k]) atomicAdd(A.G + vids[k], coef * vol.d[k]);
    }
}

// dqdp[j] += G[v] dt_v/dp_j through the parents' level set
__global__ void dqdp_chain(int64_t nv, const int32_t* vkind, const int32_t* vpar, const double* vphi,
                           const double* G, int width, const int32_t* cols, const double* tmat, double* dqdp) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv || vkind[v] != 3 || G[v] == 0.0) return;
    const int32_t p[2] = {vpar[v * 8], vpar[v * 8 + 1]};
    const double f0 = vphi[p[0]], f1 = vphi[p[1]];
    const double den = (f0 - f1) * (f0 - f1);
    // t = f0 / (f0 - f1): dt/df0 = -f1 / (f0-f1)^2, dt/df1 = f0 / (f0-f1)^2
    const double dt[2] = {-f1 / den, f0 / den};
    for (int k = 0; k < 2; ++k) {
        const int32_t q = p[k];
        const int kind = vkind[q];
        const int cnt = kind == 0 ? 1 : kind == 1 ? 4 : 8;
        const double w = G[v] * dt[k] / (double)cnt;
        for (int m = 0; m < cnt; ++m) {
            const int64_t node = vpar[(int64_t)q * 8 + m];
            for (int j = 0; j < width; ++j) {
                const double tv = tmat[node * width + j];
                if (tv != 0.0) atomicAdd(dqdp + cols[node * width + j], w * tv);
            }
        }
    }
}

__global__ void dot_kernel(int64_t n, const double* a, const double* b, double* out) {
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s = fma(a[i], b[i], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    __shared__ double ws[32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) atomicAdd(out, s);
    }
}

void dfree(DeviceBuf& b) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
}

template <class T>
cudaError_t upload(DeviceBuf& b, const std::vector<T>& v, cudaStream_t st) {
    dfree(b);
    b.bytes = std::max<size_t>(v.size() * sizeof(T), 16);
    cudaError_t e = cudaMalloc(&b.p, b.bytes);
    if (e != cudaSuccess) return e;
    if (!v.empty()) e = cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st);
    return e;
}

// in-place refresh (same size: kernel arguments and captured graphs keep their pointers)
template <class T>
cudaError_t refresh(DeviceBuf& b, const std::vector<T>& v, cudaStream_t st) {
    if (!b.p || b.bytes < v.size() * sizeof(T)) return upload(b, v, st);
    if (v.empty()) return cudaSuccess;
    return cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st);
}

fem_gpu_status sfail(fem_gpu_ctx* c, cudaError_t e, const char* what) {
    return fail(c, e == cudaErrorMemoryAllocation ? FEM_GPU_OUT_OF_MEMORY : FEM_GPU_CUDA_ERROR,
                std::string(what) + ": " + cudaGetErrorString(e));
}

double lam_of(int model, double nu) {
    return model == FEM_GPU_MODEL_PLANE_STRESS ? nu / (1.0 - nu * nu) : nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
}

bool is_cut(const SetData& s) { return s.kind == 0 && !s.ig_off.empty(); }
bool is_interface(const SetData& s) {
    return s.kind == 2 && !is_ghost_iwg(s.dside.iwg_type);
}

}  // namespace

void sensitivity_release(fem_gpu_ctx* c) {
    dfree(c->d_vkind);
    dfree(c->d_vpar);
    dfree(c->d_vx);
    dfree(c->d_adjcuts);
    dfree(c->d_vval);
    dfree(c->d_lscols);
    dfree(c->d_lst);
    c->ls_nbn = 0;
    c->ls_phi = false;
    for (auto& s : c->sets) {
        dfree(s.d_vid);
        dfree(s.d_link);
        dfree(s.d_adjul);
        dfree(s.d_items);
        dfree(s.d_tperm);
        s.nitems = 0;
        for (int64_t& o : s.tperm_off) o = 0;
    }
    c->adj_topo = c->adj_coords = false;
}

}  // namespace fem

using namespace fem;

extern "C" {

fem_gpu_status fem_gpu_set_ig_vertices(fem_gpu_ctx* c, int64_t nv, const int32_t* kind, const int32_t* parents,
                                       const double* coords, const double* value) {
    if (!c || nv <= 0 || !kind || !parents || !coords || !value) return FEM_GPU_BAD_ARG;
    c->vkind.assign(kind, kind + nv);
    c->vpar.assign(parents, parents + nv * 8);
    c->vx.assign(coords, coords + nv * 3);
    c->vval.assign(value, value + nv);
    c->adj_topo = c->adj_coords = c->ls_phi = false;
    c->ls_checked_nbn = -1;
    for (int64_t v = 0; v < nv; ++v) {
        const int k = c->vkind[v];
        if (k < 0 || k > 3) return fail(c, FEM_GPU_BAD_ARG, "IG vertex kind");
        const int cnt = k == 0 ? 1 : k == 1 ? 4 : k == 2 ? 8 : 2;
        for (int m = 0; m < cnt; ++m) {
            const int32_t p = c->vpar[v * 8 + m];
            const int64_t lim = k == 3 ? nv : c->num_nodes;
            if (p < 0 || p >= lim) return fail(c, FEM_GPU_OOB_INDEX, "IG vertex parent");
            if (k == 3 && c->vkind[p] == 3) return fail(c, FEM_GPU_BAD_ARG, "intersection of intersections");
        }
    }
    for (auto& s : c->sets) {
        if (!(is_cut(s) || is_interface(s)) || s.neq == 0) continue;
        if (s.vid.empty()) return fail(c, FEM_GPU_BAD_ARG, "cut / interface set without IG vertex ids");
        for (int32_t v : s.vid)
            if (v < 0 || v >= nv) return fail(c, FEM_GPU_OOB_INDEX, "IG vertex id");
    }
    return FEM_GPU_OK;
}

fem_gpu_status fem_gpu_update_ig_vertices(fem_gpu_ctx* c, const double* t) {
    if (!c || !t) return FEM_GPU_BAD_ARG;
    if (!c->dev_final) return FEM_GPU_NOT_FINALIZED;
    if (c->vkind.empty()) return fail(c, FEM_GPU_BAD_ARG, "no IG vertex table");
    if (c->shape != FEM_GPU_SHAPE_RECTANGULAR) return fail(c, FEM_GPU_UNSUPPORTED, "geometry update needs rectangular cells");
    const int64_t nv = (int64_t)c->vkind.size();
    for (int64_t v = 0; v < nv; ++v) {
        if (c->vkind[v] != 3) continue;
        if (!std::isfinite(t[v])) return fail(c, FEM_GPU_NONFINITE, "edge coordinate");
        const int32_t p0 = c->vpar[v * 8], p1 = c->vpar[v * 8 + 1];
        for (int d = 0; d < 3; ++d) c->vx[v * 3 + d] = c->vx[p0 * 3 + d] + t[v] * (c->vx[p1 * 3 + d] - c->vx[p0 * 3 + d]);
        c->vval[v] = t[v];
    }
    c->adj_coords = false;
    const int npe = c->npe;
    auto param = [&](int64_t cell, const double* x, double* xi) {
        const double* X0 = &c->coords[(int64_t)c->cells[cell * npe + 0] * 3];
        const double* X6 = &c->coords[(int64_t)c->cells[cell * npe + 6] * 3];
        for (int d = 0; d < 3; ++d) xi[d] = -1.0 + 2.0 * (x[d] - X0[d]) / (X6[d] - X0[d]);
    };
    cudaStream_t st = (cudaStream_t)c->stream;
    cudaError_t e = cudaSuccess;
    for (auto& s : c->sets) {
        if (s.neq == 0) continue;
        if (is_cut(s)) {
            for (int64_t i = 0; i < s.neq; ++i)
                for (int64_t g = s.ig_off[i]; g < s.ig_off[i + 1]; ++g)
                    for (int k = 0; k < 4; ++k) {
                        const int32_t v = s.vid[g * 4 + k];
                        if (c->vkind[v] != 3) continue;
                        for (int d = 0; d < 3; ++d) s.ig_coords[(g * 4 + k) * 3 + d] = c->vx[v * 3 + d];
                        param(s.ip_cell[i], &c->vx[v * 3], &s.ig_param[(g * 4 + k) * 3]);
                    }
            if (e == cudaSuccess) e = refresh(s.d_igx, s.ig_coords, st);
            if (e == cudaSuccess) e = refresh(s.d_igxi, s.ig_param, st);
        } else if (is_interface(s)) {
            for (int64_t i = 0; i < s.neq; ++i)
                for (int64_t f = s.fc_off[i]; f < s.fc_off[i + 1]; ++f)
                    for (int k = 0; k < s.nfv; ++k) {
                        const int32_t v = s.vid[f * s.nfv + k];
                        if (c->vkind[v] != 3) continue;
                        for (int d = 0; d < 3; ++d) s.fc_x[(f * s.nfv + k) * 3 + d] = c->vx[v * 3 + d];
                        param(s.ip_cell[i], &c->vx[v * 3], &s.fc_xl[(f * s.nfv + k) * 3]);
                        param(s.fcell[i], &c->vx[v * 3], &s.fc_xf[(f * s.nfv + k) * 3]);
                    }
            if (e == cudaSuccess) e = refresh(s.d_fcx, s.fc_x, st);
            if (e == cudaSuccess) e = refresh(s.d_fcxl, s.fc_xl, st);
            if (e == cudaSuccess) e = refresh(s.d_fcxf, s.fc_xf, st);
        }
    }
    fem_gpu_status r = interface_volumes(c);
    if (r != FEM_GPU_OK) return r;
    for (auto& s : c->sets)
        if (is_interface(s) && s.neq > 0 && e == cudaSuccess) e = refresh(s.d_vol, s.vol, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return sfail(c, e, "geometry update");
    return FEM_GPU_OK;
}

fem_gpu_status fem_gpu_strain_energy(fem_gpu_ctx* c, const double* u, double* dqdu, double* q) {
    if (!c || !u || !dqdu) return FEM_GPU_BAD_ARG;
    if (!c->dev_final) return FEM_GPU_NOT_FINALIZED;
    // residual-only assembly of the bulk sets: dQ/du = K_bulk u (linear CM, no body load)
    cudaStream_t st = (cudaStream_t)c->stream;
    const int64_t nad = c->num_used * c->dim;
    cudaError_t e = cudaMemsetAsync(dqdu, 0, nad * sizeof(double), st);
    if (e != cudaSuccess) return sfail(c, e, "strain energy zero");
    fem_gpu_status r = FEM_GPU_OK;
    for (int k = 0; k < (int)c->sets.size() && r == FEM_GPU_OK; ++k) {
        if (c->sets[k].kind != 0) continue;
        r = assemble_set(c, k, u, nullptr, dqdu);
    }
    if (r != FEM_GPU_OK) return r;
    if (q) {
        double* d = nullptr;
        e = cudaMallocAsync(&d, sizeof(double), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(d, 0, sizeof(double), st);
        if (e == cudaSuccess) {
            dot_kernel<<<(unsigned)sm_count() * 4, 256, 0, st>>>(nad, u, dqdu, d);
            e = cudaMemcpyAsync(q, d, sizeof(double), cudaMemcpyDeviceToHost, st);
        }
        if (d) cudaFreeAsync(d, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return sfail(c, e, "strain energy");
        *q *= 0.5;
    }
    return fem_gpu_check_status(c);
}

fem_gpu_status fem_gpu_drdp_adjoint(fem_gpu_ctx* c, const double* u, const double* lambda, double* G) {
    if (!c || !u || !lambda || !G) return FEM_GPU_BAD_ARG;
    if (!c->dev_final) return FEM_GPU_NOT_FINALIZED;
    if (c->vkind.empty()) return fail(c, FEM_GPU_BAD_ARG, "no IG vertex table");
    if (c->shape != FEM_GPU_SHAPE_RECTANGULAR || c->dim != 3)
        return fail(c, FEM_GPU_UNSUPPORTED, "shape sensitivities need 3D rectangular cells");
    cudaStream_t st = (cudaStream_t)c->stream;
    const int64_t nv = (int64_t)c->vkind.size();
    // the vertex table, vertex ids, interface links and volume items depend on
    // the topology only and go to the device once per vertex table; the
    // coordinates once per geometry update
    const bool topo = !c->adj_topo;
    c->adj_topo = false;
    cudaError_t e = cudaSuccess;
    if (topo) {
        e = refresh(c->d_vkind, c->vkind, st);
        if (e == cudaSuccess) e = refresh(c->d_vpar, c->vpar, st);
    }
    if (e == cudaSuccess && !c->adj_coords) e = refresh(c->d_vx, c->vx, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(G, 0, nv * sizeof(double), st);
    if (e != cudaSuccess) return sfail(c, e, "adjoint vertex table");
    c->adj_coords = true;
    AdjArgs A{};
    A.vkind = (const int32_t*)c->d_vkind.p;
    A.vpar = (const int32_t*)c->d_vpar.p;
    A.vx = (const double*)c->d_vx.p;
    A.G = G;
    A.u = u;
    A.lam = lambda;
    A.nu = c->num_used;
    // cut sets
    std::vector<CutSetDev> cuts;
    std::vector<int> cut_index(c->sets.size(), -1), cut_set;  // set -> cut index, cut index -> set
    std::vector<std::pair<int32_t, int64_t>> cell_cluster(topo ? c->num_cells : 0, {-1, -1});
    for (size_t k = 0; k < c->sets.size(); ++k) {
        SetData& s = c->sets[k];
        if (!is_cut(s) || s.neq == 0) continue;
        if (s.vid.empty()) return fail(c, FEM_GPU_BAD_ARG, "cut set without IG vertex ids");
        if (s.bulk.integration_rule != FEM_GPU_RULE_TET_4 && s.bulk.integration_rule != FEM_GPU_RULE_TET_11)
            return fail(c, FEM_GPU_UNSUPPORTED, "sensitivities of cut clusters need TET4 cells");
        if (topo && (e = refresh(s.d_vid, s.vid, st)) != cudaSuccess) return sfail(c, e, "vertex ids");
        CutSetDev d{};
        d.neq = s.neq;
        d.xe = (const double*)s.d_xe.p;
        d.E = (const double*)s.d_E.p;
        d.nb = (const int32_t*)s.d_nb.p;
        d.bases = (const int32_t*)s.d_bases.p;
        d.T = (const double*)s.d_T.p;
        d.W = s.nbsel;
        d.lam_c = lam_of(s.bulk.model_type, s.bulk.poisson_ratio);
        d.mu_c = 1.0 / (2.0 * (1.0 + s.bulk.poisson_ratio));
        d.ig_off = (const int64_t*)s.d_igoff.p;
        d.vid = (const int32_t*)s.d_vid.p;
        d.gp = (const double*)s.d_gp.p;
        d.gw = (const double*)s.d_gw.p;
        d.ngp = s.ngp;
        cut_index[k] = (int)cuts.size();
        cut_set.push_back((int)k);
        if (topo)
            for (int64_t i = 0; i < s.neq; ++i) cell_cluster[s.ip_cell[i]] = {(int32_t)cuts.size(), i};
        cuts.push_back(d);
    }
    for (size_t k = 0, ci = 0; k < c->sets.size(); ++k) {
        if (cut_index[k] < 0) continue;
        SetData& s = c->sets[k];
        const CutSetDev& d = cuts[ci++];
        const int64_t ncells = s.ig_off.empty() ? 0 : s.ig_off.back();
        // per-cluster pdof values of u and lambda, then one thread per cell
        // [neq][48] doubles, then [ncells] cluster indices
        const size_t need = (size_t)d.neq * 48 * sizeof(double) + (size_t)std::max<int64_t>(ncells, 1) * sizeof(int32_t);
        if (!s.d_adjul.p || s.d_adjul.bytes < need) {
            dfree(s.d_adjul);
            if ((e = cudaMalloc(&s.d_adjul.p, need)) != cudaSuccess) return sfail(c, e, "adjoint cluster values");
            s.d_adjul.bytes = need;
        }
        double* UL = (double*)s.d_adjul.p;
        int32_t* cc = reinterpret_cast<int32_t*>(UL + (size_t)d.neq * 48);
        if (topo) {
            // integration cells grouped by their number of moving (intersection)
            // vertices, 1 to 4; cells without one are left out
            std::vector<int32_t> cnt(ncells);
            int64_t grp[5] = {0, 0, 0, 0, 0};
            for (int64_t g = 0; g < ncells; ++g) {
                int m = 0;
                for (int k = 0; k < 4; ++k) m += c->vkind[s.vid[g * 4 + k]] == 3;
                cnt[g] = m;
                ++grp[m];
            }
            s.tperm_off[0] = 0;
            for (int m = 1; m <= 4; ++m) s.tperm_off[m] = s.tperm_off[m - 1] + grp[m];
            std::vector<int32_t> perm(std::max<int64_t>(s.tperm_off[4], 1));
            int64_t pos[5] = {0, s.tperm_off[0], s.tperm_off[1], s.tperm_off[2], s.tperm_off[3]};
            for (int64_t g = 0; g < ncells; ++g)
                if (cnt[g] > 0) perm[pos[cnt[g]]++] = (int32_t)g;
            if ((e = upload(s.d_tperm, perm, st)) != cudaSuccess) return sfail(c, e, "moving-vertex groups");
        }
        adjoint_cluster_values<<<(unsigned)std::max<int64_t>(d.neq, 1), 64, 0, st>>>(A, d, UL, cc);
        c->launches++;
        const int32_t* perm = (const int32_t*)s.d_tperm.p;
        for (int m = 1; m <= 4; ++m) {
            const int64_t a0 = s.tperm_off[m - 1], n = s.tperm_off[m] - a0;
            if (n <= 0) continue;
            const unsigned grid =
                (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 63) / 64, (int64_t)sm_count() * 16));
            switch (m) {
                case 1: adjoint_tets_flat<1><<<grid, 64, 0, st>>>(A, d, UL, cc, perm + a0, n); break;
                case 2: adjoint_tets_flat<2><<<grid, 64, 0, st>>>(A, d, UL, cc, perm + a0, n); break;
                case 3: adjoint_tets_flat<3><<<grid, 64, 0, st>>>(A, d, UL, cc, perm + a0, n); break;
                default: adjoint_tets_flat<4><<<grid, 64, 0, st>>>(A, d, UL, cc, perm + a0, n); break;
            }
            c->launches++;
        }
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return sfail(c, e, "adjoint tets");
    if ((e = refresh(c->d_adjcuts, cuts, st)) != cudaSuccess) return sfail(c, e, "cut table");
    fem_gpu_status r = FEM_GPU_OK;
    for (auto& s : c->sets) {
        if (!is_interface(s) || s.neq == 0) continue;
        if (s.vid.empty() || s.nfv != 3) {
            r = fail(c, FEM_GPU_UNSUPPORTED, "interface sensitivities need TRI3 facets with vertex ids");
            break;
        }
        if (topo) {
            s.link.assign(s.neq * 4, 0);
            for (int64_t i = 0; i < s.neq; ++i) {
                const auto L = cell_cluster[s.ip_cell[i]], F = cell_cluster[s.fcell[i]];
                if (L.first < 0 || F.first < 0) {
                    r = fail(c, FEM_GPU_BAD_ARG, "interface cluster without cut clusters on its cells");
                    break;
                }
                s.link[i * 4 + 0] = L.first;
                s.link[i * 4 + 1] = (int32_t)L.second;
                s.link[i * 4 + 2] = F.first;
                s.link[i * 4 + 3] = (int32_t)F.second;
            }
            if (r != FEM_GPU_OK) break;
            // volume items: (e * 2 + side) in the first half, the integration cell in the second
            std::vector<int64_t> items;
            for (int pass = 0; pass < 2; ++pass)
                for (int64_t i = 0; i < s.neq; ++i)
                    for (int side = 0; side < 2; ++side) {
                        const int cs = s.link[i * 4 + side * 2];
                        const int64_t ce = s.link[i * 4 + side * 2 + 1];
                        const std::vector<int64_t>& io = c->sets[cut_set[cs]].ig_off;
                        for (int64_t g = io[ce]; g < io[ce + 1]; ++g) items.push_back(pass == 0 ? i * 2 + side : g);
                    }
            s.nitems = (int64_t)items.size() / 2;
            if ((e = refresh(s.d_link, s.link, st)) != cudaSuccess || (e = refresh(s.d_vid, s.vid, st)) != cudaSuccess ||
                (e = upload(s.d_items, items, st)) != cudaSuccess) {
                r = sfail(c, e, "interface links");
                break;
            }
        }
        IfSetDev d{};
        d.neq = s.neq;
        d.beta_sym = s.dside.iwg_type == FEM_GPU_IWG_STRUC_LINEAR_INTERFACE_SYMMETRIC_NITSCHE;
        d.alpha = s.dside.alpha;
        d.lam_c = lam_of(s.dside.model_type, s.dside.poisson_ratio);
        d.mu_c = 1.0 / (2.0 * (1.0 + s.dside.poisson_ratio));
        d.xe = (const double*)s.d_xe.p;
        d.E = (const double*)s.d_E.p;
        d.EF = (const double*)s.d_EF.p;
        d.nb = (const int32_t*)s.d_nb.p;
        d.bases = (const int32_t*)s.d_bases.p;
        d.T = (const double*)s.d_T.p;
        d.W = s.nbsel;
        d.fc_off = (const int64_t*)s.d_fcoff.p;
        d.vid = (const int32_t*)s.d_vid.p;
        d.gp = (const double*)s.d_gp.p;
        d.gw = (const double*)s.d_gw.p;
        d.ngp = s.ngp;
        d.vol = (const double*)s.d_vol.p;
        d.link = (const int32_t*)s.d_link.p;
        // scratch: per cluster U, L (96) and sums (4); per facet the cluster
        // index and the derivative parts; the volume items
        const int64_t nf = s.fc_off.empty() ? 0 : s.fc_off.back();
        const int64_t ni = s.nitems;
        const int64_t* item_e = (const int64_t*)s.d_items.p;
        const size_t need = (size_t)s.neq * 100 * sizeof(double) + (size_t)std::max<int64_t>(nf, 1) * kIfParts * sizeof(double) +
                            (size_t)std::max<int64_t>(nf, 1) * sizeof(int32_t);
        if (!s.d_adjul.p || s.d_adjul.bytes < need) {
            dfree(s.d_adjul);
            if ((e = cudaMalloc(&s.d_adjul.p, need)) != cudaSuccess) {
                r = sfail(c, e, "interface scratch");
                break;
            }
            s.d_adjul.bytes = need;
        }
        double* UL = (double*)s.d_adjul.p;
        double* sums = UL + (size_t)s.neq * 96;
        double* parts = sums + (size_t)s.neq * 4;
        int32_t* fcl = reinterpret_cast<int32_t*>(parts + (size_t)std::max<int64_t>(nf, 1) * kIfParts);
        cudaMemsetAsync(sums, 0, (size_t)s.neq * 4 * sizeof(double), st);
        const auto grid_of = [](int64_t n) {
            return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 63) / 64, (int64_t)sm_count() * 16));
        };
        iface_cluster_values<<<(unsigned)std::max<int64_t>(s.neq, 1), 64, 0, st>>>(A, d, UL, fcl);
        iface_facets<<<grid_of(nf), 64, 0, st>>>(A, d, UL, fcl, nf, sums, parts);
        iface_apply<<<grid_of(nf), 64, 0, st>>>(A, d, fcl, nf, sums, parts);
        iface_volumes<<<grid_of(ni), 64, 0, st>>>(A, d, (const CutSetDev*)c->d_adjcuts.p, ni, item_e, item_e + ni,
                                                  sums);
        c->launches += 4;
        if ((e = cudaGetLastError()) != cudaSuccess) {
            r = sfail(c, e, "adjoint interface");
            break;
        }
    }
    if (r != FEM_GPU_OK) return r;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return sfail(c, e, "adjoint");
    c->adj_topo = true;
    return FEM_GPU_OK;
}

fem_gpu_status fem_gpu_set_level_set_field(fem_gpu_ctx* c, int64_t nbn, int32_t width, const int32_t* cols,
                                           const double* tmat, int64_t ncoef) {
    if (!c || !cols || !tmat || width <= 0 || nbn <= 0 || ncoef <= 0) return FEM_GPU_BAD_ARG;
    const int64_t n = nbn * width;
    for (int64_t k = 0; k < n; ++k)
        if (cols[k] < 0 || cols[k] >= ncoef) return fail(c, FEM_GPU_OOB_INDEX, "level-set coefficient id");
    c->ls_nbn = 0;
    cudaStream_t st = (cudaStream_t)c->stream;
    cudaError_t e = cudaSuccess;
    if (!c->d_lscols.p || c->d_lscols.bytes < (size_t)n * sizeof(int32_t)) {
        dfree(c->d_lscols);
        if ((e = cudaMalloc(&c->d_lscols.p, (size_t)n * sizeof(int32_t))) == cudaSuccess)
            c->d_lscols.bytes = (size_t)n * sizeof(int32_t);
    }
    if (e == cudaSuccess && (!c->d_lst.p || c->d_lst.bytes < (size_t)n * sizeof(double))) {
        dfree(c->d_lst);
        if ((e = cudaMalloc(&c->d_lst.p, (size_t)n * sizeof(double))) == cudaSuccess)
            c->d_lst.bytes = (size_t)n * sizeof(double);
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->d_lscols.p, cols, (size_t)n * sizeof(int32_t), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->d_lst.p, tmat, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return sfail(c, e, "level-set field");
    c->ls_nbn = nbn;
    c->ls_width = width;
    c->ls_ncoef = ncoef;
    return FEM_GPU_OK;
}

fem_gpu_status fem_gen_dqdp(fem_gpu_ctx* c, const double* G, int64_t nbn, int32_t width, const int32_t* cols,
                            const double* tmat, int64_t ncoef, double* dqdp) {
    if (!c || !G || !dqdp || width <= 0 || nbn <= 0 || ncoef <= 0 || (!cols) != (!tmat)) return FEM_GPU_BAD_ARG;
    if (c->vkind.empty()) return fail(c, FEM_GPU_BAD_ARG, "no IG vertex table");
    if (cols) {
        const fem_gpu_status r = fem_gpu_set_level_set_field(c, nbn, width, cols, tmat, ncoef);
        if (r != FEM_GPU_OK) return r;
    } else if (c->ls_nbn != nbn || c->ls_width != width || c->ls_ncoef != ncoef) {
        return fail(c, FEM_GPU_BAD_ARG, "no level-set field of these sizes (fem_gpu_set_level_set_field)");
    }
    const int64_t nv = (int64_t)c->vkind.size();
    // background parents of the vertex table against this field (once per table and field size)
    if (c->ls_checked_nbn != nbn) {
        for (int64_t v = 0; v < nv; ++v)
            if (c->vkind[v] != 3)
                for (int m = 0; m < 8; ++m)
                    if (c->vpar[v * 8 + m] >= nbn) return fail(c, FEM_GPU_OOB_INDEX, "background node of an IG vertex");
        c->ls_checked_nbn = nbn;
    }
    cudaStream_t st = (cudaStream_t)c->stream;
    // level set at the parents: vval holds phi for kinds 0-2 (set with the
    // vertex table; geometry updates change the kind-3 entries only)
    cudaError_t e = cudaSuccess;
    if (!c->ls_phi) e = refresh(c->d_vval, c->vval, st);
    if (e == cudaSuccess && !c->adj_topo) e = refresh(c->d_vkind, c->vkind, st);
    if (e == cudaSuccess && !c->adj_topo) e = refresh(c->d_vpar, c->vpar, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(dqdp, 0, ncoef * sizeof(double), st);
    if (e == cudaSuccess) {
        c->ls_phi = true;
        dqdp_chain<<<(unsigned)((nv + 255) / 256), 256, 0, st>>>(nv, (const int32_t*)c->d_vkind.p,
                                                                 (const int32_t*)c->d_vpar.p, (const double*)c->d_vval.p,
                                                                 G, width, (const int32_t*)c->d_lscols.p,
                                                                 (const double*)c->d_lst.p, dqdp);
        c->launches++;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return sfail(c, e, "dq/dp chain");
    return FEM_GPU_OK;
}

}  // extern "C"
