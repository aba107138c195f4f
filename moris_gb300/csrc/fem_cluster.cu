// fem_cluster.cu -- uneven clusters: uncut cells, cut clusters (integration
// cells inside an IP cell) and double-sided clusters (Nitsche interface,
// face-oriented ghost), all in one persistent kernel.
//
// Work items: one per equation object, a cluster with more integration
// points than the split size cut into point ranges (element matrices are
// linear in the point set, so each range scatters its own part).  A CTA takes
// the next item from a device queue (items sorted by decreasing cost), so
// clusters of 4 or 400 points keep every SM busy until the queue runs dry.
//
// Per item (one CTA, W warps):
//   bulk   per integration point: xi_IP = N_IG(xi) xihat_IG, w* = w detJ_IG,
//          g = J_IP^-1 dN/dxi(xi_IP) (Element_Bulk::compute_jacobian_and_
//          residual, FEM/INT/src/ELEM/cl_FEM_Element_Bulk.cpp:258-355); Gram
//          A = sum w* g g^T by thread-owned entries, isotropic K from A (the
//          IWG_Isotropic_Struc_Linear_Bulk products, cl_FEM_IWG_Isotropic_
//          Struc_Linear_Bulk.cpp:42-207), R = K u;
//   double per facet point: leader / follower points from the facet's
//          parametric vertices (Element_Double_Sideset, cl_FEM_Element_Double_
//          Sideset.cpp:142-347), normal and w* from the facet geometry, the
//          traction operators n.D.B of both sides and the 48x48 pdof block
//          of the interface (cl_FEM_IWG_Isotropic_Struc_Linear_Interface.cpp:
//          51-386, SP_Nitsche_Interface) or the virtual-work ghost
//          (..._Virtual_Work_Ghost.cpp:50-244, SP_Ghost_Virtual_Work);
//   then   K_a = T^T K T over the column-sparse element T and the scatter
//          red.global.add.f64 at rowptr[f nu + b_i] + g |U(b_i)| + sidx[i][j].
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fem_bits.cuh"
#include "fem_internal.hpp"
#include "fem_shape.hpp"

namespace fem {
namespace {

constexpr int kChunk = 32;  // integration points per geometry chunk
constexpr int kMaxFP = 9;   // facet rule points (TRI_3, TRI_7, QUAD_2x2; QUAD_3x3)
constexpr int kNPE = 8, kNPD = 24, kNSYM = 300;
enum { CM_ASSEMBLE = 0, CM_ELEMENT = 1 };

struct SetDev {
    int kind;        // 0 bulk, 2 double-sided
    int iwg;
    int cut;         // bulk: integration cells given
    int ngp;         // rule points per integration cell / facet
    int nfv;         // facet vertices
    int facet_cell;  // FEM_GPU_CELL_TRI3 / QUAD4
    int rect;        // rectangular IP cells
    int pad;
    double lam_c, mu_c, alpha;
    const double* gp;  // [ngp][pdim]
    const double* gw;  // [ngp]
    const double* xe;  // bulk [neq][8][3]; double [neq][2][8][3]
    const double* E;
    const double* EF;
    const int32_t* nb;     // bulk [neq]; double [neq][2]
    const int32_t* bases;  // bulk [neq][NB]; double [neq][2][NB]
    const double* T;       // bulk [neq][8][NB]; double [neq][2][8][NB]
    const uint16_t* sidx;  // bulk [neq][NB][NB]; double [neq][2NB][2NB]
    const int64_t* ig_off;
    const double* ig_x;    // [ig][4][3]
    const double* ig_xi;
    const int64_t* fc_off;
    const double* fc_x;    // [facet][nfv][3]
    const double* fc_xl;
    const double* fc_xf;
    const double* vol;     // [neq][2]
    const double* g0;      // bulk, uncut: rule Gram table sum_q w dN/dxi dN/dxi [24][24]
};

struct Item {
    int32_t set;
    int32_t q0, q1;
    int32_t pad;
    int64_t eq;
};

struct ClusterArgs {
    const SetDev* sets;
    const Item* items;
    int64_t nitems;       // items of the CTA phase; the warp phase follows them
    int64_t nwarp_items;  // uncut rectangular cells (one warp each)
    unsigned long long* counter;  // [2]: CTA queue, warp queue
    const int32_t* rowptr;
    const int32_t* ulen;
    int64_t nu;
    const double* u;
    double* vals;
    double* rhs;
    double* Kout;
    double* Rout;
    int nmax;
    int mode;
    int64_t first;
    int* status;
};

// shared-memory layout: the bulk and the double-sided paths overlay one region
template <int NB>
struct CL {
    // bulk (doubles)
    static constexpr int sX = 0, sT = sX + 24, sTW = sT + 8 * NB, sU = sTW + 8 * NB, sUA = sU + 24,
                         sRP = sUA + 3 * NB, sA = sRP + 24, sK = sA + 576, sKT = sK + 576, sG = sKT + 72 * NB,
                         sWG = sG + kChunk * 24, sEnd = sWG + kChunk * 24;
    // double-sided (doubles)
    static constexpr int dX = 0, dT = dX + 48, dTW = dT + 16 * NB, dU = dTW + 16 * NB, dUA = dU + 48,
                         dR = dUA + 6 * NB, dK = dR + 48, dKT = dK + 2304, dWN = dKT + 288 * NB,
                         dNR = dWN + kMaxFP * 16, dGG = dNR + kMaxFP * 16, dWQ = dGG + kMaxFP * 48, dSC = dWQ + kMaxFP, dP = dSC + 8,
                         dEnd = dP + 2 * kMaxFP * 144;
    static constexpr int ND = sEnd > dEnd ? sEnd : dEnd;
    // ints (after the doubles): bases, row offsets, union lengths
    static constexpr int iB = 0, iRB = iB + 2 * NB, iUL = iRB + 6 * NB, NI = iUL + 2 * NB;
    // bytes: T node ids, counts, scatter slots
    static constexpr int bTN = 0, bTC = bTN + 16 * NB, bS = ((bTC + 2 * NB + 1) / 2) * 2, NBYTE = bS + 8 * NB * NB;
    static constexpr size_t bytes = ((size_t)ND * 8 + (size_t)NI * 4 + (size_t)NBYTE + 15) / 16 * 16;
};

__device__ __forceinline__ void ip_jacobian(const double* X, const double* dN, bool rect, double Ji[3][3],
                                            double& detJ) {
    double J[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            if (!rect || i == j)
                for (int a = 0; a < 8; ++a) s = fma(dN[i * 8 + a], X[a * 3 + j], s);
            J[i][j] = s;
        }
    if (rect) {
        detJ = J[1][1] * J[0][0] * J[2][2];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) Ji[i][j] = i == j ? 1.0 / J[i][i] : 0.0;
        return;
    }
    detJ = +J[0][0] * (J[1][1] * J[2][2] - J[2][1] * J[1][2]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
           J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    const double id = 1.0 / detJ;
    Ji[0][0] = (J[1][1] * J[2][2] - J[2][1] * J[1][2]) * id;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
    Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
    Ji[1][2] = (J[1][0] * J[0][2] - J[0][0] * J[1][2]) * id;
    Ji[2][0] = (J[1][0] * J[2][1] - J[2][0] * J[1][1]) * id;
    Ji[2][1] = (J[2][0] * J[0][1] - J[0][0] * J[2][1]) * id;
    Ji[2][2] = (J[0][0] * J[1][1] - J[1][0] * J[0][1]) * id;
}

// g = J^-1 dN/dxi at an IP-parametric point, g[i*8+a] = dN_a/dx_i
__device__ __forceinline__ void ip_gradients(const double* X, const double* xi, bool rect, double* N, double* g,
                                             double& detJ) {
    double dN[24], Ji[3][3];
    Shape<1>::eval(xi, N, dN);
    ip_jacobian(X, dN, rect, Ji, detJ);
    for (int i = 0; i < 3; ++i)
        for (int a = 0; a < 8; ++a) {
            double s;
            if (rect) {
                s = Ji[i][i] * dN[i * 8 + a];
            } else {
                s = 0.0;
                for (int k = 0; k < 3; ++k) s = fma(Ji[i][k], dN[k * 8 + a], s);
            }
            g[i * 8 + a] = s;
        }
}

// one integration point of a cut cluster: its IP-parametric position xi and
// w* = w detJ_IG (0 for points the reference skips)
__device__ void cut_point(const SetDev& S, int64_t e, int q, double* xi, double& ws) {
    const int k = q / S.ngp, qq = q - k * S.ngp;
    const int64_t gi = S.ig_off[e] + k;
    const double* xh = S.ig_xi + gi * 12;
    const double* xx = S.ig_x + gi * 12;
    double Nt[4], dNt[12];
    Shape<3>::eval(S.gp + qq * 3, Nt, dNt);
    for (int d = 0; d < 3; ++d) {
        double s = 0.0;
        for (int a = 0; a < 4; ++a) s = fma(Nt[a], xh[a * 3 + d], s);
        xi[d] = s;
    }
    // TET4 Jacobian rows x0-x2, x1-x2, x3-x2; detJ / 6
    double a0[3], a1[3], a3[3];
    for (int d = 0; d < 3; ++d) {
        a0[d] = xx[0 * 3 + d] - xx[2 * 3 + d];
        a1[d] = xx[1 * 3 + d] - xx[2 * 3 + d];
        a3[d] = xx[3 * 3 + d] - xx[2 * 3 + d];
    }
    const double detJ = (a0[0] * (a1[1] * a3[2] - a3[1] * a1[2]) - a0[1] * (a1[0] * a3[2] - a1[2] * a3[0]) +
                         a0[2] * (a1[0] * a3[1] - a1[1] * a3[0])) /
                        6.0;
    // points with detJ below -1e-6 are skipped (cl_FEM_Element_Bulk.cpp:164)
    ws = detJ < -1.0e-6 ? 0.0 : S.gw[qq] * detJ;
}

// one bulk integration point: gradients and w* (0 for points the reference skips)
__device__ void bulk_point(const SetDev& S, int64_t e, int q, const double* X, double* g, double& ws) {
    double xi[3], N[8], dj;
    if (!S.cut) {
        for (int d = 0; d < 3; ++d) xi[d] = S.gp[q * 3 + d];
        double detJ;
        ip_gradients(X, xi, S.rect, N, g, detJ);
        ws = detJ < -1.0e-6 ? 0.0 : S.gw[q] * detJ;
        return;
    }
    cut_point(S, e, q, xi, ws);
    ip_gradients(X, xi, S.rect, N, g, dj);
}

// Gram matrix of a rectangular IP cell from the moments of its points.  On a
// brick dN_a/dx_i = (1 / jd_i) dN_a/dxi_i, and dN_a/dxi_i is a combination of
// four of the seven monomials m = (1, xi, eta, zeta, xi eta, eta zeta, xi zeta):
//   dN_a/dxi   = s_x / 8 (1 + s_y eta + s_z zeta + s_y s_z eta zeta)
//   dN_a/deta  = s_y / 8 (1 + s_x xi  + s_z zeta + s_x s_z xi zeta)
//   dN_a/dzeta = s_z / 8 (1 + s_x xi  + s_y eta  + s_x s_y xi eta)
// so A[(i,a),(j,b)] = sum_q w*_q g_ia g_jb is a signed sum of 16 entries of the
// moment matrix M = sum_q w*_q m m^T, formed at 28 products per point instead
// of 300.
__device__ __forceinline__ void grad_monomials(int i, int a, int mono[4], double sgn[4]) {
    const double s[3] = {((a & 3) == 1 || (a & 3) == 2) ? 1.0 : -1.0, ((a & 3) >= 2) ? 1.0 : -1.0,
                         a >= 4 ? 1.0 : -1.0};
    // the two other coordinates of direction i and their product monomial
    const int o1 = i == 0 ? 1 : 0, o2 = i == 2 ? 1 : 2;
    const int prod = i == 0 ? 5 : i == 1 ? 6 : 4;
    mono[0] = 0;
    mono[1] = 1 + o1;
    mono[2] = 1 + o2;
    mono[3] = prod;
    sgn[0] = s[i];
    sgn[1] = s[i] * s[o1];
    sgn[2] = s[i] * s[o2];
    sgn[3] = s[i] * s[o1] * s[o2];
}

template <int NB, int W>
__device__ void bulk_item(const ClusterArgs& p, const SetDev& S, const Item& it, double* sd, int32_t* si,
                          unsigned char* sb) {
    using Lo = CL<NB>;
    constexpr int TH = 32 * W, NAD = 3 * NB;
    constexpr int PER = (kNSYM + TH - 1) / TH;
    const int tid = threadIdx.x;
    const int64_t e = it.eq;
    double* X = sd + Lo::sX;
    double* T = sd + Lo::sT;
    double* TW = sd + Lo::sTW;
    double* U = sd + Lo::sU;
    double* UA = sd + Lo::sUA;
    double* RP = sd + Lo::sRP;
    double* A = sd + Lo::sA;
    double* K = sd + Lo::sK;
    double* KT = sd + Lo::sKT;
    double* G = sd + Lo::sG;
    double* WG = sd + Lo::sWG;
    int32_t* B = si + Lo::iB;
    int32_t* RB = si + Lo::iRB;
    int32_t* UL = si + Lo::iUL;
    uint8_t* TN = sb + Lo::bTN;
    uint8_t* TC = sb + Lo::bTC;
    uint16_t* SL = reinterpret_cast<uint16_t*>(sb + Lo::bS);
    const int nb = S.nb[e];
    const double E = S.E[e];
    const bool assemble = p.mode == CM_ASSEMBLE;
    for (int i = tid; i < 24; i += TH) X[i] = S.xe[e * 24 + i];
    for (int i = tid; i < 8 * NB; i += TH) T[i] = S.T[e * 8 * NB + i];
    for (int i = tid; i < NB; i += TH) B[i] = S.bases[e * NB + i];
    if (assemble && p.vals)
        for (int i = tid; i < NB * NB; i += TH) SL[i] = S.sidx[e * NB * NB + i];
    __syncthreads();
    if (assemble) {
        for (int r = tid; r < NAD; r += TH) {
            const int f = r / NB, i = r - f * NB;
            RB[r] = i < nb ? p.rowptr[f * p.nu + B[i]] : 0;
        }
        for (int i = tid; i < NB; i += TH) UL[i] = i < nb ? p.ulen[B[i]] : 0;
    }
    for (int r = tid; r < NAD; r += TH) {
        const int f = r / NB, i = r - f * NB;
        UA[r] = (p.u && i < nb) ? p.u[f * p.nu + B[i]] : 0.0;
    }
    for (int j = tid; j < NB; j += TH) {
        int cnt = 0;
        for (int a = 0; a < 8; ++a) {
            const double t = T[a * NB + j];
            if (fem_nonzero(t)) {
                TN[j * 8 + cnt] = (uint8_t)a;
                TW[j * 8 + cnt] = t;
                ++cnt;
            }
        }
        TC[j] = (uint8_t)cnt;
    }
    // owned Gram entries
    int pr[PER], pc[PER];
    double acc[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        const int k = tid + j * TH;
        int r = 0, rem = k < kNSYM ? k : 0;
        while (rem >= kNPD - r) {
            rem -= kNPD - r;
            ++r;
        }
        pr[j] = r;
        pc[j] = r + rem;
        acc[j] = 0.0;
    }
    __syncthreads();
    if (!S.cut && S.rect && S.g0) {
        // constant Jacobian: A = detJ J^-1_i J^-1_j G0 (the rule's Gram table),
        // no per-point work (uncut rectangular cells)
        double jd[3];
        for (int i = 0; i < 3; ++i) {
            // edge lengths / 2 from the corner coordinates (J of the affine map)
            jd[i] = 0.5 * (X[6 * 3 + i] - X[0 * 3 + i]);
        }
        const double detJ = jd[1] * jd[0] * jd[2];
        const bool skip = detJ < -1.0e-6;  // cl_FEM_Element_Bulk.cpp:164
        // detJ / (J_ii J_jj): the product of the remaining diagonal entries
        // (off-diagonal pairs) or one division (diagonal pairs)
        const double cd[3] = {jd[1] * jd[2] / jd[0], jd[0] * jd[2] / jd[1], jd[0] * jd[1] / jd[2]};
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            if (tid + j * TH >= kNSYM) continue;
            const int i1 = pr[j] / 8, i2 = pc[j] / 8;
            const double cj = i1 == i2 ? cd[i1] : jd[3 - i1 - i2];
            acc[j] = skip ? 0.0 : cj * S.g0[pr[j] * 24 + pc[j]];
        }
    } else if (S.cut && S.rect) {
        // moments M = sum_q w* m m^T of the item's points (28 entries, lane l
        // < 28 of every warp owns entry l over the warp's share of the points)
        double* MM = G;   // [kChunk][8] monomials of the chunk's points
        double* WM = WG;  // [kChunk][8] w* times them
        const int lane = tid & 31, warp = tid >> 5;
        int ma = 0, mb = 0;
        {
            int rem = lane < 28 ? lane : 0;
            while (rem >= 7 - ma) {
                rem -= 7 - ma;
                ++ma;
            }
            mb = ma + rem;
        }
        double macc = 0.0;
        for (int q0 = it.q0; q0 < it.q1; q0 += kChunk) {
            const int nq = min(kChunk, it.q1 - q0);
            if (tid < kChunk) {
                double xi[3] = {0.0, 0.0, 0.0}, ws = 0.0;
                if (tid < nq) cut_point(S, e, q0 + tid, xi, ws);
                const double m[7] = {1.0, xi[0], xi[1], xi[2], xi[0] * xi[1], xi[1] * xi[2], xi[0] * xi[2]};
                for (int k = 0; k < 7; ++k) {
                    MM[tid * 8 + k] = m[k];
                    WM[tid * 8 + k] = ws * m[k];
                }
            }
            __syncthreads();
            if (lane < 28)
                for (int t = warp; t < nq; t += W) macc = fma(WM[t * 8 + ma], MM[t * 8 + mb], macc);
            __syncthreads();
        }
        // warp partial sums, then M (7 x 7) in the KT region (free until K T)
        double* part = KT + 64;
        if (lane < 28) part[warp * 28 + lane] = macc;
        __syncthreads();
        double* Mm = KT;
        if (tid < 28) {
            double v = 0.0;
            for (int w2 = 0; w2 < W; ++w2) v += part[w2 * 28 + tid];
            Mm[ma * 7 + mb] = v;
            Mm[mb * 7 + ma] = v;
        }
        __syncthreads();
        const double ij[3] = {1.0 / (0.5 * (X[6 * 3 + 0] - X[0])), 1.0 / (0.5 * (X[6 * 3 + 1] - X[1])),
                              1.0 / (0.5 * (X[6 * 3 + 2] - X[2]))};
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            if (tid + j * TH >= kNSYM) continue;
            const int i1 = pr[j] / 8, a = pr[j] - i1 * 8, i2 = pc[j] / 8, b = pc[j] - i2 * 8;
            int mu[4], mv[4];
            double su[4], sv[4];
            grad_monomials(i1, a, mu, su);
            grad_monomials(i2, b, mv, sv);
            double v = 0.0;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                double t = 0.0;
#pragma unroll
                for (int w2 = 0; w2 < 4; ++w2) t = fma(sv[w2], Mm[mu[u] * 7 + mv[w2]], t);
                v = fma(su[u], t, v);
            }
            acc[j] = v * (ij[i1] * ij[i2] * (1.0 / 64.0));
        }
        __syncthreads();
    } else
    for (int q0 = it.q0; q0 < it.q1; q0 += kChunk) {
        const int nq = min(kChunk, it.q1 - q0);
        if (tid < kChunk) {
            double g[24], ws = 0.0;
            if (tid < nq) bulk_point(S, e, q0 + tid, X, g, ws);
            else
                for (int i = 0; i < 24; ++i) g[i] = 0.0;
            for (int i = 0; i < 24; ++i) {
                G[tid * 24 + i] = g[i];
                WG[tid * 24 + i] = ws * g[i];
            }
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            if (tid + j * TH >= kNSYM) continue;
            double s = acc[j];
            for (int t = 0; t < nq; ++t) s = fma(WG[t * 24 + pr[j]], G[t * 24 + pc[j]], s);
            acc[j] = s;
        }
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        if (tid + j * TH >= kNSYM) continue;
        A[pr[j] * 24 + pc[j]] = acc[j];
        A[pc[j] * 24 + pr[j]] = acc[j];
    }
    // pdof values u = T u_a
    for (int r = tid; r < 24; r += TH) {
        const int f = r / 8, a = r - f * 8;
        double s = 0.0;
        for (int j = 0; j < nb; ++j) {
            const double t = T[a * NB + j];
            if (fem_nonzero(t)) s = fma(t, UA[f * NB + j], s);
        }
        U[r] = s;
    }
    __syncthreads();
    {
        const double lam = E * S.lam_c, mu = E * S.mu_c;
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            if (tid + j * TH >= kNSYM) continue;
            const int r = pr[j], c = pc[j];
            const int f = r / 8, a = r - f * 8, gg = c / 8, b = c - gg * 8;
            double v = lam * A[r * 24 + c] + mu * A[(gg * 8 + a) * 24 + f * 8 + b];
            if (f == gg) {
                double tr = 0.0;
                for (int kk = 0; kk < 3; ++kk) tr += A[(kk * 8 + a) * 24 + kk * 8 + b];
                v = fma(mu, tr, v);
            }
            K[r * 24 + c] = v;
            K[c * 24 + r] = v;
        }
    }
    __syncthreads();
    const bool want_r = (assemble && p.rhs) || (!assemble && p.Rout);
    if (want_r) {
        for (int r = tid; r < 24; r += TH) {
            double s = 0.0;
            for (int c = 0; c < 24; ++c) s = fma(K[r * 24 + c], U[c], s);
            RP[r] = s;
        }
        __syncthreads();
        for (int r = tid; r < NAD; r += TH) {
            const int f = r / NB, i = r - f * NB;
            if (i >= nb) continue;
            double s = 0.0;
            for (int k = 0; k < TC[i]; ++k) s = fma(TW[i * 8 + k], RP[f * 8 + TN[i * 8 + k]], s);
            if (assemble) atomicAdd(p.rhs + f * p.nu + B[i], s);
            else atomicAdd(p.Rout + (e - p.first) * p.nmax + r, s);
        }
    }
    const bool want_k = (assemble && p.vals) || (!assemble && p.Kout);
    if (!want_k) return;
    // KT = K T (24 x NAD)
    for (int idx = tid; idx < 24 * NAD; idx += TH) {
        const int row = idx / NAD, c = idx - row * NAD;
        const int gg = c / NB, j = c - gg * NB;
        double s = 0.0;
        const int cnt = j < nb ? TC[j] : 0;
        for (int k = 0; k < cnt; ++k) s = fma(K[row * 24 + gg * 8 + TN[j * 8 + k]], TW[j * 8 + k], s);
        KT[idx] = s;
    }
    __syncthreads();
    // K_a = T^T KT, upper triangle, scattered to both halves
    bool bad = false;
    constexpr int NUP = NAD * (NAD + 1) / 2;
    for (int k = tid; k < NUP; k += TH) {
        int r = 0, rem = k;
        while (rem >= NAD - r) {
            rem -= NAD - r;
            ++r;
        }
        const int c = r + rem;
        const int f = r / NB, i = r - f * NB, gg = c / NB, j = c - gg * NB;
        if (i >= nb || j >= nb) continue;
        double v = 0.0;
        for (int kk = 0; kk < TC[i]; ++kk) v = fma(TW[i * 8 + kk], KT[(f * 8 + TN[i * 8 + kk]) * NAD + c], v);
        bad |= !fem_finite(v);
        if (assemble) {
            atomicAdd(p.vals + RB[r] + gg * UL[i] + SL[i * NB + j], v);
            if (c != r) atomicAdd(p.vals + RB[c] + f * UL[j] + SL[j * NB + i], v);
        } else {
            double* Ko = p.Kout + (e - p.first) * (int64_t)p.nmax * p.nmax;
            atomicAdd(Ko + r + (int64_t)c * p.nmax, v);
            if (c != r) atomicAdd(Ko + c + (int64_t)r * p.nmax, v);
        }
    }
    if (bad) atomicOr(p.status, 1);
}

// facet geometry at a facet point: detJ (TRI3 |t1 x t2| / 2, QUAD4 |t1 x t2|,
// cl_MTK_Space_Interpolator.cpp:808-850) and the unit normal t1 x t2 / |.|
__device__ void facet_geometry(const SetDev& S, int64_t f, const double* xq, double& detJ, double* n) {
    double Nf[4], dNf[8];
    const int nfv = S.nfv;
    if (S.facet_cell == FEM_GPU_CELL_TRI3) Shape<2>::eval(xq, Nf, dNf);
    else Shape<0>::eval(xq, Nf, dNf);
    double t[2][3] = {{0, 0, 0}, {0, 0, 0}};
    for (int k = 0; k < nfv; ++k)
        for (int d = 0; d < 3; ++d)
            for (int m = 0; m < 2; ++m) t[m][d] = fma(dNf[m * nfv + k], S.fc_x[(f * nfv + k) * 3 + d], t[m][d]);
    const double c0 = t[0][1] * t[1][2] - t[0][2] * t[1][1];
    const double c1 = t[0][2] * t[1][0] - t[0][0] * t[1][2];
    const double c2 = t[0][0] * t[1][1] - t[0][1] * t[1][0];
    const double nn = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
    detJ = S.facet_cell == FEM_GPU_CELL_TRI3 ? nn / 2.0 : nn;
    // a degenerate facet contributes nothing (no normal)
    const double inv = nn > 0.0 ? 1.0 / nn : 0.0;
    n[0] = c0 * inv;
    n[1] = c1 * inv;
    n[2] = c2 * inv;
}

template <int NB, int W>
__device__ void double_item(const ClusterArgs& p, const SetDev& S, const Item& it, double* sd, int32_t* si,
                            unsigned char* sb) {
    using Lo = CL<NB>;
    constexpr int TH = 32 * W, NAD = 6 * NB, PER = 2304 / TH;
    const int tid = threadIdx.x;
    const int64_t e = it.eq;
    double* X = sd + Lo::dX;    // [2][8][3]
    double* T = sd + Lo::dT;    // [2][8][NB]
    double* TW = sd + Lo::dTW;  // [2][NB][8]
    double* U = sd + Lo::dU;    // [48]
    double* UA = sd + Lo::dUA;  // [2][3][NB]
    double* R = sd + Lo::dR;    // [48]
    double* K = sd + Lo::dK;    // [48][48]
    double* KT = sd + Lo::dKT;  // [48][NAD]
    double* WN = sd + Lo::dWN;  // [q][2][8]   w* N of both sides
    double* NR = sd + Lo::dNR;  // [q][2][8]   N of both sides
    double* GG = sd + Lo::dGG;  // [q][2][24]  gradients of both sides
    double* WQ = sd + Lo::dWQ;  // [q]         w* per facet point
    double* SC = sd + Lo::dSC;  // n0, n1, n2, area, wL, wF
    double* P = sd + Lo::dP;    // interface moments [2][8][2][3][8]
    double* Q = P + 768;        // interface moments [2][8][2][8] (whole cluster)
    double* GS = sd + Lo::dP;   // ghost: w* (n-projected strain) [q][2][3][24]
    double* TR = GS + kMaxFP * 144;  // ghost: traction operators [q][2][3][24]
    int32_t* B = si + Lo::iB;   // [2][NB]
    int32_t* RB = si + Lo::iRB; // [2][3][NB]
    int32_t* UL = si + Lo::iUL; // [2][NB]
    uint8_t* TN = sb + Lo::bTN; // [2][NB][8]
    uint8_t* TC = sb + Lo::bTC; // [2][NB]
    uint16_t* SL = reinterpret_cast<uint16_t*>(sb + Lo::bS);  // [2NB][2NB]
    const bool assemble = p.mode == CM_ASSEMBLE;
    // ghost penalties: virtual work (traction jump) or normal field (jump of du/dn)
    const bool normal_field = S.iwg == FEM_GPU_IWG_GHOST_NORMAL_FIELD;
    const bool ghost = S.iwg == FEM_GPU_IWG_STRUC_LINEAR_VW_GHOST || normal_field;
    const double beta = S.iwg == FEM_GPU_IWG_STRUC_LINEAR_INTERFACE_SYMMETRIC_NITSCHE ? -1.0 : 1.0;
    const int nbs[2] = {S.nb[2 * e], S.nb[2 * e + 1]};
    const double Es[2] = {S.E[e], S.EF[e]};
    const int ngp = S.ngp, nfv = S.nfv;
    for (int i = tid; i < 48; i += TH) X[i] = S.xe[e * 48 + i];
    for (int i = tid; i < 16 * NB; i += TH) T[i] = S.T[e * 16 * NB + i];
    for (int i = tid; i < 2 * NB; i += TH) B[i] = S.bases[e * 2 * NB + i];
    if (assemble && p.vals)
        for (int i = tid; i < 4 * NB * NB; i += TH) SL[i] = S.sidx[e * 4 * NB * NB + i];
    for (int j = tid; j < 2304; j += TH) K[j] = 0.0;
    if (!ghost) {
        for (int j = tid; j < 256; j += TH) Q[j] = 0.0;
        for (int j = tid; j < 2304; j += TH) KT[j] = 0.0;  // A1 (see below)
    }
    if (tid == 0) {
        SC[3] = 0.0;
        if (!ghost) {
            // SP_Nitsche_Interface weights (the surface measure enters at the end)
            const double vl = S.vol[2 * e] / Es[0], vf = S.vol[2 * e + 1] / Es[1];
            SC[4] = vl / (vl + vf);
            SC[5] = vf / (vl + vf);
        }
    }
    __syncthreads();
    for (int r = tid; r < NAD; r += TH) {
        const int s = r / (3 * NB), f = (r / NB) % 3, i = r % NB;
        const bool ok = i < nbs[s];
        if (assemble) RB[r] = ok ? p.rowptr[f * p.nu + B[s * NB + i]] : 0;
        UA[r] = (p.u && ok) ? p.u[f * p.nu + B[s * NB + i]] : 0.0;
    }
    if (assemble)
        for (int i = tid; i < 2 * NB; i += TH) UL[i] = (i % NB) < nbs[i / NB] ? p.ulen[B[i]] : 0;
    for (int jj = tid; jj < 2 * NB; jj += TH) {
        const int s = jj / NB, j = jj % NB;
        int cnt = 0;
        for (int a = 0; a < 8; ++a) {
            const double t = T[(s * 8 + a) * NB + j];
            if (fem_nonzero(t)) {
                TN[jj * 8 + cnt] = (uint8_t)a;
                TW[jj * 8 + cnt] = t;
                ++cnt;
            }
        }
        TC[jj] = (uint8_t)cnt;
    }
    const double wsd[2] = {SC[4], SC[5]};
    for (int64_t f = S.fc_off[e]; f < S.fc_off[e + 1]; ++f) {
        __syncthreads();
        // (A) facet points in parallel: lanes (q, side) for the gradients of the
        // IP cells, lanes q (second warp) for w* and the normal of the facet
        if (tid < 2 * ngp) {
            const int q = tid >> 1, side = tid & 1;
            const double* fx = side == 0 ? S.fc_xl : S.fc_xf;
            double Nf[4], dNf[8], xi[3] = {0, 0, 0};
            if (S.facet_cell == FEM_GPU_CELL_TRI3) Shape<2>::eval(S.gp + q * 2, Nf, dNf);
            else Shape<0>::eval(S.gp + q * 2, Nf, dNf);
            for (int k = 0; k < nfv; ++k)
                for (int d = 0; d < 3; ++d) xi[d] = fma(Nf[k], fx[(f * nfv + k) * 3 + d], xi[d]);
            double N[8], g[24], dj;
            ip_gradients(X + side * 24, xi, S.rect, N, g, dj);
            for (int a = 0; a < 8; ++a) NR[(q * 2 + side) * 8 + a] = N[a];
            for (int i = 0; i < 24; ++i) GG[(q * 2 + side) * 24 + i] = g[i];
        } else if (tid >= 32 && tid < 32 + ngp) {
            const int q = tid - 32;
            double dj, n[3];
            facet_geometry(S, f, S.gp + q * 2, dj, n);
            WQ[q] = dj < -1.0e-6 ? 0.0 : S.gw[q] * dj;
            if (q == 0) {
                SC[0] = n[0];
                SC[1] = n[1];
                SC[2] = n[2];
            }
        }
        __syncthreads();
        const double n[3] = {SC[0], SC[1], SC[2]};
        if (tid == 0) {
            double a = 0.0;
            for (int q = 0; q < ngp; ++q) a += WQ[q];
            SC[3] += a;  // facet measure (interface surface / ghost side)
        }
        if (!ghost) {
            // Interface.  The normal is constant on a flat facet, so every point
            // sum factors through the facet moments
            //   P[s][a][s'][k][b] = sum_q w* N_s[a] g_s'[k][b]
            //   Q[s][a][s'][b]    = sum_q w* N_s[a] N_s'[b]   (whole cluster)
            for (int i = tid; i < 16 * ngp; i += TH) WN[i] = NR[i] * WQ[i >> 4];
            __syncthreads();
            for (int j = tid; j < 1024; j += TH) {
                if (j < 768) {
                    // ((((s*8 + a)*2 + s2)*3 + k)*8 + b)
                    const int b = j & 7, k = (j >> 3) % 3, s2 = (j / 24) & 1, a = (j / 48) & 7, s1 = j / 384;
                    double v = 0.0;
                    for (int q = 0; q < ngp; ++q) v = fma(WN[(q * 2 + s1) * 8 + a], GG[(q * 2 + s2) * 24 + k * 8 + b], v);
                    P[j] = v;
                } else {
                    const int jj = j - 768, b = jj & 7, s2 = (jj >> 3) & 1, a = (jj >> 4) & 7, s1 = jj >> 7;
                    double v = Q[jj];
                    for (int q = 0; q < ngp; ++q) v = fma(WN[(q * 2 + s1) * 8 + a], NR[(q * 2 + s2) * 8 + b], v);
                    Q[jj] = v;
                }
            }
            __syncthreads();
            // A1[s][a][s'][i][k][b] += n_i P[s][a][s'][k][b]: the normal-weighted
            // moments of the whole cluster (K is formed once, after the last facet)
            for (int j = tid; j < 2304; j += TH) {
                const int kb = j % 24, i = (j / 24) % 3, pre = j / 72;  // pre = (s*8 + a)*2 + s'
                KT[j] = fma(n[i], P[pre * 24 + kb], KT[j]);
            }
        } else if (normal_field) {
            // Normal-field ghost: per point the normal derivatives DN[s][a] = n . g_s[:, a]
            // of both sides, then K[(s,f,a),(s',f,b)] += +-sum_q w* DN[s][a] DN[s'][b]
            // (the same for every component f; gamma at the end)
            for (int idx = tid; idx < ngp * 16; idx += TH) {
                const int q = idx >> 4, sd_ = (idx >> 3) & 1, a = idx & 7;
                const double* g = GG + (q * 2 + sd_) * 24;
                GS[idx] = n[0] * g[a] + n[1] * g[8 + a] + n[2] * g[16 + a];
            }
            __syncthreads();
            for (int j = 0; j < PER; ++j) {
                const int idx = tid + j * TH;
                const int r = idx / 48, c = idx % 48;
                const int sr = r / 24, rr = r % 24, sc = c / 24, cc = c % 24;
                if (rr / 8 != cc / 8) continue;
                double v = 0.0;
                for (int q = 0; q < ngp; ++q)
                    v = fma(WQ[q] * GS[q * 16 + sr * 8 + rr % 8], GS[q * 16 + sc * 8 + cc % 8], v);
                K[idx] = fma(sr == sc ? 1.0 : -1.0, v, K[idx]);
            }
        } else {
            // Ghost: per point w* (n-projected strain) and the traction operators of
            // both sides, then K += sum_q sum_h GS_q[h]^T TR_q[h] (alpha h_G at the end)
            for (int idx = tid; idx < ngp * 144; idx += TH) {
                const int q = idx / 144, rem = idx % 144, s = rem / 72, fr = (rem / 24) % 3, c = rem % 24;
                const int gg = c / 8, b = c % 8;
                const double* g = GG + (q * 2 + s) * 24;
                const double ng = n[0] * g[b] + n[1] * g[8 + b] + n[2] * g[16 + b];
                const double lam = Es[s] * S.lam_c, mu = Es[s] * S.mu_c;
                TR[idx] = lam * n[fr] * g[gg * 8 + b] + mu * (n[gg] * g[fr * 8 + b] + (fr == gg ? ng : 0.0));
                const double gs = (fr == gg ? ng - n[fr] * g[fr * 8 + b] : 0.0) + n[gg] * g[fr * 8 + b];
                GS[idx] = (s == 0 ? WQ[q] : -WQ[q]) * gs;
            }
            __syncthreads();
            for (int j = 0; j < PER; ++j) {
                const int idx = tid + j * TH;
                const int r = idx / 48, c = idx % 48;
                const int sr = r / 24, rr = r % 24, sc = c / 24, cc = c % 24;
                double v = 0.0;
                for (int q = 0; q < ngp; ++q) {
                    const double* gs = GS + q * 144 + sr * 72 + rr;
                    const double* tr = TR + q * 144 + sc * 72 + cc;
                    v = fma(gs[0], tr[0], v);
                    v = fma(gs[24], tr[24], v);
                    v = fma(gs[48], tr[48], v);
                }
                K[idx] = fma(sc == 0 ? 1.0 : -1.0, v, K[idx]);
            }
        }
    }
    __syncthreads();
    if (!ghost) {
        // Interface K from the cluster moments (IWG_Isotropic_Struc_Linear_
        // Interface::compute_jacobian with the linear CM's traction operators):
        //   T1 = -s_r w_c sum w* N_r[a] TR_c[f][(g,b)]
        //      = -s_r w_c (lam_c A1[r][c][f][g][b] + mu_c A1[r][c][g][f][b] + d_fg mu_c sum_k A1[r][c][k][k][b])
        //   T2 = beta w_r s_c sum w* TR_r[g][(f,a)] N_c[b]   (the same with the roles of r and c swapped)
        const double* A1 = KT;
        for (int j = 0; j < PER; ++j) {
            const int idx = tid + j * TH;
            const int r = idx / 48, c = idx % 48;
            const int sr = r / 24, rr = r % 24, sc = c / 24, cc = c % 24;
            const int fr = rr / 8, a = rr % 8, gc = cc / 8, b = cc % 8;
            const double sgr = sr == 0 ? 1.0 : -1.0, sgc = sc == 0 ? 1.0 : -1.0;
            const double* M1 = A1 + ((sr * 8 + a) * 2 + sc) * 72;  // [i][k][b] of (sr, a, sc)
            const double* M2 = A1 + ((sc * 8 + b) * 2 + sr) * 72;  // [i][k][a] of (sc, b, sr)
            double t1 = Es[sc] * (S.lam_c * M1[fr * 24 + gc * 8 + b] + S.mu_c * M1[gc * 24 + fr * 8 + b]);
            double t2 = Es[sr] * (S.lam_c * M2[gc * 24 + fr * 8 + a] + S.mu_c * M2[fr * 24 + gc * 8 + a]);
            if (fr == gc) {
                t1 += Es[sc] * S.mu_c * (M1[b] + M1[24 + 8 + b] + M1[48 + 16 + b]);
                t2 += Es[sr] * S.mu_c * (M2[a] + M2[24 + 8 + a] + M2[48 + 16 + a]);
            }
            K[idx] += -sgr * wsd[sc] * t1 + beta * wsd[sr] * sgc * t2;  // thread-owned entry
        }
    }
    // stabilization parameters from the cluster measures, applied once
    if (!ghost) {
        // SP_Nitsche_Interface: gamma = 2 alpha |G| / (V_L/E_L + V_F/E_F)
        const double vl = S.vol[2 * e] / Es[0], vf = S.vol[2 * e + 1] / Es[1];
        const double gamma = 2.0 * S.alpha * SC[3] / (vl + vf);
        for (int j = 0; j < PER; ++j) {
            const int idx = tid + j * TH;
            const int r = idx / 48, c = idx % 48;
            const int sr = r / 24, rr = r % 24, sc = c / 24, cc = c % 24;
            if (rr / 8 != cc / 8) continue;
            const double sg = (sr == sc) ? gamma : -gamma;
            K[idx] = fma(sg, Q[((sr * 8 + rr % 8) * 2 + sc) * 8 + cc % 8], K[idx]);
        }
    } else {
        // SP_Ghost_Virtual_Work: alpha h^(2(p-1)+1), p = 1, h = sqrt(4 A / pi);
        // SP_Ghost_Displacement: the same times the leader's modulus
        const double h = sqrt(4.0 * SC[3] / 3.14159265358979323846);
        const double gamma = normal_field ? S.alpha * h * Es[0] : S.alpha * h;
        for (int j = 0; j < PER; ++j) K[tid + j * TH] *= gamma;
    }
    // pdof values of both sides
    for (int r = tid; r < 48; r += TH) {
        const int s = r / 24, fr = (r / 8) % 3, a = r % 8;
        double v = 0.0;
        for (int j = 0; j < nbs[s]; ++j) {
            const double t = T[(s * 8 + a) * NB + j];
            if (fem_nonzero(t)) v = fma(t, UA[(s * 3 + fr) * NB + j], v);
        }
        U[r] = v;
    }
    __syncthreads();
    const bool want_r = (assemble && p.rhs) || (!assemble && p.Rout);
    if (want_r) {
        for (int r = tid; r < 48; r += TH) {
            double s = 0.0;
            for (int c = 0; c < 48; ++c) s = fma(K[r * 48 + c], U[c], s);
            R[r] = s;
        }
        __syncthreads();
        for (int r = tid; r < NAD; r += TH) {
            const int s = r / (3 * NB), fr = (r / NB) % 3, i = r % NB;
            if (i >= nbs[s]) continue;
            const int col = s * NB + i;
            double v = 0.0;
            for (int k = 0; k < TC[col]; ++k) v = fma(TW[col * 8 + k], R[s * 24 + fr * 8 + TN[col * 8 + k]], v);
            if (assemble) atomicAdd(p.rhs + fr * p.nu + B[col], v);
            else atomicAdd(p.Rout + (e - p.first) * p.nmax + r, v);
        }
    }
    const bool want_k = (assemble && p.vals) || (!assemble && p.Kout);
    if (!want_k) return;
    for (int idx = tid; idx < 48 * NAD; idx += TH) {
        const int row = idx / NAD, c = idx % NAD;
        const int s = c / (3 * NB), gc = (c / NB) % 3, j = c % NB;
        const int col = s * NB + j;
        double v = 0.0;
        const int cnt = j < nbs[s] ? TC[col] : 0;
        for (int k = 0; k < cnt; ++k) v = fma(K[row * 48 + s * 24 + gc * 8 + TN[col * 8 + k]], TW[col * 8 + k], v);
        KT[idx] = v;
    }
    __syncthreads();
    bool bad = false;
    for (int idx = tid; idx < NAD * NAD; idx += TH) {
        const int r = idx / NAD, c = idx % NAD;
        const int sr = r / (3 * NB), fr = (r / NB) % 3, i = r % NB;
        const int sc = c / (3 * NB), gc = (c / NB) % 3, j = c % NB;
        if (i >= nbs[sr] || j >= nbs[sc]) continue;
        const int coli = sr * NB + i, colj = sc * NB + j;
        double v = 0.0;
        for (int k = 0; k < TC[coli]; ++k)
            v = fma(TW[coli * 8 + k], KT[(sr * 24 + fr * 8 + TN[coli * 8 + k]) * NAD + c], v);
        bad |= !fem_finite(v);
        if (assemble) atomicAdd(p.vals + RB[r] + gc * UL[coli] + SL[coli * 2 * NB + colj], v);
        else atomicAdd(p.Kout + (e - p.first) * (int64_t)p.nmax * p.nmax + r + (int64_t)c * p.nmax, v);
    }
    if (bad) atomicOr(p.status, 1);
}

// per-warp layout of the uncut-cell phase (one cell per warp)
template <int NB>
struct WLay {
    static constexpr int oX = 0, oT = oX + 24, oTW = oT + 8 * NB, oU = oTW + 8 * NB, oUA = oU + 24,
                         oRP = oUA + 3 * NB, oK = oRP + 24, oKT = oK + 576, ND = oKT + 72 * NB;
    static constexpr int iB = 0, iRB = iB + NB, iUL = iRB + 3 * NB, NI = iUL + NB;
    static constexpr int bTN = 0, bTC = bTN + 8 * NB, bS = ((bTC + NB + 1) / 2) * 2, NBYTE = bS + 2 * NB * NB;
    static constexpr size_t bytes = ((size_t)ND * 8 + (size_t)NI * 4 + (size_t)NBYTE + 15) / 16 * 16;
};

// An uncut rectangular cell on one warp (no CTA barriers): A = detJ J^-1_i
// J^-1_j G0 from the rule's Gram table, the isotropic K, R = K u, K_a = T^T K T
// and the scatter -- the same arithmetic as bulk_item's constant-Jacobian branch.
template <int NB>
__device__ void uncut_warp(const ClusterArgs& p, const SetDev& S, int64_t e, unsigned char* ws) {
    using L = WLay<NB>;
    constexpr int NAD = 3 * NB, NUP = NAD * (NAD + 1) / 2;
    const int lane = threadIdx.x & 31;
    double* sd = reinterpret_cast<double*>(ws);
    int32_t* si = reinterpret_cast<int32_t*>(sd + L::ND);
    unsigned char* sb = reinterpret_cast<unsigned char*>(si + L::NI);
    double* X = sd + L::oX;
    double* T = sd + L::oT;
    double* TW = sd + L::oTW;
    double* U = sd + L::oU;
    double* UA = sd + L::oUA;
    double* RP = sd + L::oRP;
    double* K = sd + L::oK;
    double* KT = sd + L::oKT;
    int32_t* B = si + L::iB;
    int32_t* RB = si + L::iRB;
    int32_t* UL = si + L::iUL;
    uint8_t* TN = sb + L::bTN;
    uint8_t* TC = sb + L::bTC;
    uint16_t* SL = reinterpret_cast<uint16_t*>(sb + L::bS);
    const bool assemble = p.mode == CM_ASSEMBLE;
    const int nb = S.nb[e];
    const double E = S.E[e];
    if (lane < 24) X[lane] = S.xe[e * 24 + lane];
    for (int i = lane; i < 8 * NB; i += 32) T[i] = S.T[e * 8 * NB + i];
    if (lane < NB) B[lane] = S.bases[e * NB + lane];
    if (assemble && p.vals)
        for (int i = lane; i < NB * NB; i += 32) SL[i] = S.sidx[e * NB * NB + i];
    __syncwarp();
    for (int r = lane; r < NAD; r += 32) {
        const int f = r / NB, i = r - f * NB;
        if (assemble) RB[r] = i < nb ? p.rowptr[f * p.nu + B[i]] : 0;
        UA[r] = (p.u && i < nb) ? p.u[f * p.nu + B[i]] : 0.0;
    }
    if (assemble && lane < NB) UL[lane] = lane < nb ? p.ulen[B[lane]] : 0;
    if (lane < NB) {
        int cnt = 0;
        for (int a = 0; a < 8; ++a) {
            const double t = T[a * NB + lane];
            if (fem_nonzero(t)) {
                TN[lane * 8 + cnt] = (uint8_t)a;
                TW[lane * 8 + cnt] = t;
                ++cnt;
            }
        }
        TC[lane] = (uint8_t)cnt;
    }
    __syncwarp();
    double jd[3];
    for (int i = 0; i < 3; ++i) jd[i] = 0.5 * (X[6 * 3 + i] - X[0 * 3 + i]);
    const bool skip = jd[1] * jd[0] * jd[2] < -1.0e-6;  // cl_FEM_Element_Bulk.cpp:164
    const double cd[3] = {jd[1] * jd[2] / jd[0], jd[0] * jd[2] / jd[1], jd[0] * jd[1] / jd[2]};
    const double lam = E * S.lam_c, mu = E * S.mu_c;
    const double* G0 = S.g0;
    for (int k = lane; k < kNSYM; k += 32) {
        int r = 0, rem = k;
        while (rem >= kNPD - r) {
            rem -= kNPD - r;
            ++r;
        }
        const int c = r + rem;
        const int f = r / 8, a = r - f * 8, gg = c / 8, b = c - gg * 8;
        const double cfg = f == gg ? cd[f] : jd[3 - f - gg];
        double v = lam * cfg * __ldg(G0 + r * 24 + c) + mu * cfg * __ldg(G0 + (gg * 8 + a) * 24 + f * 8 + b);
        if (f == gg)
            for (int kk = 0; kk < 3; ++kk) v = fma(mu * cd[kk], __ldg(G0 + (kk * 8 + a) * 24 + kk * 8 + b), v);
        if (skip) v = 0.0;
        K[r * 24 + c] = v;
        K[c * 24 + r] = v;
    }
    if (lane < 24) {
        const int f = lane / 8, a = lane - f * 8;
        double v = 0.0;
        for (int j = 0; j < nb; ++j) {
            const double t = T[a * NB + j];
            if (fem_nonzero(t)) v = fma(t, UA[f * NB + j], v);
        }
        U[lane] = v;
    }
    __syncwarp();
    const bool want_r = (assemble && p.rhs) || (!assemble && p.Rout);
    if (want_r) {
        if (lane < 24) {
            double v = 0.0;
            for (int c = 0; c < 24; ++c) v = fma(K[lane * 24 + c], U[c], v);
            RP[lane] = v;
        }
        __syncwarp();
        for (int r = lane; r < NAD; r += 32) {
            const int f = r / NB, i = r - f * NB;
            if (i >= nb) continue;
            double v = 0.0;
            for (int k = 0; k < TC[i]; ++k) v = fma(TW[i * 8 + k], RP[f * 8 + TN[i * 8 + k]], v);
            if (assemble) atomicAdd(p.rhs + f * p.nu + B[i], v);
            else atomicAdd(p.Rout + (e - p.first) * p.nmax + r, v);
        }
    }
    const bool want_k = (assemble && p.vals) || (!assemble && p.Kout);
    if (!want_k) {
        __syncwarp();
        return;
    }
    for (int idx = lane; idx < 24 * NAD; idx += 32) {
        const int row = idx / NAD, c = idx - row * NAD;
        const int gg = c / NB, j = c - gg * NB;
        double v = 0.0;
        const int cnt = j < nb ? TC[j] : 0;
        for (int k = 0; k < cnt; ++k) v = fma(K[row * 24 + gg * 8 + TN[j * 8 + k]], TW[j * 8 + k], v);
        KT[idx] = v;
    }
    __syncwarp();
    bool bad = false;
    for (int k = lane; k < NUP; k += 32) {
        int r = 0, rem = k;
        while (rem >= NAD - r) {
            rem -= NAD - r;
            ++r;
        }
        const int c = r + rem;
        const int f = r / NB, i = r - f * NB, gg = c / NB, j = c - gg * NB;
        if (i >= nb || j >= nb) continue;
        double v = 0.0;
        for (int kk = 0; kk < TC[i]; ++kk) v = fma(TW[i * 8 + kk], KT[(f * 8 + TN[i * 8 + kk]) * NAD + c], v);
        bad |= !fem_finite(v);
        if (assemble) {
            atomicAdd(p.vals + RB[r] + gg * UL[i] + SL[i * NB + j], v);
            if (c != r) atomicAdd(p.vals + RB[c] + f * UL[j] + SL[j * NB + i], v);
        } else {
            double* Ko = p.Kout + (e - p.first) * (int64_t)p.nmax * p.nmax;
            atomicAdd(Ko + r + (int64_t)c * p.nmax, v);
            if (c != r) atomicAdd(Ko + c + (int64_t)r * p.nmax, v);
        }
    }
    if (bad) atomicOr(p.status, 1);
    __syncwarp();
}

template <int NB, int W>
__global__ void __launch_bounds__(32 * W, (384 / (32 * W)) > 0 ? 384 / (32 * W) : 1) cluster_kernel(ClusterArgs p) {
    using Lo = CL<NB>;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ long long s_item;
    double* sd = reinterpret_cast<double*>(smem);
    int32_t* si = reinterpret_cast<int32_t*>(sd + Lo::ND);
    unsigned char* sb = reinterpret_cast<unsigned char*>(si + Lo::NI);
    // phase 1: heavy clusters (cut, interface, ghost), one per CTA
    for (;;) {
        if (threadIdx.x == 0) s_item = (long long)atomicAdd(p.counter, 1ull);
        __syncthreads();
        const long long idx = s_item;
        if (idx >= p.nitems) break;
        const Item it = p.items[idx];
        const SetDev& S = p.sets[it.set];
        if (S.kind == 2) double_item<NB, W>(p, S, it, sd, si, sb);
        else bulk_item<NB, W>(p, S, it, sd, si, sb);
        __syncthreads();
    }
    // phase 2: uncut rectangular cells, one per warp
    constexpr int WFIT = (int)(Lo::bytes / WLay<NB>::bytes) < W ? (int)(Lo::bytes / WLay<NB>::bytes) : W;
    const int warp = threadIdx.x >> 5;
    if (p.nwarp_items == 0 || warp >= WFIT) return;
    unsigned char* ws = smem + (size_t)warp * WLay<NB>::bytes;
    for (;;) {
        long long idx = 0;
        if ((threadIdx.x & 31) == 0) idx = (long long)atomicAdd(p.counter + 1, 1ull);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= p.nwarp_items) break;
        const Item it = p.items[p.nitems + idx];
        uncut_warp<NB>(p, p.sets[it.set], it.eq, ws);
    }
}

// ---------------------------------------------------------------------------
// host side
struct Kernel {
    const void* fn;
    size_t smem;
    int threads;
};

bool pick_kernel(int nb, int warps, Kernel& k) {
#define FEM_CL(NBV, WV)                                                              \
    if (nb == NBV && warps == WV) {                                                  \
        k = {(const void*)cluster_kernel<NBV, WV>, CL<NBV>::bytes, 32 * WV};         \
        return true;                                                                 \
    }
    FEM_CL(8, 2)
    FEM_CL(8, 4)
    FEM_CL(8, 8)
    FEM_CL(27, 2)
    FEM_CL(27, 4)
    FEM_CL(27, 8)
#undef FEM_CL
    return false;
}

struct Batch {
    DeviceBuf sets, items, counter;
    int64_t nitems = 0;   // CTA-phase items (the warp-phase items follow them)
    int64_t nwarp = 0;    // uncut rectangular cells
    int nb = 0;
    int warps = 4, split = 64;
    bool built = false;
    cudaStream_t cap = nullptr;
    cudaGraphExec_t exec = nullptr;
    const void *gu = nullptr, *gv = nullptr, *gr = nullptr;
    int nside = 0;
};

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

fem_gpu_status cfail(fem_gpu_ctx* c, cudaError_t e, const char* what) {
    return fail(c, e == cudaErrorMemoryAllocation ? FEM_GPU_OUT_OF_MEMORY : FEM_GPU_CUDA_ERROR,
                std::string(what) + ": " + cudaGetErrorString(e));
}

double lam_of(int model, double nu) {
    return model == FEM_GPU_MODEL_PLANE_STRESS ? nu / (1.0 - nu * nu) : nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
}

int width_of(int maxnb) { return maxnb <= 8 ? 8 : maxnb <= 27 ? 27 : 0; }

// device descriptor of a set for the cluster kernel (bulk sets of any kind, double-sided sets)
bool set_dev(const fem_gpu_ctx* c, const SetData& s, SetDev& d) {
    std::memset(&d, 0, sizeof(d));
    d.kind = s.kind;
    d.rect = c->shape == FEM_GPU_SHAPE_RECTANGULAR;
    d.gp = (const double*)s.d_gp.p;
    d.gw = (const double*)s.d_gw.p;
    d.xe = (const double*)s.d_xe.p;
    d.E = (const double*)s.d_E.p;
    d.nb = (const int32_t*)s.d_nb.p;
    d.bases = (const int32_t*)s.d_bases.p;
    d.T = (const double*)s.d_T.p;
    d.sidx = (const uint16_t*)s.d_sidx.p;
    d.ngp = s.ngp;
    if (s.kind == 0) {
        d.iwg = s.bulk.iwg_type;
        d.cut = !s.ig_off.empty();
        d.lam_c = lam_of(s.bulk.model_type, s.bulk.poisson_ratio);
        d.mu_c = 1.0 / (2.0 * (1.0 + s.bulk.poisson_ratio));
        d.ig_off = (const int64_t*)s.d_igoff.p;
        d.ig_x = (const double*)s.d_igx.p;
        d.ig_xi = (const double*)s.d_igxi.p;
        d.g0 = d.cut ? nullptr : (const double*)s.d_g0.p;
        return s.rhoe.empty();
    }
    if (s.kind == 2) {
        d.iwg = s.dside.iwg_type;
        d.nfv = s.nfv;
        d.facet_cell = s.dside.facet_cell_type;
        d.lam_c = lam_of(s.dside.model_type, s.dside.poisson_ratio);
        d.mu_c = 1.0 / (2.0 * (1.0 + s.dside.poisson_ratio));
        d.alpha = s.dside.alpha;
        d.EF = (const double*)s.d_EF.p;
        d.fc_off = (const int64_t*)s.d_fcoff.p;
        d.fc_x = (const double*)s.d_fcx.p;
        d.fc_xl = (const double*)s.d_fcxl.p;
        d.fc_xf = (const double*)s.d_fcxf.p;
        d.vol = (const double*)s.d_vol.p;
        return true;
    }
    return false;
}

// integration points of an equation object (bulk) or facet points (double)
int64_t points_of(const SetData& s, int64_t e) {
    if (s.kind == 2) return (s.fc_off[e + 1] - s.fc_off[e]) * s.ngp;
    if (s.ig_off.empty()) return s.ngp;
    return (s.ig_off[e + 1] - s.ig_off[e]) * s.ngp;
}

void add_items(const SetData& s, int set, int64_t first, int64_t count, int split, std::vector<Item>& items,
               std::vector<double>& cost) {
    for (int64_t e = first; e < first + count; ++e) {
        const int64_t np = points_of(s, e);
        if (s.kind == 2 || split <= 0 || np <= split) {
            items.push_back({set, 0, (int32_t)np, 0, e});
            cost.push_back(s.kind == 2 ? 200.0 + 24.0 * np : 60.0 + np);
            continue;
        }
        for (int64_t q = 0; q < np; q += split) {
            items.push_back({set, (int32_t)q, (int32_t)std::min<int64_t>(np, q + split), 0, e});
            cost.push_back(60.0 + (double)std::min<int64_t>(split, np - q));
        }
    }
}

// items in decreasing cost order (stable: equal-cost items keep mesh order)
std::vector<Item> lpt_order(const std::vector<Item>& items, const std::vector<double>& cost) {
    std::vector<int64_t> idx(items.size());
    for (size_t i = 0; i < idx.size(); ++i) idx[i] = (int64_t)i;
    std::stable_sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) { return cost[a] > cost[b]; });
    std::vector<Item> out(items.size());
    for (size_t i = 0; i < idx.size(); ++i) out[i] = items[idx[i]];
    return out;
}

fem_gpu_status launch(fem_gpu_ctx* c, const Kernel& k, ClusterArgs& a, cudaStream_t st) {
    cudaError_t e = cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem);
    if (e != cudaSuccess) return cfail(c, e, "cluster smem attribute");
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k.fn, k.threads, k.smem);
    if (e != cudaSuccess) return cfail(c, e, "cluster occupancy");
    if (per_sm < 1) return fail(c, FEM_GPU_UNSUPPORTED, "cluster kernel does not fit on an SM");
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t blocks = (int64_t)std::max(sms, 1) * per_sm;
    const int64_t work = a.nitems + (a.nwarp_items + k.threads / 32 - 1) / (k.threads / 32);
    if (blocks > work) blocks = std::max<int64_t>(work, 1);
    void* args[] = {&a};
    e = cudaLaunchKernel(k.fn, dim3((unsigned)blocks), dim3(k.threads), args, k.smem, st);
    if (e != cudaSuccess) return cfail(c, e, "cluster launch");
    c->launches++;
    return FEM_GPU_OK;
}

ClusterArgs base_args(fem_gpu_ctx* c) {
    ClusterArgs a{};
    a.rowptr = (const int32_t*)c->d_rowptr.p;
    a.ulen = (const int32_t*)c->d_ulen.p;
    a.nu = c->num_used;
    a.status = (int*)c->d_status.p;
    return a;
}

Batch* batch_of(fem_gpu_ctx* c) {
    if (!c->batch) c->batch = new Batch;
    return (Batch*)c->batch;
}

void drop_graph(Batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    b->gu = b->gv = b->gr = nullptr;
}

// sets of the batched launch and their common basis width
fem_gpu_status build_batch(fem_gpu_ctx* c, Batch* b) {
    cudaStream_t st = (cudaStream_t)c->stream;
    std::vector<SetDev> devs(c->sets.size());
    std::vector<Item> items, warp_items;
    std::vector<double> cost;
    int nb = 0;
    b->nside = 0;
    for (size_t k = 0; k < c->sets.size(); ++k) {
        const SetData& s = c->sets[k];
        if (s.neq == 0) continue;
        if (s.kind == 1) {
            b->nside++;
            continue;
        }
        const int w = s.kind == 2 ? s.maxnb : s.nbsel;
        if (nb && w != nb) return fail(c, FEM_GPU_UNSUPPORTED, "batched launch needs one basis width for all sets");
        nb = w;
        if (!set_dev(c, s, devs[k])) return fail(c, FEM_GPU_UNSUPPORTED, "density sets are not batched");
        if (!devs[k].gp) return fail(c, FEM_GPU_NOT_FINALIZED, "set rule tables");
        if (s.kind == 0 && !devs[k].cut && devs[k].rect && devs[k].g0) {
            // uncut rectangular cells: the warp phase, in mesh order
            for (int64_t e = 0; e < s.neq; ++e) warp_items.push_back({(int32_t)k, 0, s.ngp, 0, e});
            continue;
        }
        add_items(s, (int)k, 0, s.neq, b->split, items, cost);
    }
    if (!nb && items.empty() && warp_items.empty()) nb = 8;  // every volume set empty: the launch finds no items
    if (nb != 8 && nb != 27) return fail(c, FEM_GPU_UNSUPPORTED, "batched launch: basis width must be 8 or 27");
    std::vector<Item> ordered = lpt_order(items, cost);
    const int64_t ncta = (int64_t)ordered.size();
    ordered.insert(ordered.end(), warp_items.begin(), warp_items.end());
    cudaError_t e = upload(b->sets, devs, st);
    if (e == cudaSuccess) e = upload(b->items, ordered, st);
    if (e == cudaSuccess && !b->counter.p) {
        std::vector<unsigned long long> z(2, 0);
        e = upload(b->counter, z, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cfail(c, e, "batch upload");
    b->nitems = ncta;
    b->nwarp = (int64_t)warp_items.size();
    b->nb = nb;
    b->built = true;
    drop_graph(b);
    return FEM_GPU_OK;
}

fem_gpu_status enqueue_batch(fem_gpu_ctx* c, Batch* b, const double* u, double* vals, double* rhs, cudaStream_t st,
                             bool zero, fem_gpu_status (*side)(fem_gpu_ctx*, int, const double*, double*, double*,
                                                               cudaStream_t)) {
    const int64_t nad = c->num_used * c->dim;
    if (zero) {
        if (vals) cudaMemsetAsync(vals, 0, c->nnz * sizeof(double), st);
        if (rhs) cudaMemsetAsync(rhs, 0, nad * sizeof(double), st);
    }
    cudaMemsetAsync(b->counter.p, 0, 2 * sizeof(unsigned long long), st);
    Kernel k;
    if (!pick_kernel(b->nb, b->warps, k)) return fail(c, FEM_GPU_UNSUPPORTED, "no cluster kernel instance");
    ClusterArgs a = base_args(c);
    a.sets = (const SetDev*)b->sets.p;
    a.items = (const Item*)b->items.p;
    a.nitems = b->nitems;
    a.nwarp_items = b->nwarp;
    a.counter = (unsigned long long*)b->counter.p;
    a.u = u;
    a.vals = vals;
    a.rhs = rhs;
    a.mode = CM_ASSEMBLE;
    fem_gpu_status r = launch(c, k, a, st);
    for (size_t s = 0; s < c->sets.size() && r == FEM_GPU_OK; ++s)
        if (c->sets[s].kind == 1 && c->sets[s].neq > 0) r = side(c, (int)s, u, vals, rhs, st);
    return r;
}

}  // namespace

bool cluster_set(const fem_gpu_ctx* c, int set) {
    const SetData& s = c->sets[set];
    return s.kind == 2 || (s.kind == 0 && !s.ig_off.empty());
}

// upload of a cut or double-sided set, arrays repacked to the kernel width
fem_gpu_status cluster_finalize(fem_gpu_ctx* c, int set) {
    SetData& s = c->sets[set];
    cudaStream_t st = (cudaStream_t)c->stream;
    if (c->dim != 3 || c->ip_cell != FEM_GPU_CELL_HEX8)
        return fail(c, FEM_GPU_UNSUPPORTED, "cut and double-sided clusters need a 3D HEX8 model");
    if (s.kind == 0 && s.bulk.ig_cell_type != FEM_GPU_CELL_TET4)
        return fail(c, FEM_GPU_UNSUPPORTED, "cut clusters need TET4 integration cells");
    if (s.kind == 0 && !s.rhoe.empty()) return fail(c, FEM_GPU_UNSUPPORTED, "density field on cut clusters");
    const int W = width_of(s.maxnb);
    if (!W) return fail(c, FEM_GPU_UNSUPPORTED, "more than 27 bases per cell");
    const int sides = s.kind == 2 ? 2 : 1;
    const Rule r = gauss_rule(s.kind == 2 ? s.dside.integration_rule : s.bulk.integration_rule);
    s.ngp = r.n;
    // repack to the kernel width W (the host arrays are already in that layout
    // when the set's basis width is W)
    const bool same = W == s.maxnb;
    std::vector<int32_t> bases(same ? 0 : (size_t)s.neq * sides * W, -1);
    std::vector<double> T(same ? 0 : (size_t)s.neq * sides * 8 * W, 0.0);
    const int W2 = sides * W, M2 = sides * s.maxnb;
    std::vector<uint16_t> sidx(same ? 0 : (size_t)s.neq * W2 * W2, 0);
    for (int64_t i = 0; i < (same ? 0 : s.neq); ++i) {
        for (int sd = 0; sd < sides; ++sd) {
            for (int j = 0; j < s.maxnb; ++j) bases[(i * sides + sd) * W + j] = s.bases[(i * sides + sd) * s.maxnb + j];
            for (int a = 0; a < 8; ++a)
                for (int j = 0; j < s.maxnb; ++j)
                    T[((i * sides + sd) * 8 + a) * W + j] = s.T[((i * sides + sd) * 8 + a) * s.maxnb + j];
        }
        for (int ii = 0; ii < M2; ++ii)
            for (int jj = 0; jj < M2; ++jj) {
                const int si2 = (ii / s.maxnb) * W + ii % s.maxnb, sj2 = (jj / s.maxnb) * W + jj % s.maxnb;
                sidx[(i * W2 + si2) * W2 + sj2] = s.sidx[(i * M2 + ii) * M2 + jj];
            }
    }
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = upload(s.d_gp, r.pts, st);
    if (e == cudaSuccess) e = upload(s.d_gw, r.w, st);
    if (e == cudaSuccess) e = upload(s.d_nb, s.nb, st);
    if (e == cudaSuccess) e = upload(s.d_bases, same ? s.bases : bases, st);
    if (e == cudaSuccess) e = upload(s.d_T, same ? s.T : T, st);
    if (e == cudaSuccess) e = upload(s.d_sidx, same ? s.sidx : sidx, st);
    if (e == cudaSuccess) e = upload(s.d_xe, s.xe, st);
    if (e == cudaSuccess) e = upload(s.d_E, s.E, st);
    if (s.kind == 0) {
        if (e == cudaSuccess) e = upload(s.d_igoff, s.ig_off, st);
        if (e == cudaSuccess) e = upload(s.d_igx, s.ig_coords, st);
        if (e == cudaSuccess) e = upload(s.d_igxi, s.ig_param, st);
    } else {
        if (e == cudaSuccess) e = upload(s.d_EF, s.EF, st);
        if (e == cudaSuccess) e = upload(s.d_fcoff, s.fc_off, st);
        if (e == cudaSuccess) e = upload(s.d_fcx, s.fc_x, st);
        if (e == cudaSuccess) e = upload(s.d_fcxl, s.fc_xl, st);
        if (e == cudaSuccess) e = upload(s.d_fcxf, s.fc_xf, st);
        if (e == cudaSuccess) e = upload(s.d_vol, s.vol, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cfail(c, e, "cluster set upload");
    if (!same) s.bases.swap(bases);
    s.maxnb = W;
    s.nbsel = W;
    s.T.clear();
    s.T.shrink_to_fit();
    s.sidx.clear();
    s.sidx.shrink_to_fit();
    return FEM_GPU_OK;
}

void cluster_release(fem_gpu_ctx* c) {
    for (auto& s : c->sets) {
        dfree(s.d_igoff);
        dfree(s.d_igx);
        dfree(s.d_igxi);
        dfree(s.d_fcoff);
        dfree(s.d_fcx);
        dfree(s.d_fcxl);
        dfree(s.d_fcxf);
        dfree(s.d_EF);
        dfree(s.d_vol);
    }
    if (c->batch) {
        Batch* b = (Batch*)c->batch;
        drop_graph(b);
        dfree(b->sets);
        dfree(b->items);
        dfree(b->counter);
        if (b->cap) cudaStreamDestroy(b->cap);
        delete b;
        c->batch = nullptr;
    }
}

// one set through the cluster kernel (fem_gpu_assemble / fem_gpu_element_matrices)
fem_gpu_status cluster_launch_set(fem_gpu_ctx* c, int set, int mode, int64_t first, int64_t count, const double* u,
                                  double* vals, double* rhs, double* Kout, double* Rout, int nmax) {
    if (count <= 0) return FEM_GPU_OK;
    const SetData& s = c->sets[set];
    cudaStream_t st = (cudaStream_t)c->stream;
    SetDev d;
    if (!set_dev(c, s, d)) return fail(c, FEM_GPU_UNSUPPORTED, "set not supported by the cluster kernel");
    std::vector<Item> items;
    std::vector<double> cost;
    add_items(s, 0, first, count, mode == 1 ? 0 : 64, items, cost);
    Kernel k;
    if (!pick_kernel(s.nbsel, 4, k)) return fail(c, FEM_GPU_UNSUPPORTED, "no cluster kernel instance");
    void* dsets = nullptr;
    void* ditems = nullptr;
    void* dctr = nullptr;
    cudaError_t e = cudaMallocAsync(&dsets, sizeof(SetDev), st);
    if (e == cudaSuccess) e = cudaMallocAsync(&ditems, std::max<size_t>(items.size(), 1) * sizeof(Item), st);
    if (e == cudaSuccess) e = cudaMallocAsync(&dctr, 2 * sizeof(unsigned long long), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dsets, &d, sizeof(SetDev), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !items.empty())
        e = cudaMemcpyAsync(ditems, items.data(), items.size() * sizeof(Item), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(dctr, 0, 2 * sizeof(unsigned long long), st);
    fem_gpu_status r = FEM_GPU_OK;
    if (e != cudaSuccess) r = cfail(c, e, "cluster staging");
    if (r == FEM_GPU_OK) {
        ClusterArgs a = base_args(c);
        a.sets = (const SetDev*)dsets;
        a.items = (const Item*)ditems;
        a.nitems = (int64_t)items.size();
        a.counter = (unsigned long long*)dctr;
        a.u = u;
        a.vals = vals;
        a.rhs = rhs;
        a.Kout = Kout;
        a.Rout = Rout;
        a.nmax = nmax;
        a.mode = mode == 1 ? CM_ELEMENT : CM_ASSEMBLE;
        a.first = first;
        r = launch(c, k, a, st);
    }
    // the items were copied from pageable host memory: finish before they go
    cudaStreamSynchronize(st);
    if (dsets) cudaFreeAsync(dsets, st);
    if (ditems) cudaFreeAsync(ditems, st);
    if (dctr) cudaFreeAsync(dctr, st);
    return r;
}

fem_gpu_status side_launch_on(fem_gpu_ctx* c, int set, const double* u, double* vals, double* rhs, cudaStream_t st);

}  // namespace fem

using namespace fem;

extern "C" {

fem_gpu_status fem_gpu_set_batched_config(fem_gpu_ctx* c, int32_t warps, int32_t split) {
    if (!c || (warps != 2 && warps != 4 && warps != 8) || split < 0) return FEM_GPU_BAD_ARG;
    Batch* b = batch_of(c);
    if (b->warps != warps || b->split != split) {
        b->warps = warps;
        b->split = split;
        b->built = false;
        drop_graph(b);
    }
    return FEM_GPU_OK;
}

fem_gpu_status fem_gpu_assemble_batched(fem_gpu_ctx* c, const double* u, double* vals, double* rhs, uint32_t flags) {
    if (!c) return FEM_GPU_BAD_ARG;
    if (!c->dev_final) return FEM_GPU_NOT_FINALIZED;
    if (flags & FEM_GPU_HOST_BUFFERS) return fail(c, FEM_GPU_BAD_ARG, "batched assembly takes device buffers");
    double* v = (flags & FEM_GPU_NO_JACOBIAN) ? nullptr : vals;
    double* r = (flags & FEM_GPU_NO_RESIDUAL) ? nullptr : rhs;
    if (!v && !r) return FEM_GPU_BAD_ARG;
    Batch* b = batch_of(c);
    fem_gpu_status st;
    if (!b->built && (st = build_batch(c, b)) != FEM_GPU_OK) return st;
    const bool zero = !(flags & FEM_GPU_ACCUMULATE);
    if (b->exec && (b->gu != u || b->gv != v || b->gr != r)) drop_graph(b);
    if (!b->exec) {
        if (!b->cap) {
            cudaError_t e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
            if (e != cudaSuccess) return cfail(c, e, "capture stream");
        }
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cfail(c, e, "begin capture");
        const int64_t before = c->launches;
        st = enqueue_batch(c, b, u, v, r, b->cap, zero, side_launch_on);
        e = cudaStreamEndCapture(b->cap, &g);
        c->launches = before;
        if (st != FEM_GPU_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return cfail(c, e, "end capture");
        e = cudaGraphInstantiate(&b->exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            b->exec = nullptr;
            return cfail(c, e, "graph instantiate");
        }
        b->gu = u;
        b->gv = v;
        b->gr = r;
    }
    cudaError_t e = cudaGraphLaunch(b->exec, (cudaStream_t)c->stream);
    if (e != cudaSuccess) return cfail(c, e, "graph launch");
    c->launches += 1 + b->nside;
    if (flags & FEM_GPU_ASYNC) return FEM_GPU_OK;
    return fem_gpu_check_status(c);
}

fem_gpu_status fem_gpu_autotune_batched(fem_gpu_ctx* c, int32_t* warps, int32_t* split, double* ms) {
    if (!c) return FEM_GPU_BAD_ARG;
    if (!c->dev_final) return FEM_GPU_NOT_FINALIZED;
    Batch* b = batch_of(c);
    cudaStream_t st = (cudaStream_t)c->stream;
    const int64_t nad = c->num_used * c->dim;
    double *vals = nullptr, *rhs = nullptr;
    cudaError_t e = cudaMallocAsync(&vals, std::max<int64_t>(c->nnz, 1) * sizeof(double), st);
    if (e == cudaSuccess) e = cudaMallocAsync(&rhs, nad * sizeof(double), st);
    if (e != cudaSuccess) return cfail(c, e, "autotune scratch");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int wl[3] = {2, 4, 8}, sl[4] = {32, 64, 128, 0};
    double best = 1e30;
    int bw = b->warps, bs = b->split;
    fem_gpu_status r = FEM_GPU_OK;
    for (int wi = 0; wi < 3 && r == FEM_GPU_OK; ++wi)
        for (int sj = 0; sj < 4 && r == FEM_GPU_OK; ++sj) {
            b->warps = wl[wi];
            b->split = sl[sj];
            if ((r = build_batch(c, b)) != FEM_GPU_OK) break;
            r = enqueue_batch(c, b, nullptr, vals, rhs, st, true, side_launch_on);
            if (r == FEM_GPU_UNSUPPORTED) {
                r = FEM_GPU_OK;
                cudaGetLastError();
                continue;
            }
            cudaEventRecord(e0, st);
            const int reps = 3;
            for (int k = 0; k < reps && r == FEM_GPU_OK; ++k)
                r = enqueue_batch(c, b, nullptr, vals, rhs, st, true, side_launch_on);
            cudaEventRecord(e1, st);
            e = cudaEventSynchronize(e1);
            if (e != cudaSuccess) {
                r = cfail(c, e, "autotune run");
                break;
            }
            float t = 0.f;
            cudaEventElapsedTime(&t, e0, e1);
            if (t / reps < best) {
                best = t / reps;
                bw = wl[wi];
                bs = sl[sj];
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(vals, st);
    cudaFreeAsync(rhs, st);
    cudaStreamSynchronize(st);
    b->warps = bw;
    b->split = bs;
    b->built = false;
    drop_graph(b);
    if (r == FEM_GPU_OK) r = build_batch(c, b);
    if (warps) *warps = bw;
    if (split) *split = bs;
    if (ms) *ms = best;
    return r;
}

}  // extern "C"
