// fem_device.cu -- device memory, the element kernels and the C ABI entry
// points that launch them.
//
// Bulk elasticity (IWG_Isotropic_Struc_Linear_Bulk + CM_Struc_Linear_
// Isotropic, FEM/INT/src/IWG/cl_FEM_IWG_Isotropic_Struc_Linear_Bulk.cpp:42-207)
// is evaluated one element per warp.  GB300 issues FP64 at a small fraction of
// its FP32 rate, so the kernel is built to minimise FP64 instructions rather
// than to mirror the reference's dense products:
//
//   per Gauss point   g = J^-1 dN/dxi, w* = w detJ          (lane per GP)
//   Gram matrix       A[(i,a),(j,b)] = sum_q w*_q g_ia g_jb  (upper triangle)
//   isotropic K       K[(f,a),(g,b)] = lam A[(f,a),(g,b)] + mu A[(g,a),(f,b)]
//                                      + mu delta_fg sum_k A[(k,a),(k,b)]
//   extraction        KT = K T, K_a = T^T KT over the column-sparse T
//   scatter           red.global.add.f64 into CSR at
//                     rowptr[f*nu+b_i] + g*|U(b_i)| + sidx[i][j]
//
// which equals w B^T D B summed over Gauss points (the reference's
// CM_Struc_Linear::testStrain/dFluxdDOF products, cl_FEM_CM_Struc_Linear.cpp:
// 503-826) and the reference's T^T K T (FEM/MSI/src/cl_MSI_Equation_Object.
// cpp:806-841) up to rounding.  The residual of the linear IWG is R = K u.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "fem_bits.cuh"
#include "fem_internal.hpp"
#include "fem_shape.hpp"

namespace fem {

// ---------------------------------------------------------------------------
// device buffers
namespace {

fem_gpu_status cuda_fail(fem_gpu_ctx* c, cudaError_t e, const char* what) {
    return fail(c, e == cudaErrorMemoryAllocation ? FEM_GPU_OUT_OF_MEMORY : FEM_GPU_CUDA_ERROR,
                std::string(what) + ": " + cudaGetErrorString(e));
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

cudaStream_t stream_of(const fem_gpu_ctx* c) { return (cudaStream_t)c->stream; }

}  // namespace

// ---------------------------------------------------------------------------
// bulk kernel
constexpr int kMaxGP = 32;

struct BulkArgs {
    int64_t ne;
    int64_t first;        // first equation object (element-matrix mode)
    const double* xe;     // [ne][NPE][D]
    const double* E;      // [ne]
    const int32_t* nb;    // [ne]
    const int32_t* bases; // [ne][NB]
    const double* T;      // [ne][NPE][NB]
    const uint16_t* sidx; // [ne][NB][NB]
    const int32_t* rowptr;
    const int32_t* ulen;
    const double* dn;     // [NGP][D][NPE]
    const double* w;      // [NGP]
    const uint32_t* pairs;// upper-triangle (r << 16 | c) pairs of the pdof Gram matrix
    const uint32_t* ktab; // K T items of bulk_cta_kernel (fem_bulk_cta.cuh)
    const uint16_t* tri;  // T^T K T upper-triangle items of bulk_cta_kernel
    const double* g0;     // [NPD][NPD] reference Gram table sum_q w_q dN dN (rectangular cells)
    const double* rho;    // [ne][NPE] nodal densities (nullable: constant E per element)
    const double* nq;     // [NGP][NPE] N of the IP cell at the Gauss points
    double beta;          // density exponent
    int npe;              // nodes per IP cell
    int64_t nu;
    double lam_c, mu_c;   // lambda / E and mu / E
    const double* u;      // adof vector (nullable)
    double* vals;         // CSR values (nullable)
    double* rhs;          // residual (nullable)
    double* Kout;         // element matrices [count][nmax][nmax] col-major (nullable)
    double* Rout;         // element residuals [count][nmax]
    int nmax;
    int kw;               // basis stride of Kout / Rout rows (the set's padding width, <= NB)
    const double* x;      // apply mode input (adof)
    double* y;            // apply mode output (adof)
    int* status;          // device error flags
    unsigned long long* queue;  // element counter of the CTA kernels (zeroed per launch)
};

template <int D, int NPE, int NGP, int NB>
struct BulkLayout {
    static constexpr int NPD = D * NPE;
    static constexpr int NAD = D * NB;
    static constexpr int NSYM = NPD * (NPD + 1) / 2;
    static constexpr int R1 = (2 * NGP * NPD > NPD * NAD) ? 2 * NGP * NPD : NPD * NAD;
    // doubles
    static constexpr int oX = 0;
    static constexpr int oR1 = oX + NPE * D;
    static constexpr int oA = oR1 + R1;
    static constexpr int oK = oA + NPD * NPD;
    static constexpr int oT = oK + NPD * NPD;
    static constexpr int oTW = oT + NPE * NB;
    static constexpr int oU = oTW + NB * NPE;
    static constexpr int oUA = oU + NPD;
    static constexpr int oRP = oUA + NAD;
    static constexpr int oW = oRP + NPD;
    static constexpr int ND = oW + NGP;
    // 4-byte ints
    static constexpr int iB = 0;             // bases [NB]
    static constexpr int iRB = iB + NB;      // rowptr of row (f,i) [NAD]
    static constexpr int iUL = iRB + NAD;    // |U(b_i)| [NB]
    static constexpr int NI = iUL + NB;
    // bytes
    static constexpr int bTN = 0;            // column-sparse T node ids [NB][NPE] (u8)
    static constexpr int bTC = bTN + NB * NPE;  // counts [NB]
    static constexpr int bS = ((bTC + NB + 1) / 2) * 2;  // sidx [NB][NB] (u16)
    static constexpr int NBYTE = bS + 2 * NB * NB;
    // per-warp region, a 16-byte multiple so every warp's doubles stay aligned
    static constexpr size_t kWarpBytes = ((size_t)ND * 8 + (size_t)NI * 4 + (size_t)NBYTE + 15) / 16 * 16;
    // per CTA: dn table, weights, sym pair table (16-byte multiple)
    static constexpr size_t kCtaBytes = (((size_t)(NGP * D * NPE + NGP) * 8 + (size_t)NSYM * 2 * 2) + 15) / 16 * 16;
};

static_assert(BulkLayout<3, 8, 27, 27>::kWarpBytes % 16 == 0, "warp region alignment");
static_assert(BulkLayout<2, 4, 4, 9>::kWarpBytes % 16 == 0, "warp region alignment");

enum { MODE_ASSEMBLE = 0, MODE_ELEMENT = 1, MODE_APPLY = 2 };

template <int D, int NPE, int NGP, int NB, bool RECT>
__global__ void __launch_bounds__(256) bulk_kernel(BulkArgs p, int mode, int warps_per_cta) {
    using L = BulkLayout<D, NPE, NGP, NB>;
    constexpr int NPD = L::NPD, NAD = L::NAD, NSYM = L::NSYM;
    extern __shared__ __align__(16) unsigned char smem[];
    double* cdn = reinterpret_cast<double*>(smem);
    double* cw = cdn + NGP * D * NPE;
    uint16_t* pairs = reinterpret_cast<uint16_t*>(cw + NGP);
    // CTA tables
    for (int i = threadIdx.x; i < NGP * D * NPE; i += blockDim.x) cdn[i] = p.dn[i];
    for (int i = threadIdx.x; i < NGP; i += blockDim.x) cw[i] = p.w[i];
    for (int k = threadIdx.x; k < NSYM; k += blockDim.x) {
        // k-th pair of the upper triangle, row-major: (r, c) with r <= c
        int r = 0, rem = k;
        while (rem >= NPD - r) {
            rem -= NPD - r;
            ++r;
        }
        pairs[2 * k] = (uint16_t)r;
        pairs[2 * k + 1] = (uint16_t)(r + rem);
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* wbase = smem + L::kCtaBytes + (size_t)warp * L::kWarpBytes;
    double* sd = reinterpret_cast<double*>(wbase);
    int32_t* si = reinterpret_cast<int32_t*>(sd + L::ND);
    unsigned char* sb = reinterpret_cast<unsigned char*>(si + L::NI);
    double* X = sd + L::oX;
    double* R1 = sd + L::oR1;
    double* g = R1;                  // [NGP][NPD]
    double* wg = R1 + NGP * NPD;     // [NGP][NPD]
    double* KT = R1;                 // [NPD][NAD] (after A is formed)
    double* A = sd + L::oA;
    double* K = sd + L::oK;
    double* T = sd + L::oT;
    double* TW = sd + L::oTW;        // [NB][NPE]
    double* U = sd + L::oU;          // pdof values [NPD]
    double* UA = sd + L::oUA;        // adof values [NAD]
    double* RP = sd + L::oRP;        // pdof residual [NPD]
    double* WS = sd + L::oW;         // w* per GP
    int32_t* B = si + L::iB;
    int32_t* RB = si + L::iRB;
    int32_t* UL = si + L::iUL;
    uint8_t* TN = sb + L::bTN;
    uint8_t* TC = sb + L::bTC;
    uint16_t* S = reinterpret_cast<uint16_t*>(sb + L::bS);

    const int64_t stride = (int64_t)gridDim.x * warps_per_cta;
    for (int64_t e = (int64_t)blockIdx.x * warps_per_cta + warp; e < p.ne; e += stride) {
        const int nb = p.nb[e];
        const double E = p.E[e];
        // ---- loads -------------------------------------------------------
        for (int i = lane; i < NPE * D; i += 32) X[i] = p.xe[e * (NPE * D) + i];
        for (int i = lane; i < NPE * NB; i += 32) T[i] = p.T[e * (NPE * NB) + i];
        for (int i = lane; i < NB; i += 32) B[i] = p.bases[e * NB + i];
        if (mode == MODE_ASSEMBLE && p.vals)
            for (int i = lane; i < NB * NB; i += 32) S[i] = p.sidx[e * (NB * NB) + i];
        __syncwarp();
        if (mode == MODE_ASSEMBLE) {
            for (int r = lane; r < NAD; r += 32) {
                const int f = r / NB, i = r - f * NB;
                RB[r] = i < nb ? p.rowptr[f * p.nu + B[i]] : 0;
            }
            for (int i = lane; i < NB; i += 32) UL[i] = i < nb ? p.ulen[B[i]] : 0;
        }
        const double* uin = mode == MODE_APPLY ? p.x : p.u;
        for (int r = lane; r < NAD; r += 32) {
            const int f = r / NB, i = r - f * NB;
            UA[r] = (uin && i < nb) ? uin[f * p.nu + B[i]] : 0.0;
        }
        // column-sparse extraction lists
        for (int j = lane; j < NB; j += 32) {
            int cnt = 0;
            for (int a = 0; a < NPE; ++a) {
                const double t = T[a * NB + j];
                if (fem_nonzero(t)) {
                    TN[j * NPE + cnt] = (uint8_t)a;
                    TW[j * NPE + cnt] = t;
                    ++cnt;
                }
            }
            TC[j] = (uint8_t)cnt;
        }
        // ---- Gauss-point geometry: g = J^-1 dN/dxi, w* = w detJ ----------
        for (int q = lane; q < NGP; q += 32) {
            const double* dn = cdn + q * D * NPE;
            double detJ;
            double Ji[D][D];
            if (RECT) {
                double jd[D];
                for (int i = 0; i < D; ++i) {
                    double s = 0.0;
                    for (int a = 0; a < NPE; ++a) s = fma(dn[i * NPE + a], X[a * D + i], s);
                    jd[i] = s;
                }
                detJ = (D == 3) ? jd[1] * jd[0] * jd[2] : jd[0] * jd[1];
                for (int i = 0; i < D; ++i)
                    for (int j = 0; j < D; ++j) Ji[i][j] = (i == j) ? 1.0 / jd[i] : 0.0;
            } else {
                double J[D][D];
                for (int i = 0; i < D; ++i)
                    for (int j = 0; j < D; ++j) {
                        double s = 0.0;
                        for (int a = 0; a < NPE; ++a) s = fma(dn[i * NPE + a], X[a * D + j], s);
                        J[i][j] = s;
                    }
                if (D == 2) {
                    detJ = J[0][0] * J[1][1] - J[0][1] * J[1][0];
                    const double id = 1.0 / detJ;
                    Ji[0][0] = J[1][1] * id;
                    Ji[0][1] = -J[0][1] * id;
                    Ji[1][0] = -J[1][0] * id;
                    Ji[1][1] = J[0][0] * id;
                } else {
                    detJ = +J[0][0] * (J[1][1] * J[2][2] - J[2][1] * J[1][2]) -
                           J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
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
            }
            // integration points with detJ below -1e-6 are skipped by the
            // reference element loop (cl_FEM_Element_Bulk.cpp:164)
            const double ws = (detJ < -1.0e-6) ? 0.0 : cw[q] * detJ;
            WS[q] = ws;
            for (int i = 0; i < D; ++i)
                for (int a = 0; a < NPE; ++a) {
                    double s;
                    if (RECT) {
                        s = Ji[i][i] * dn[i * NPE + a];
                    } else {
                        s = 0.0;
                        for (int k = 0; k < D; ++k) s = fma(Ji[i][k], dn[k * NPE + a], s);
                    }
                    g[q * NPD + i * NPE + a] = s;
                    wg[q * NPD + i * NPE + a] = ws * s;
                }
        }
        __syncwarp();
        // pdof values u = T u_a (compute_my_pdof_values)
        for (int r = lane; r < NPD; r += 32) {
            const int f = r / NPE, a = r - f * NPE;
            double s = 0.0;
            for (int j = 0; j < nb; ++j) {
                const double t = T[a * NB + j];
                if (fem_nonzero(t)) s = fma(t, UA[f * NB + j], s);
            }
            U[r] = s;
        }
        if (mode == MODE_APPLY) {
            // matrix-free: per GP stress sigma = lam tr(grad u) I + mu (grad u + grad u^T),
            // stored as w* sigma in A ([q][f][i]); then f_(f,a) = sum_q sum_i g_ia (w sigma)_fi
            __syncwarp();
            for (int q = lane; q < NGP; q += 32) {
                double G[D][D];
                for (int f = 0; f < D; ++f)
                    for (int i = 0; i < D; ++i) {
                        double s = 0.0;
                        for (int a = 0; a < NPE; ++a) s = fma(g[q * NPD + i * NPE + a], U[f * NPE + a], s);
                        G[f][i] = s;  // du_f / dx_i
                    }
                double tr = 0.0;
                for (int k = 0; k < D; ++k) tr += G[k][k];
                const double lam = E * p.lam_c, mu = E * p.mu_c, ws = WS[q];
                for (int f = 0; f < D; ++f)
                    for (int i = 0; i < D; ++i)
                        A[q * D * D + f * D + i] = ws * ((f == i ? lam * tr : 0.0) + mu * (G[f][i] + G[i][f]));
            }
            __syncwarp();
            for (int r = lane; r < NPD; r += 32) {
                const int f = r / NPE, a = r - f * NPE;
                double s = 0.0;
                for (int q = 0; q < NGP; ++q)
                    for (int i = 0; i < D; ++i) s = fma(g[q * NPD + i * NPE + a], A[q * D * D + f * D + i], s);
                RP[r] = s;
            }
            __syncwarp();
            for (int r = lane; r < NAD; r += 32) {
                const int f = r / NB, i = r - f * NB;
                if (i >= nb) continue;
                double s = 0.0;
                for (int k = 0; k < TC[i]; ++k) s = fma(TW[i * NPE + k], RP[f * NPE + TN[i * NPE + k]], s);
                atomicAdd(p.y + f * p.nu + B[i], s);
            }
            __syncwarp();
            continue;
        }
        // ---- Gram matrix (upper triangle) --------------------------------
        for (int k = lane; k < NSYM; k += 32) {
            const int r = pairs[2 * k], c = pairs[2 * k + 1];
            double s = 0.0;
#pragma unroll 9
            for (int q = 0; q < NGP; ++q) s = fma(wg[q * NPD + r], g[q * NPD + c], s);
            A[r * NPD + c] = s;
            A[c * NPD + r] = s;
        }
        __syncwarp();
        // ---- isotropic element stiffness (pdof space) ----------------------
        {
            const double lam = E * p.lam_c, mu = E * p.mu_c;
            for (int k = lane; k < NSYM; k += 32) {
                const int r = pairs[2 * k], c = pairs[2 * k + 1];
                const int f = r / NPE, a = r - f * NPE, gg = c / NPE, b = c - gg * NPE;
                double v = lam * A[r * NPD + c] + mu * A[(gg * NPE + a) * NPD + f * NPE + b];
                if (f == gg) {
                    double tr = 0.0;
                    for (int kk = 0; kk < D; ++kk) tr += A[(kk * NPE + a) * NPD + kk * NPE + b];
                    v = fma(mu, tr, v);
                }
                K[r * NPD + c] = v;
                K[c * NPD + r] = v;
            }
        }
        __syncwarp();
        // ---- residual R_a = T^T (K u) --------------------------------------
        const bool want_r = (mode == MODE_ASSEMBLE && p.rhs) || (mode == MODE_ELEMENT && p.Rout);
        if (want_r) {
            for (int r = lane; r < NPD; r += 32) {
                double s = 0.0;
                for (int c = 0; c < NPD; ++c) s = fma(K[r * NPD + c], U[c], s);
                RP[r] = s;
            }
            __syncwarp();
            for (int r = lane; r < NAD; r += 32) {
                const int f = r / NB, i = r - f * NB;
                double s = 0.0;
                if (i < nb)
                    for (int k = 0; k < TC[i]; ++k) s = fma(TW[i * NPE + k], RP[f * NPE + TN[i * NPE + k]], s);
                if (mode == MODE_ASSEMBLE) {
                    if (i < nb) atomicAdd(p.rhs + f * p.nu + B[i], s);
                } else if (i < p.kw) {
                    p.Rout[(e - p.first) * p.nmax + f * p.kw + i] = s;
                }
            }
        }
        const bool want_k = (mode == MODE_ASSEMBLE && p.vals) || (mode == MODE_ELEMENT && p.Kout);
        if (!want_k) {
            __syncwarp();
            continue;
        }
        // ---- KT = K T (column-sparse T) ------------------------------------
        {
            constexpr int CPP = NPD >= 32 ? 1 : 32 / NPD;  // columns per pass
            const int row = lane % NPD, sub = lane / NPD;
            if (row < NPD && sub < CPP && lane < CPP * NPD) {
                for (int c0 = 0; c0 < NAD; c0 += CPP) {
                    const int c = c0 + sub;
                    if (c >= NAD) break;
                    const int gg = c / NB, j = c - gg * NB;
                    double s = 0.0;
                    const int cnt = j < nb ? TC[j] : 0;
                    for (int k = 0; k < cnt; ++k)
                        s = fma(K[row * NPD + gg * NPE + TN[j * NPE + k]], TW[j * NPE + k], s);
                    KT[row * NAD + c] = s;
                }
            }
        }
        __syncwarp();
        // ---- K_a = T^T KT (upper triangle) and scatter ----------------------
        bool bad = false;
        for (int r = 0; r < NAD; ++r) {
            const int f = r / NB, i = r - f * NB;
            if (i >= nb) continue;
            const int cnt = TC[i];
            for (int c = r + lane; c < NAD; c += 32) {
                const int gg = c / NB, j = c - gg * NB;
                if (j >= nb) continue;
                double v = 0.0;
                for (int k = 0; k < cnt; ++k) v = fma(TW[i * NPE + k], KT[(f * NPE + TN[i * NPE + k]) * NAD + c], v);
                bad |= !fem_finite(v);
                if (mode == MODE_ASSEMBLE) {
                    atomicAdd(p.vals + RB[r] + gg * UL[i] + S[i * NB + j], v);
                    if (c != r) atomicAdd(p.vals + RB[c] + f * UL[j] + S[j * NB + i], v);
                } else {
                    double* Ko = p.Kout + (e - p.first) * (int64_t)p.nmax * p.nmax;
                    const int ro = f * p.kw + i, co = gg * p.kw + j;
                    Ko[ro + (int64_t)co * p.nmax] = v;
                    Ko[co + (int64_t)ro * p.nmax] = v;
                }
            }
        }
        if (bad) atomicOr(p.status, 1);
        __syncwarp();
    }
}

#include "fem_bulk_cta.cuh"

// ---------------------------------------------------------------------------
// side sets (Neumann traction, Nitsche Dirichlet) on interpolation-cell
// facets: Element_Sideset (FEM/INT/src/ELEM/cl_FEM_Element_Sideset.cpp:
// 261-330), IWG_Isotropic_Struc_Linear_Neumann (:38-80) and _Dirichlet
// (:52-240) with their Thickness (w* times thickness) and Select (a dim x dim
// projection M of the prescribed components) properties,
// SP_Dirichlet_Nitsche (gamma = alpha E / h).
//
// One CTA per facet (grid-stride over the facets).  Everything of a facet
// lives in shared memory: the IP-cell coordinates and extraction T (with the
// nonzeros of every T column as a list), the pdof values, per Gauss point N,
// dN/dx, w*, the traction operator nDB[f][(g,b)] = lam n_f g_gb + mu (n_g g_fb
// + delta_fg n.g_b) and its projections (w* and beta folded in), the facet
// Gram matrix sum_q w* N_a N_b, the pdof K and R, and K T.  Threads own Gauss
// points for the geometry, then pdof entries for K and R, then (entry, column)
// pairs of K T and T^T (K T), which contract over the nonzeros of one T column
// only, and whose results are scattered into the CSR.  FP64 is the bound on
// this GPU, so the stages that add nothing are skipped: a Neumann set (or a
// zero Select matrix) has K = 0, and pdof pairs of two nodes off the facet
// (N_a = N_b = 0 at every point) have K = 0.
// per (facet ordinal, Gauss point): the facet's own shape derivatives
// [(D-1) x NFV], the cell's N [NPE] and dN/dxi [D x NPE] at the point
__host__ __device__ constexpr int side_ref_len(int D) {
    return D == 2 ? 1 * 2 + 4 + 2 * 4 : 2 * 4 + 8 + 3 * 8;
}
// facet vertices of each ordinal (QUAD4 edges, HEX8 faces: the MTK node order)
__host__ __device__ inline int side_face_vertex(int D, int ord, int k) {
    const int quad_f[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};
    const int hex_f[6][4] = {{1, 5, 4, 0}, {1, 2, 6, 5}, {3, 7, 6, 2}, {0, 4, 7, 3}, {0, 3, 2, 1}, {4, 5, 6, 7}};
    return D == 2 ? quad_f[ord][k] : hex_f[ord][k];
}

// per facet: for every Gauss point w* (w detJ times the thickness, 0 where
// detJ < -1e-6), w detJ, the unit normal (3) and the inverse cell Jacobian
// (3 x 3), then 1/h of SP_Dirichlet_Nitsche (h = the facet measure in 2-D,
// sqrt(4 A / pi) in 3-D)
constexpr int kSideGeoPerPoint = 14;
__host__ __device__ constexpr int side_geo_len(int ngp) { return ngp * kSideGeoPerPoint + 2; }

// The facet geometry depends on the mesh alone, so it is computed once when
// the set is uploaded, one thread per (facet, Gauss point) -- the per-point
// divisions and square roots would otherwise occupy the FP64 pipe on a few
// lanes of every assembly.
template <int D>
__global__ void side_geometry_kernel(int64_t ns, int ngp, const double* xe, const int32_t* ordv, const double* gw,
                                     const double* sref, int rect, double thickness, double* out) {
    constexpr int NPE = D == 2 ? 4 : 8, NFV = D == 2 ? 2 : 4, REF = side_ref_len(D);
    const int SG = side_geo_len(ngp);
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < ns * ngp; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = k / ngp;
        const int q = (int)(k - s * ngp), ord = ordv[s];
        const double* X = xe + s * NPE * D;
        const double* dNf = sref + (ord * ngp + q) * REF;
        const double* dN = dNf + (D - 1) * NFV + NPE;
        double t[2][3] = {{0, 0, 0}, {0, 0, 0}};
        for (int kk = 0; kk < NFV; ++kk) {
            const int v = side_face_vertex(D, ord, kk);
            for (int d = 0; d < D; ++d)
                for (int m = 0; m < D - 1; ++m) t[m][d] = fma(dNf[m * NFV + kk], X[v * D + d], t[m][d]);
        }
        double detJ, nrm[3] = {0, 0, 0};
        if (D == 2) {
            detJ = sqrt(t[0][0] * t[0][0] + t[0][1] * t[0][1]);
            nrm[0] = t[0][1] / detJ;
            nrm[1] = -t[0][0] / detJ;
        } else {
            const double c0 = t[0][1] * t[1][2] - t[0][2] * t[1][1];
            const double c1 = t[0][2] * t[1][0] - t[0][0] * t[1][2];
            const double c2 = t[0][0] * t[1][1] - t[0][1] * t[1][0];
            detJ = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
            nrm[0] = c0 / detJ;
            nrm[1] = c1 / detJ;
            nrm[2] = c2 / detJ;
        }
        double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, Ji[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int i = 0; i < D; ++i)
            for (int j = 0; j < D; ++j)
                if (!rect || i == j)
                    for (int a = 0; a < NPE; ++a) J[i * 3 + j] = fma(dN[i * NPE + a], X[a * D + j], J[i * 3 + j]);
        if (rect) {
            for (int i = 0; i < D; ++i) Ji[i * 3 + i] = 1.0 / J[i * 3 + i];
        } else if (D == 2) {
            const double det = J[0] * J[4] - J[1] * J[3], id = 1.0 / det;
            Ji[0] = J[4] * id; Ji[1] = -J[1] * id; Ji[3] = -J[3] * id; Ji[4] = J[0] * id;
        } else {
            const double det = J[0] * (J[4] * J[8] - J[7] * J[5]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                               J[2] * (J[3] * J[7] - J[4] * J[6]);
            const double id = 1.0 / det;
            Ji[0] = (J[4] * J[8] - J[7] * J[5]) * id;
            Ji[1] = (J[2] * J[7] - J[1] * J[8]) * id;
            Ji[2] = (J[1] * J[5] - J[2] * J[4]) * id;
            Ji[3] = (J[5] * J[6] - J[3] * J[8]) * id;
            Ji[4] = (J[0] * J[8] - J[2] * J[6]) * id;
            Ji[5] = (J[3] * J[2] - J[0] * J[5]) * id;
            Ji[6] = (J[3] * J[7] - J[6] * J[4]) * id;
            Ji[7] = (J[6] * J[1] - J[0] * J[7]) * id;
            Ji[8] = (J[0] * J[4] - J[3] * J[1]) * id;
        }
        double* o = out + s * SG + q * kSideGeoPerPoint;
        o[0] = detJ < -1.0e-6 ? 0.0 : gw[q] * detJ * thickness;
        o[1] = gw[q] * detJ;
        for (int d = 0; d < 3; ++d) o[2 + d] = nrm[d];
        for (int m = 0; m < 9; ++m) o[5 + m] = Ji[m];
    }
}

// 1/h per facet from the measures of its points
template <int D>
__global__ void side_h_kernel(int64_t ns, int ngp, double* out) {
    const int SG = side_geo_len(ngp);
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += (int64_t)gridDim.x * blockDim.x) {
        double meas = 0.0;
        for (int q = 0; q < ngp; ++q) meas += out[s * SG + q * kSideGeoPerPoint + 1];
        const double h = D == 2 ? meas : sqrt(4.0 * meas / 3.14159265358979323846);
        out[s * SG + ngp * kSideGeoPerPoint] = 1.0 / h;
        out[s * SG + ngp * kSideGeoPerPoint + 1] = 0.0;
    }
}

struct SideArgs {
    int64_t ns;
    int iwg, model, ngp, maxnb;
    const double* xe;
    const double* E;
    const int32_t* ord;
    const int32_t* nb;
    const int32_t* bases;
    const double* T;
    const uint16_t* sidx;
    const int32_t* rowptr;
    const int32_t* ulen;
    const double* gp;   // [ngp] facet Gauss points (dim-1 coords each)
    const double* gw;   // [ngp]
    const double* sref; // [ordinal][ngp][side_ref_len(D)]: facet dN, cell N, cell dN/dxi
    const double* sgeo; // [facet][side_geo_len(ngp)]: per point w*, measure, normal, J^-1; 1/h
    int rect;           // axis-aligned brick cells: diagonal, constant Jacobian
    int select_identity; // M = I (no Select property): the projections are copies
    int64_t nu;
    double nu_p, alpha;
    double value[3];
    double thickness;   // w* factor
    double select[9];   // M, row-major 3 x 3 (the leading dim x dim block is used)
    const double* u;
    double* vals;
    double* rhs;
    double* Kout;
    double* Rout;
    int nmax;
    int64_t first;
    int mode;
    int* status;
};

// shared-memory layout of one facet, in doubles (the basis ids follow as ints)
struct SideSmem {
    int X, T, TW, NG, U, R, K, KT, QN, QG, QW, QNRM, QB, QMB, QMTB, QT, QJ, QJI, QTU, QJU, misc, total;
    __host__ __device__ SideSmem(int D, int maxnb, int ngp) {
        const int NPE = D == 2 ? 4 : 8, NPD = D * NPE;
        int o = 0;
        X = o; o += NPE * D;
        T = o; o += NPE * maxnb;
        TW = o; o += NPE * maxnb;
        NG = o; o += NPE * NPE;
        U = o; o += NPD;
        R = o; o += NPD;
        K = o; o += NPD * NPD;
        KT = o; o += NPD * D * maxnb;
        QN = o; o += ngp * NPE;
        QG = o; o += ngp * D * NPE;
        QW = o; o += ngp;
        QNRM = o; o += ngp * 3;
        QB = o; o += ngp * D * NPD;
        QMB = o; o += ngp * D * NPD;
        QMTB = o; o += ngp * D * NPD;
        QT = o; o += ngp * D;
        QJ = o; o += ngp * D;
        QJI = o; o += ngp * 9;
        QTU = o; o += ngp * D;
        QJU = o; o += ngp * D;
        misc = o; o += 4;
        total = o;
    }
    // doubles, then the basis ids (int32), the T column lists (uint8 node
    // index per nonzero), their counts (uint8) and the cell nodes with those
    // on the facet first (uint8)
    static size_t bytes(int D, int maxnb, int ngp) {
        const int NPE = D == 2 ? 4 : 8;
        return SideSmem(D, maxnb, ngp).total * sizeof(double) + (size_t)maxnb * (sizeof(int32_t) + NPE + 1) + NPE;
    }
};

template <int D>
__global__ void __launch_bounds__(128, 8) side_cta_kernel(SideArgs p) {
    constexpr int NPE = D == 2 ? 4 : 8, NPD = D * NPE, NFV = D == 2 ? 2 : 4;
    extern __shared__ double sm[];
    const int maxnb = p.maxnb, ngp = p.ngp, tid = threadIdx.x, NT = blockDim.x;
    const SideSmem L(D, maxnb, ngp);
    double* X = sm + L.X;
    double* T = sm + L.T;
    double* TW = sm + L.TW;
    double* NG = sm + L.NG;
    double* U = sm + L.U;
    double* R = sm + L.R;
    double* K = sm + L.K;
    double* KT = sm + L.KT;
    double* QN = sm + L.QN;
    double* QG = sm + L.QG;
    double* QW = sm + L.QW;
    double* QNRM = sm + L.QNRM;
    double* QB = sm + L.QB;
    double* QMB = sm + L.QMB;
    double* QMTB = sm + L.QMTB;
    double* QT = sm + L.QT;
    double* QJ = sm + L.QJ;
    double* QJI = sm + L.QJI;
    double* QTU = sm + L.QTU;
    double* QJU = sm + L.QJU;
    double* misc = sm + L.misc;
    int32_t* bs = reinterpret_cast<int32_t*>(sm + L.total);
    uint8_t* TN = reinterpret_cast<uint8_t*>(bs + maxnb);  // [maxnb][NPE]
    uint8_t* TC = TN + maxnb * NPE;                          // [maxnb]
    uint8_t* FP = TC + maxnb;                                // [NPE]: facet nodes first
    const bool neumann = p.iwg == FEM_GPU_IWG_STRUC_LINEAR_NEUMANN;
    const double beta = p.iwg == FEM_GPU_IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE ? -1.0 : 1.0;
    const double mu_c = 1.0 / (2.0 * (1.0 + p.nu_p));
    const double lam_c = p.model == FEM_GPU_MODEL_PLANE_STRESS ? p.nu_p / (1.0 - p.nu_p * p.nu_p)
                                                               : p.nu_p / ((1.0 + p.nu_p) * (1.0 - 2.0 * p.nu_p));
    // a zero projection adds nothing (the reference skips the IWG)
    double mnorm = 0.0;
    for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) mnorm = fma(p.select[i * 3 + j], p.select[i * 3 + j], mnorm);
    const bool active = neumann || sqrt(mnorm) >= 2.220446049250313e-16;
    // K = 0 for a Neumann set and for a zero projection: the assembly skips the
    // K, K T and T^T K T stages (element outputs still write the zeros)
    const bool k_zero = neumann || !active;
    for (int64_t s = blockIdx.x; s < p.ns; s += gridDim.x) {
        const int nb = p.nb[s];
        const int ord = p.ord[s];
        const double E = p.E[s];
        const double lam = E * lam_c, mu = E * mu_c;
        // ---- stage the facet's cell ------------------------------------------------
        for (int i = tid; i < NPE * D; i += NT) X[i] = p.xe[s * NPE * D + i];
        for (int i = tid; i < NPE * maxnb; i += NT) T[i] = p.T[s * NPE * maxnb + i];
        for (int j = tid; j < maxnb; j += NT) bs[j] = p.bases[s * maxnb + j];
        __syncthreads();
        // the nonzeros of every T column, in node order (the products they skip
        // are exact zeros)
        for (int j = tid; j < maxnb; j += NT) {
            int cnt = 0;
            for (int a = 0; a < NPE; ++a) {
                const double t = T[a * maxnb + j];
                if (fem_nonzero(t)) {
                    TN[j * NPE + cnt] = (uint8_t)a;
                    TW[j * NPE + cnt] = t;
                    ++cnt;
                }
            }
            TC[j] = (uint8_t)cnt;
        }
        // ---- pdof values; per-point geometry -----------------------------------------
        for (int r = tid; r < NPD; r += NT) {
            const int f = r / NPE, a = r - f * NPE;
            double v = 0.0;
            if (p.u)
                for (int j = 0; j < nb; ++j) {
                    const double t = T[a * maxnb + j];
                    if (fem_nonzero(t)) v = fma(t, p.u[f * p.nu + bs[j]], v);
                }
            U[r] = v;
            R[r] = 0.0;
        }
        // per point: w*, the normal and J^-1 (computed once per mesh), N from
        // the reference table
        constexpr int REF = side_ref_len(D);
        const double* geo = p.sgeo + s * side_geo_len(ngp);
        for (int k = tid; k < ngp * kSideGeoPerPoint; k += NT) {
            const int q = k / kSideGeoPerPoint, m = k - q * kSideGeoPerPoint;
            const double v = geo[k];
            if (m == 0) QW[q] = v;
            else if (m >= 2 && m < 5) QNRM[q * 3 + m - 2] = v;
            else if (m >= 5) QJI[q * 9 + m - 5] = v;
        }
        for (int k = tid; k < ngp * NPE; k += NT) {
            const int q = k / NPE, a = k - q * NPE;
            QN[k] = p.sref[(ord * ngp + q) * REF + (D - 1) * NFV + a];
        }
        if (tid == 0) misc[0] = p.alpha * E * geo[ngp * kSideGeoPerPoint];
        __syncthreads();
        // dN/dx = J^-1 dN/dxi (lanes over point, component and node)
        for (int k = tid; k < ngp * D * NPE; k += NT) {
            const int q = k / (D * NPE), i = (k / NPE) % D, a = k % NPE;
            const double* dN = p.sref + (ord * ngp + q) * REF + (D - 1) * NFV + NPE;
            const double* Ji = QJI + q * 9;
            double v = 0.0;
            for (int kk = 0; kk < D; ++kk) v = fma(Ji[i * 3 + kk], dN[kk * NPE + a], v);
            QG[k] = v;
        }
        __syncthreads();
        // ---- traction operator per point -------------------------------------------
        if (!neumann)
            for (int k = tid; k < ngp * D * NPD; k += NT) {
                const int q = k / (D * NPD), rem = k - q * D * NPD, f = rem / NPD, c = rem - f * NPD;
                const int gg = c / NPE, b = c - gg * NPE;
                const double* nrm = QNRM + q * 3;
                const double* g = QG + q * D * NPE;
                double ng = 0.0;
                for (int kk = 0; kk < D; ++kk) ng += nrm[kk] * g[kk * NPE + b];
                const double qb = lam * nrm[f] * g[gg * NPE + b] + mu * (nrm[gg] * g[f * NPE + b] + (f == gg ? ng : 0.0));
                QB[k] = qb;
                if (p.select_identity) {
                    // M nDB = M^T nDB = nDB: the projections below, without the zero terms
                    QMB[k] = QW[q] * qb;
                    QMTB[k] = beta * QW[q] * qb;
                }
            }
        __syncthreads();
        // projections M nDB and M^T nDB
        if (!neumann && !p.select_identity)
            for (int k = tid; k < ngp * D * NPD; k += NT) {
                const int q = k / (D * NPD), rem = k - q * D * NPD, f = rem / NPD, c = rem - f * NPD;
                const double* B = QB + q * D * NPD;
                double mb = 0.0, mtb = 0.0;
                for (int kk = 0; kk < D; ++kk) {
                    mb = fma(p.select[f * 3 + kk], B[kk * NPD + c], mb);
                    mtb = fma(p.select[kk * 3 + f], B[kk * NPD + c], mtb);
                }
                // w* folded in, and beta into M^T nDB (both only feed K)
                QMB[k] = QW[q] * mb;
                QMTB[k] = beta * QW[q] * mtb;
            }
        // facet Gram matrix sum_q w* N_a N_b (the gamma term of K)
        if (!k_zero)
            for (int k = tid; k < NPE * NPE; k += NT) {
                const int a = k / NPE, b = k - a * NPE;
                double g = 0.0;
                for (int q = 0; q < ngp; ++q) g = fma(QW[q] * QN[q * NPE + a], QN[q * NPE + b], g);
                NG[k] = g;
            }
        // traction and jump per point and component, then projected: M t(u), M (u - g)
        if (!neumann)
            for (int k = tid; k < ngp * D; k += NT) {
                const int q = k / D, f = k - q * D;
                double tt = 0.0, uu = 0.0;
                for (int c = 0; c < NPD; ++c) tt = fma(QB[(q * D + f) * NPD + c], U[c], tt);
                for (int a = 0; a < NPE; ++a) uu = fma(QN[q * NPE + a], U[f * NPE + a], uu);
                QTU[k] = tt;
                QJU[k] = uu - p.value[f];
                if (p.select_identity) {
                    QT[k] = tt;
                    QJ[k] = uu - p.value[f];
                }
            }
        __syncthreads();
        // the cell nodes on the facet (N_a nonzero at some point: a nonzero
        // diagonal Gram entry) first, then the others
        if (!k_zero && tid == 0) {
            int nf = 0;
            for (int a = 0; a < NPE; ++a)
                if (fem_nonzero(NG[a * NPE + a])) FP[nf++] = (uint8_t)a;
            int o = nf;
            for (int a = 0; a < NPE; ++a)
                if (!fem_nonzero(NG[a * NPE + a])) FP[o++] = (uint8_t)a;
            misc[1] = nf;
        }
        if (!neumann && !p.select_identity)
            for (int k = tid; k < ngp * D; k += NT) {
                const int q = k / D, f = k - q * D;
                double mt = 0.0, mj = 0.0;
                for (int kk = 0; kk < D; ++kk) {
                    mt = fma(p.select[f * 3 + kk], QTU[q * D + kk], mt);
                    mj = fma(p.select[f * 3 + kk], QJU[q * D + kk], mj);
                }
                QT[k] = mt;
                QJ[k] = mj;
            }
        __syncthreads();
        // ---- pdof residual and Jacobian --------------------------------------------
        const double gamma = misc[0];
        for (int r = tid; r < NPD; r += NT) {
            const int f = r / NPE, a = r - f * NPE;
            double v = 0.0;
            for (int q = 0; q < ngp; ++q) {
                const double na = QN[q * NPE + a];
                double t;
                if (neumann) {
                    t = -na * p.value[f];
                } else {
                    t = na * (gamma * QJ[q * D + f] - QT[q * D + f]);
                    for (int kk = 0; kk < D; ++kk) t = fma(beta * QB[(q * D + kk) * NPD + r], QJ[q * D + kk], t);
                }
                v = fma(QW[q], t, v);
            }
            R[r] = active ? v : 0.0;
        }
        // K[(f,a),(g,b)] = sum_q w*[beta (M^T nDB)_(g,(f,a)) N_b - N_a (M nDB)_(f,(g,b))]
        //                 + gamma M_fg sum_q w* N_a N_b
        // (w* and beta are inside QMTB / QMB).  N_b = 0 at every point for a
        // node b off the facet, so its terms are exact zeros: the entries are
        // taken block by block -- both nodes on the facet (every term), row
        // node on (the N_a terms), column node on (the N_b terms), both off
        // (K = 0) -- which keeps the work of a warp uniform
        if (!k_zero) {
            const int nf = (int)misc[1], no = NPE - nf;
            const int non = D * nf, noff = D * no;
            // block (row class, column class): 0 on-on, 1 on-off, 2 off-on, 3 off-off
            for (int blk = 0; blk < 4; ++blk) {
                const bool ron = blk < 2, con = (blk & 1) == 0;
                const int nr = ron ? non : noff, nc_ = con ? non : noff, nrn = ron ? nf : no, ncn = con ? nf : no;
                for (int k = tid; k < nr * nc_; k += NT) {
                    const int ri = k / nc_, ci = k - ri * nc_;
                    const int f = ri / nrn, a = FP[(ron ? 0 : nf) + ri % nrn];
                    const int gg = ci / ncn, b = FP[(con ? 0 : nf) + ci % ncn];
                    const int r = f * NPE + a, c = gg * NPE + b;
                    double v = 0.0;
                    if (ron && con) {
                        for (int q = 0; q < ngp; ++q) {
                            v = fma(QMTB[(q * D + gg) * NPD + r], QN[q * NPE + b], v);
                            v = fma(-QN[q * NPE + a], QMB[(q * D + f) * NPD + c], v);
                        }
                        v = fma(gamma * p.select[f * 3 + gg], NG[a * NPE + b], v);
                    } else if (con) {
                        for (int q = 0; q < ngp; ++q) v = fma(QMTB[(q * D + gg) * NPD + r], QN[q * NPE + b], v);
                    } else if (ron) {
                        for (int q = 0; q < ngp; ++q) v = fma(-QN[q * NPE + a], QMB[(q * D + f) * NPD + c], v);
                    }
                    K[r * NPD + c] = v;
                }
            }
        }
        else if (p.mode != MODE_ASSEMBLE)
            for (int k = tid; k < NPD * NPD; k += NT) K[k] = 0.0;
        __syncthreads();
        // ---- extraction: R_a = T^T R, K T, then T^T (K T) and the scatter -----------
        for (int k = tid; k < D * nb; k += NT) {
            const int f = k / nb, i = k - f * nb;
            double ra = 0.0;
            for (int m = 0; m < TC[i]; ++m) ra = fma(TW[i * NPE + m], R[f * NPE + TN[i * NPE + m]], ra);
            if (p.mode == MODE_ASSEMBLE) {
                if (p.rhs) atomicAdd(p.rhs + f * p.nu + bs[i], ra);
            } else if (p.Rout) {
                p.Rout[(s - p.first) * p.nmax + f * maxnb + i] = ra;
            }
        }
        const bool want_k = !((p.mode == MODE_ASSEMBLE && (!p.vals || k_zero)) || (p.mode == MODE_ELEMENT && !p.Kout));
        const int nc = D * nb;
        if (want_k)
            for (int k = tid; k < NPD * nc; k += NT) {
                const int r = k / nc, c = k - r * nc, gg = c / nb, j = c - gg * nb;
                double v = 0.0;
                for (int m = 0; m < TC[j]; ++m) v = fma(K[r * NPD + gg * NPE + TN[j * NPE + m]], TW[j * NPE + m], v);
                KT[r * nc + c] = v;
            }
        __syncthreads();
        if (want_k) {
            bool bad = false;
            for (int k = tid; k < nc * nc; k += NT) {
                const int rr = k / nc, c = k - rr * nc;
                const int f = rr / nb, i = rr - f * nb, gg = c / nb, j = c - gg * nb;
                double v = 0.0;
                for (int m = 0; m < TC[i]; ++m) v = fma(TW[i * NPE + m], KT[(f * NPE + TN[i * NPE + m]) * nc + c], v);
                bad |= !fem_finite(v);
                if (p.mode == MODE_ASSEMBLE) {
                    const int32_t rbase = p.rowptr[f * p.nu + bs[i]];
                    const int32_t ul = p.ulen[bs[i]];
                    atomicAdd(p.vals + rbase + gg * ul + p.sidx[(s * maxnb + i) * maxnb + j], v);
                } else {
                    p.Kout[(s - p.first) * (int64_t)p.nmax * p.nmax + (f * maxnb + i) + (int64_t)(gg * maxnb + j) * p.nmax] = v;
                }
            }
            if (bad) atomicOr(p.status, 1);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// launch plumbing
// Kernel variants of one element type; the autotuner picks one per set.
enum { VAR_WARP4 = 0, VAR_CTA2 = 1, VAR_CTA4 = 2, VAR_CTA8 = 3, NUM_VARIANTS = 4 };
const char* const kVariantNames[NUM_VARIANTS] = {"warp-per-element x4", "cta-per-element 2 warps",
                                                 "cta-per-element 4 warps", "cta-per-element 8 warps"};

struct BulkVariant {
    const void* fn = nullptr;
    int threads = 0;       // per CTA
    int per_cta = 0;       // elements in flight per CTA (warp kernel: warps)
    size_t smem = 0;
    bool warp_kernel = false;
};

template <int D, int NPE, int NGP, int NB, bool RECT>
void fill_variants(BulkVariant* v) {
    using LW = BulkLayout<D, NPE, NGP, NB>;
    using LC = CtaLayout<D, NPE, NGP, NB, RECT>;
    v[VAR_WARP4] = {(const void*)bulk_kernel<D, NPE, NGP, NB, RECT>, 128, 4, LW::kCtaBytes + 4 * LW::kWarpBytes, true};
    v[VAR_CTA2] = {(const void*)bulk_cta_kernel<D, NPE, NGP, NB, RECT, 2>, 64, 1, LC::kBytes, false};
    v[VAR_CTA4] = {(const void*)bulk_cta_kernel<D, NPE, NGP, NB, RECT, 4>, 128, 1, LC::kBytes, false};
    v[VAR_CTA8] = {(const void*)bulk_cta_kernel<D, NPE, NGP, NB, RECT, 8>, 256, 1, LC::kBytes, false};
}

bool pick_bulk(int dim, int ngp, int nb, bool rect, BulkVariant* out, int& NBsel) {
#define FEM_PICK(D, NPE, NGP, NB)                                                               \
    if (dim == D && ngp == NGP && nb <= NB) {                                                   \
        if (rect) fill_variants<D, NPE, NGP, NB, true>(out);                                    \
        else fill_variants<D, NPE, NGP, NB, false>(out);                                        \
        NBsel = NB;                                                                             \
        return true;                                                                            \
    }
    FEM_PICK(2, 4, 4, 4)
    FEM_PICK(2, 4, 4, 9)
    FEM_PICK(2, 4, 4, 16)
    FEM_PICK(3, 8, 8, 8)
    FEM_PICK(3, 8, 8, 27)
    FEM_PICK(3, 8, 27, 8)
    FEM_PICK(3, 8, 27, 27)
#undef FEM_PICK
    return false;
}

}  // namespace fem

// ===========================================================================
using namespace fem;

namespace fem_nodal {

__global__ void nodal_field_kernel(int64_t nn, int dim, int64_t nu, const int64_t* off, const int32_t* rank,
                                   const double* w, const double* u, double* out) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nn * dim;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int f = (int)(t / nn);
        const int64_t n = t - f * nn;
        double s = 0.0;
        for (int64_t k = off[n]; k < off[n + 1]; ++k)
            if (rank[k] >= 0) s = fma(w[k], u[f * nu + rank[k]], s);
        out[t] = s;
    }
}

}  // namespace fem_nodal

namespace {

fem_gpu_status check_kernel(fem_gpu_ctx* c, const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, what);
    return FEM_GPU_OK;
}

fem_gpu_status ensure_device(fem_gpu_ctx* c) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(c, FEM_GPU_NO_DEVICE, "no CUDA device");
    }
    if (!c->stream && !c->stream_set) {
        cudaStream_t s;
        cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e != cudaSuccess) return cuda_fail(c, e, "stream create");
        c->stream = s;
        c->own_stream = true;
    }
    // keep stream-ordered staging buffers cached between calls (host-buffer
    // entry points allocate and free them on every call)
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
    return FEM_GPU_OK;
}

// A buffer argument: device pointer as given, or a staging copy for host data.
struct Staged {
    void* dev = nullptr;
    bool owned = false;
};

fem_gpu_status stage_in(fem_gpu_ctx* c, const void* host_or_dev, size_t bytes, bool host, Staged& s) {
    s = Staged{};
    if (!host_or_dev) return FEM_GPU_OK;
    if (!host) {
        s.dev = const_cast<void*>(host_or_dev);
        return FEM_GPU_OK;
    }
    cudaError_t e = cudaMallocAsync(&s.dev, std::max<size_t>(bytes, 16), stream_of(c));
    if (e != cudaSuccess) return cuda_fail(c, e, "staging alloc");
    s.owned = true;
    e = cudaMemcpyAsync(s.dev, host_or_dev, bytes, cudaMemcpyHostToDevice, stream_of(c));
    if (e != cudaSuccess) return cuda_fail(c, e, "staging copy");
    return FEM_GPU_OK;
}

fem_gpu_status stage_out_alloc(fem_gpu_ctx* c, void* host_or_dev, size_t bytes, bool host, Staged& s) {
    s = Staged{};
    if (!host_or_dev) return FEM_GPU_OK;
    if (!host) {
        s.dev = host_or_dev;
        return FEM_GPU_OK;
    }
    cudaError_t e = cudaMallocAsync(&s.dev, std::max<size_t>(bytes, 16), stream_of(c));
    if (e != cudaSuccess) return cuda_fail(c, e, "staging alloc");
    s.owned = true;
    return FEM_GPU_OK;
}

void release(fem_gpu_ctx* c, Staged& s) {
    if (s.owned && s.dev) cudaFreeAsync(s.dev, stream_of(c));
    s = Staged{};
}

int* status_ptr(fem_gpu_ctx* c) { return (int*)c->d_status.p; }

fem_gpu_status read_status(fem_gpu_ctx* c) {
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, c->d_status.p, sizeof(int), cudaMemcpyDeviceToHost, stream_of(c));
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream_of(c));
    if (e != cudaSuccess) return cuda_fail(c, e, "status read");
    if (h & 1) return fail(c, FEM_GPU_NONFINITE, "non-finite element operator");
    return FEM_GPU_OK;
}

double lam_coef(int model, double nu) {
    return model == FEM_GPU_MODEL_PLANE_STRESS ? nu / (1.0 - nu * nu) : nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
}


fem_gpu_status launch_bulk(fem_gpu_ctx* c, int si, int mode, int64_t first, int64_t count, const double* u,
                           double* vals, double* rhs, double* Kout, double* Rout, int nmax, const double* x,
                           double* y, int force_variant = -1) {
    if (count <= 0) return FEM_GPU_OK;
    SetData& s = c->sets[si];
    BulkVariant vars[NUM_VARIANTS];
    int nbsel = 0;
    const bool rect = c->shape == FEM_GPU_SHAPE_RECTANGULAR;
    if (!s.ig_off.empty()) return fail(c, FEM_GPU_UNSUPPORTED, "non-trivial clusters use the cut-cell kernel");
    if (!pick_bulk(c->dim, s.ngp, s.maxnb, rect, vars, nbsel) || nbsel != s.nbsel)
        return fail(c, FEM_GPU_UNSUPPORTED, "no bulk kernel instance for this element");
    int vi = force_variant >= 0 ? force_variant : s.variant;
    if (!s.rhoe.empty() && vi == VAR_WARP4) {
        if (force_variant >= 0) return fail(c, FEM_GPU_UNSUPPORTED, "density sets use the CTA kernels");
        vi = VAR_CTA4;
    }
    if (mode == MODE_APPLY && vi == VAR_WARP4) vi = VAR_CTA4;
    const BulkVariant& V = vars[vi];
    BulkArgs a{};
    a.ne = count;
    a.first = 0;
    const int NPE = c->npe, D = c->dim;
    a.xe = (const double*)s.d_xe.p + first * NPE * D;
    a.E = (const double*)s.d_E.p + first;
    a.nb = (const int32_t*)s.d_nb.p + first;
    a.bases = (const int32_t*)s.d_bases.p + first * nbsel;
    a.T = (const double*)s.d_T.p + first * NPE * nbsel;
    a.sidx = (const uint16_t*)s.d_sidx.p + first * nbsel * nbsel;
    a.rowptr = (const int32_t*)c->d_rowptr.p;
    a.ulen = (const int32_t*)c->d_ulen.p;
    a.dn = (const double*)s.d_dn.p;
    a.w = (const double*)s.d_w.p;
    a.pairs = (const uint32_t*)s.d_pairs.p;
    a.ktab = (const uint32_t*)s.d_ktab.p;
    a.tri = (const uint16_t*)s.d_tri.p;
    a.g0 = (const double*)s.d_g0.p;
    a.rho = s.rhoe.empty() ? nullptr : (const double*)s.d_rho.p + first * NPE;
    a.nq = (const double*)s.d_nq.p;
    a.beta = s.bulk.density_exponent;
    a.npe = NPE;
    a.nu = c->num_used;
    a.lam_c = lam_coef(s.bulk.model_type, s.bulk.poisson_ratio);
    a.mu_c = 1.0 / (2.0 * (1.0 + s.bulk.poisson_ratio));
    a.u = u;
    a.vals = vals;
    a.rhs = rhs;
    a.Kout = Kout;
    a.Rout = Rout;
    a.nmax = nmax;
    a.kw = s.maxnb;
    a.x = x;
    a.y = y;
    a.status = status_ptr(c);
    // status words 2-3: the element counter of the CTA kernels
    a.queue = reinterpret_cast<unsigned long long*>(status_ptr(c) + 2);
    cudaError_t e = cudaFuncSetAttribute(V.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)V.smem);
    if (e != cudaSuccess) return cuda_fail(c, e, "bulk smem attribute");
    if (!V.warp_kernel) {
        e = cudaMemsetAsync(a.queue, 0, sizeof(unsigned long long), stream_of(c));
        if (e != cudaSuccess) return cuda_fail(c, e, "bulk element counter");
    }
    // exactly the resident CTAs: they take elements in order (the CTA kernels
    // from a device counter, the warp kernel by grid stride), one compact
    // front whose CSR rows stay in L2
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, V.fn, V.threads, V.smem);
    if (e != cudaSuccess) return cuda_fail(c, e, "bulk occupancy");
    if (per_sm < 1) return fail(c, FEM_GPU_UNSUPPORTED, "bulk kernel does not fit on an SM");
    int64_t blocks = (count + V.per_cta - 1) / V.per_cta;
    const int64_t cap = (int64_t)sm_count() * per_sm;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    int W = V.per_cta;
    void* args_w[] = {&a, &mode, &W};
    void* args_c[] = {&a, &mode};
    e = cudaLaunchKernel(V.fn, dim3((unsigned)blocks), dim3(V.threads), V.warp_kernel ? args_w : args_c, V.smem,
                         stream_of(c));
    if (e != cudaSuccess) return cuda_fail(c, e, "bulk launch");
    c->launches++;
    return FEM_GPU_OK;
}

fem_gpu_status launch_side(fem_gpu_ctx* c, int si, int mode, int64_t first, int64_t count, const double* u,
                           double* vals, double* rhs, double* Kout, double* Rout, int nmax) {
    if (count <= 0) return FEM_GPU_OK;
    SetData& s = c->sets[si];
    SetData& ds = s;
    SideArgs a{};
    a.ns = count;
    a.iwg = s.side.iwg_type;
    a.model = s.side.model_type;
    a.ngp = ds.ngp;
    a.maxnb = s.maxnb;
    const int NPE = c->npe, D = c->dim;
    a.xe = (const double*)s.d_xe.p + first * NPE * D;
    a.E = (const double*)s.d_E.p + first;
    a.ord = (const int32_t*)s.d_ord.p + first;
    a.nb = (const int32_t*)s.d_nb.p + first;
    a.bases = (const int32_t*)s.d_bases.p + first * s.maxnb;
    a.T = (const double*)s.d_T.p + first * NPE * s.maxnb;
    a.sidx = (const uint16_t*)s.d_sidx.p + first * s.maxnb * s.maxnb;
    a.rowptr = (const int32_t*)c->d_rowptr.p;
    a.ulen = (const int32_t*)c->d_ulen.p;
    a.gp = (const double*)ds.d_gp.p;
    a.gw = (const double*)ds.d_gw.p;
    a.sref = (const double*)ds.d_sref.p;
    a.sgeo = (const double*)ds.d_sgeo.p + first * side_geo_len(ds.ngp);
    a.rect = c->shape == FEM_GPU_SHAPE_RECTANGULAR;
    a.select_identity = 1;
    for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j)
            if (s.side_select[i * 3 + j] != (i == j ? 1.0 : 0.0)) a.select_identity = 0;
    a.nu = c->num_used;
    a.nu_p = s.side.poisson_ratio;
    a.alpha = s.side.nitsche_alpha;
    for (int d = 0; d < 3; ++d) a.value[d] = s.side.value[d];
    a.thickness = s.side_thickness;
    for (int k = 0; k < 9; ++k) a.select[k] = s.side_select[k];
    a.u = u;
    a.vals = vals;
    a.rhs = rhs;
    a.Kout = Kout;
    a.Rout = Rout;
    a.nmax = nmax;
    a.first = 0;
    a.mode = mode;
    a.status = status_ptr(c);
    const size_t smem = SideSmem::bytes(D, s.maxnb, ds.ngp);
    const void* fn = D == 2 ? (const void*)side_cta_kernel<2> : (const void*)side_cta_kernel<3>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return cuda_fail(c, e, "side kernel shared memory");
    }
    const int threads = 128;
    const unsigned blocks = (unsigned)std::min<int64_t>(count, (int64_t)sm_count() * 8);
    if (D == 2) side_cta_kernel<2><<<blocks, threads, smem, stream_of(c)>>>(a);
    else side_cta_kernel<3><<<blocks, threads, smem, stream_of(c)>>>(a);
    c->launches++;
    return check_kernel(c, "side launch");
}

}  // namespace

namespace fem {

int sm_count() {
    // multiprocessor count of the current device, read once per device
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) {
        cudaGetLastError();
        return 1;
    }
    if (dev < 64) {
        const int v = cache[dev].load(std::memory_order_relaxed);
        if (v > 0) return v;
    }
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    n = n > 0 ? n : 1;
    if (dev < 64) cache[dev].store(n, std::memory_order_relaxed);
    return n;
}


fem_gpu_status assemble_set(fem_gpu_ctx* c, int set, const double* u, double* vals, double* rhs) {
    SetData& s = c->sets[set];
    if (cluster_set(c, set))
        return cluster_launch_set(c, set, MODE_ASSEMBLE, 0, s.neq, u, vals, rhs, nullptr, nullptr, 0);
    if (s.kind == 0)
        return launch_bulk(c, set, MODE_ASSEMBLE, 0, s.neq, u, vals, rhs, nullptr, nullptr, 0, nullptr, nullptr);
    return launch_side(c, set, MODE_ASSEMBLE, 0, s.neq, u, vals, rhs, nullptr, nullptr, 0);
}

// a side set launched on a given stream (the batched graph captures it)
fem_gpu_status side_launch_on(fem_gpu_ctx* c, int set, const double* u, double* vals, double* rhs, cudaStream_t st) {
    void* keep = c->stream;
    c->stream = st;
    fem_gpu_status r = launch_side(c, set, MODE_ASSEMBLE, 0, c->sets[set].neq, u, vals, rhs, nullptr, nullptr, 0);
    c->stream = keep;
    return r;
}

// Host-buffer assembly overlaps the copy-back of the CSR values with the
// element loop: the work runs in chunks (bulk sets split by element index, the
// other sets whole); after chunk w every CSR row whose basis rank is below
// final_rank[w] -- the smallest basis rank any later chunk touches -- is final,
// and its values go to the host on a copy stream while the next chunk computes.
// On the reference's mesh orderings (x fastest, z slowest) the rows finish in
// slabs, so nearly all of the transfer hides behind the kernels.
struct HostPipe {
    std::vector<int> set;
    std::vector<int64_t> first, count, final_rank;
    cudaStream_t copy = nullptr;
    std::vector<cudaEvent_t> done;  // one per chunk, and the copy stream's end
};

void host_pipe_release(fem_gpu_ctx* c) {
    HostPipe* hp = (HostPipe*)c->host_pipe;
    if (!hp) return;
    if (hp->copy) cudaStreamSynchronize(hp->copy);
    for (cudaEvent_t e : hp->done) cudaEventDestroy(e);
    if (hp->copy) cudaStreamDestroy(hp->copy);
    delete hp;
    c->host_pipe = nullptr;
}

HostPipe* host_pipe(fem_gpu_ctx* c) {
    if (c->host_pipe) return (HostPipe*)c->host_pipe;
    HostPipe* hp = new HostPipe();
    // the copy of the last chunk and the kernel of the first are not
    // overlapped, and every chunk has a fixed cost (launch, event, copy): on
    // the 64^3 benchmark 16 chunks measured best (8 and 32 were slower)
    constexpr int64_t kChunk = 16384;  // elements per bulk chunk (at least)
    constexpr int64_t kChunks = 16;
    std::vector<int64_t> minb;
    for (int k = 0; k < (int)c->sets.size(); ++k) {
        const SetData& s = c->sets[k];
        const int64_t step =
            (!cluster_set(c, k) && s.kind == 0) ? std::max<int64_t>(kChunk, (s.neq + kChunks - 1) / kChunks) : s.neq;
        const int64_t width = s.neq ? (int64_t)s.bases.size() / s.neq : 0;
        for (int64_t f = 0; f < s.neq; f += step) {
            const int64_t n = std::min(step, s.neq - f);
            int64_t mb = c->num_used;
            for (int64_t i = f * width; i < (f + n) * width; ++i)
                if (s.bases[i] >= 0) mb = std::min<int64_t>(mb, s.bases[i]);
            hp->set.push_back(k);
            hp->first.push_back(f);
            hp->count.push_back(n);
            minb.push_back(mb);
        }
    }
    hp->final_rank.assign(minb.size(), c->num_used);
    for (int64_t w = (int64_t)minb.size() - 2; w >= 0; --w)
        hp->final_rank[w] = std::min(hp->final_rank[w + 1], minb[w + 1]);
    cudaError_t e = cudaStreamCreateWithFlags(&hp->copy, cudaStreamNonBlocking);
    hp->done.assign(minb.size() + 1, nullptr);
    for (auto& ev : hp->done)
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    c->host_pipe = hp;
    if (e != cudaSuccess) {
        host_pipe_release(c);
        return nullptr;
    }
    return hp;
}

void device_release(fem_gpu_ctx* c) {
    host_pipe_release(c);
    cluster_release(c);
    sensitivity_release(c);
    for (auto& s : c->sets) {
        dfree(s.d_nb);
        dfree(s.d_bases);
        dfree(s.d_T);
        dfree(s.d_sidx);
        dfree(s.d_xe);
        dfree(s.d_E);
        dfree(s.d_ord);
        dfree(s.d_dn);
        dfree(s.d_w);
        dfree(s.d_pairs);
        dfree(s.d_ktab);
        dfree(s.d_tri);
        dfree(s.d_g0);
        dfree(s.d_rho);
        dfree(s.d_nq);
        dfree(s.d_gp);
        dfree(s.d_gw);
        dfree(s.d_sref);
        dfree(s.d_sgeo);
    }
    dfree(c->d_rowptr);
    dfree(c->d_ulen);
    dfree(c->d_tables);
    dfree(c->d_scratch);
    dfree(c->d_status);
    if (c->own_stream && c->stream) cudaStreamDestroy((cudaStream_t)c->stream);
    c->stream = nullptr;
    c->own_stream = false;
    c->dev_final = false;
}

fem_gpu_status device_finalize(fem_gpu_ctx* c) {
    fem_gpu_status st = ensure_device(c);
    if (st != FEM_GPU_OK) return st;
    cudaStream_t sm = stream_of(c);
    cudaError_t e;
    if ((e = upload(c->d_rowptr, c->rowptr, sm)) != cudaSuccess) return cuda_fail(c, e, "rowptr");
    if ((e = upload(c->d_ulen, c->ulen, sm)) != cudaSuccess) return cuda_fail(c, e, "ulen");
    std::vector<int> zero(4, 0);
    if ((e = upload(c->d_status, zero, sm)) != cudaSuccess) return cuda_fail(c, e, "status");
    for (size_t k = 0; k < c->sets.size(); ++k) {
        SetData& s = c->sets[k];
        SetData& ds = s;
        const int NPE = c->npe, D = c->dim;
        if (s.neq == 0) continue;  // an empty set has no device data
        if (cluster_set(c, (int)k)) {
            if ((st = cluster_finalize(c, (int)k)) != FEM_GPU_OK) return st;
            continue;
        }
        if (s.kind == 0) {
            const Rule r = gauss_rule(s.bulk.integration_rule);
            if (r.n > kMaxGP) return fail(c, FEM_GPU_UNSUPPORTED, "too many Gauss points");
            ds.ngp = r.n;
            std::vector<double> dn((size_t)r.n * D * NPE), w(r.w), nq((size_t)r.n * NPE);
            for (int q = 0; q < r.n; ++q) {
                double N[8], d[24];
                lagrange(c->ip_cell, &r.pts[(size_t)q * r.dim], N, d);
                for (int i = 0; i < D * NPE; ++i) dn[(size_t)q * D * NPE + i] = d[i];
                for (int a = 0; a < NPE; ++a) nq[(size_t)q * NPE + a] = N[a];
            }
            if ((e = upload(ds.d_nq, nq, sm)) != cudaSuccess) return cuda_fail(c, e, "N table");
            if (!s.rhoe.empty())
                if ((e = upload(ds.d_rho, s.rhoe, sm)) != cudaSuccess) return cuda_fail(c, e, "densities");
            if ((e = upload(ds.d_dn, dn, sm)) != cudaSuccess) return cuda_fail(c, e, "dn table");
            if ((e = upload(ds.d_w, w, sm)) != cudaSuccess) return cuda_fail(c, e, "w table");
            // rule points for the cluster kernel (batched launch)
            if ((e = upload(ds.d_gp, r.pts, sm)) != cudaSuccess) return cuda_fail(c, e, "rule points");
            if ((e = upload(ds.d_gw, r.w, sm)) != cudaSuccess) return cuda_fail(c, e, "rule weights");
            const int npd = D * NPE;
            // upper-triangle pdof pairs, those of the diagonal field blocks (which
            // carry the trace term) first, so that warps of the stiffness phase
            // run one branch
            std::vector<uint32_t> pairs;
            for (int diag = 1; diag >= 0; --diag)
                for (int rr = 0; rr < npd; ++rr)
                    for (int cc = rr; cc < npd; ++cc)
                        if ((rr / NPE == cc / NPE) == (diag == 1)) pairs.push_back((uint32_t)rr << 16 | (uint32_t)cc);
            if ((e = upload(ds.d_pairs, pairs, sm)) != cudaSuccess) return cuda_fail(c, e, "pair table");
            // reference Gram table of the rule (constant-Jacobian cells)
            std::vector<double> g0((size_t)npd * npd, 0.0);
            for (int rr = 0; rr < npd; ++rr)
                for (int cc = 0; cc < npd; ++cc) {
                    double acc = 0.0;
                    for (int q = 0; q < r.n; ++q)
                        acc += r.w[q] * dn[(size_t)q * npd + rr] * dn[(size_t)q * npd + cc];
                    g0[(size_t)rr * npd + cc] = acc;
                }
            if ((e = upload(ds.d_g0, g0, sm)) != cudaSuccess) return cuda_fail(c, e, "g0 table");
            BulkVariant vars[NUM_VARIANTS];
            int nbsel = 0;
            if (s.ig_off.empty() && !pick_bulk(D, r.n, s.maxnb, c->shape == FEM_GPU_SHAPE_RECTANGULAR, vars, nbsel))
                return fail(c, FEM_GPU_UNSUPPORTED, "no bulk kernel instance for this element");
            ds.nbsel = nbsel ? nbsel : s.maxnb;
            ds.variant = VAR_CTA4;
            if (nbsel) {
                // item tables of bulk_cta_kernel, in the packing its loads decode
                const int NB = nbsel, NAD = D * NB;
                std::vector<uint32_t> kt;
                for (int sl = 0; sl < NB; ++sl)
                    for (int gg = 0; gg < D; ++gg)
                        for (int f = 0; f < D; ++f)
                            for (int a = 0; a < NPE; ++a) {
                                const uint32_t kb = (uint32_t)(gg * NPE * npd + f * NPE + a);
                                const uint32_t dst = (uint32_t)((f * NPE + a) * NAD + sl * D + gg);
                                kt.push_back((uint32_t)sl | kb << 6 | dst << 16);
                            }
                std::vector<uint16_t> tri;
                for (int x = 0; x < NAD; ++x)
                    for (int y = x; y < NAD; ++y)
                        tri.push_back((uint16_t)((x / D) | (x % D) << 5 | (y / D) << 7 | (y % D) << 12));
                if ((e = upload(ds.d_ktab, kt, sm)) != cudaSuccess) return cuda_fail(c, e, "K T table");
                if ((e = upload(ds.d_tri, tri, sm)) != cudaSuccess) return cuda_fail(c, e, "triangle table");
            }
        } else {
            const Rule r = gauss_rule(s.side.integration_rule);
            ds.ngp = r.n;
            if ((e = upload(ds.d_gp, r.pts, sm)) != cudaSuccess) return cuda_fail(c, e, "side gp");
            if ((e = upload(ds.d_gw, r.w, sm)) != cudaSuccess) return cuda_fail(c, e, "side gw");
            // the geometry-independent shape values of every facet ordinal and
            // point: the facet's own derivatives, the cell's N and dN/dxi at the
            // point's image in the cell
            {
                const int D = c->dim, NFV = D == 2 ? 2 : 4, nord = D == 2 ? 4 : 6, REF = side_ref_len(D);
                std::vector<double> ref((size_t)nord * r.n * REF, 0.0);
                for (int o = 0; o < nord; ++o)
                    for (int q = 0; q < r.n; ++q) {
                        double* out = ref.data() + ((size_t)o * r.n + q) * REF;
                        double Nf[4], dNf[8], xip[3] = {0, 0, 0};
                        const double* xq = r.pts.data() + q * (D - 1);
                        if (D == 2) Shape<4>::eval(xq, Nf, dNf);
                        else Shape<0>::eval(xq, Nf, dNf);
                        for (int k = 0; k < NFV; ++k) {
                            const int v = side_face_vertex(D, o, k);
                            const double xiv[3] = {((v & 3) == 1 || (v & 3) == 2) ? 1.0 : -1.0,
                                                   ((v & 3) >= 2) ? 1.0 : -1.0, v >= 4 ? 1.0 : -1.0};
                            for (int d = 0; d < D; ++d) xip[d] = std::fma(Nf[k], xiv[d], xip[d]);
                        }
                        for (int k = 0; k < (D - 1) * NFV; ++k) out[k] = dNf[k];
                        if (D == 2) Shape<0>::eval(xip, out + (D - 1) * NFV, out + (D - 1) * NFV + 4);
                        else Shape<1>::eval(xip, out + (D - 1) * NFV, out + (D - 1) * NFV + 8);
                    }
                if ((e = upload(ds.d_sref, ref, sm)) != cudaSuccess) return cuda_fail(c, e, "side reference table");
            }
            ds.nbsel = s.maxnb;
        }
        // repack element data to the kernel's padded basis width (the host
        // arrays are already in that layout when the set's width is W)
        const int W = ds.nbsel;
        const bool same = W == s.maxnb;
        std::vector<int32_t> bases(same ? 0 : (size_t)s.neq * W, -1);
        std::vector<double> T(same ? 0 : (size_t)s.neq * NPE * W, 0.0);
        std::vector<uint16_t> sidx(same ? 0 : (size_t)s.neq * W * W, 0);
        for (int64_t i = 0; i < (same ? 0 : s.neq); ++i) {
            for (int j = 0; j < s.maxnb; ++j) bases[i * W + j] = s.bases[i * s.maxnb + j];
            for (int a = 0; a < NPE; ++a)
                for (int j = 0; j < s.maxnb; ++j) T[(i * NPE + a) * W + j] = s.T[(i * NPE + a) * s.maxnb + j];
            for (int ii = 0; ii < s.maxnb; ++ii)
                for (int jj = 0; jj < s.maxnb; ++jj)
                    sidx[(i * W + ii) * W + jj] = s.sidx[(i * s.maxnb + ii) * s.maxnb + jj];
        }
        if ((e = upload(s.d_nb, s.nb, sm)) != cudaSuccess) return cuda_fail(c, e, "nb");
        if ((e = upload(s.d_bases, same ? s.bases : bases, sm)) != cudaSuccess) return cuda_fail(c, e, "bases");
        if ((e = upload(s.d_T, same ? s.T : T, sm)) != cudaSuccess) return cuda_fail(c, e, "T");
        if ((e = upload(s.d_sidx, same ? s.sidx : sidx, sm)) != cudaSuccess) return cuda_fail(c, e, "sidx");
        if ((e = upload(s.d_xe, s.xe, sm)) != cudaSuccess) return cuda_fail(c, e, "xe");
        if ((e = upload(s.d_E, s.E, sm)) != cudaSuccess) return cuda_fail(c, e, "E");
        if (s.kind == 1) {
            if ((e = upload(s.d_ord, s.ordinal, sm)) != cudaSuccess) return cuda_fail(c, e, "ordinals");
            // the facet geometry, once
            const int64_t ns = s.neq;
            const std::vector<double> zeros((size_t)std::max<int64_t>(ns, 1) * side_geo_len(s.ngp), 0.0);
            if ((e = upload(s.d_sgeo, zeros, sm)) != cudaSuccess) return cuda_fail(c, e, "side geometry");
            if (ns > 0) {
                const int rect = c->shape == FEM_GPU_SHAPE_RECTANGULAR;
                const unsigned g1 = (unsigned)std::min<int64_t>((ns * s.ngp + 255) / 256, (int64_t)sm_count() * 8);
                const unsigned g2 = (unsigned)std::min<int64_t>((ns + 255) / 256, (int64_t)sm_count() * 8);
                double* out = (double*)s.d_sgeo.p;
                if (c->dim == 2) {
                    side_geometry_kernel<2><<<g1, 256, 0, sm>>>(ns, s.ngp, (const double*)s.d_xe.p,
                                                                (const int32_t*)s.d_ord.p, (const double*)s.d_gw.p,
                                                                (const double*)s.d_sref.p, rect, s.side_thickness, out);
                    side_h_kernel<2><<<g2, 256, 0, sm>>>(ns, s.ngp, out);
                } else {
                    side_geometry_kernel<3><<<g1, 256, 0, sm>>>(ns, s.ngp, (const double*)s.d_xe.p,
                                                                (const int32_t*)s.d_ord.p, (const double*)s.d_gw.p,
                                                                (const double*)s.d_sref.p, rect, s.side_thickness, out);
                    side_h_kernel<3><<<g2, 256, 0, sm>>>(ns, s.ngp, out);
                }
                if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(c, e, "side geometry kernel");
            }
        }
        if (s.kind == 1) s.maxnb = W;
    }
    // the side kernel and host topology read maxnb-padded arrays: keep the
    // host copies consistent with the device padding for bulk sets too
    for (size_t k = 0; k < c->sets.size(); ++k) {
        SetData& s = c->sets[k];
        const int W = s.nbsel;
        if (cluster_set(c, (int)k)) continue;
        if (s.kind == 0 && W != s.maxnb) {
            std::vector<int32_t> b((size_t)s.neq * W, -1);
            for (int64_t i = 0; i < s.neq; ++i)
                for (int j = 0; j < s.maxnb; ++j) b[i * W + j] = s.bases[i * s.maxnb + j];
            s.bases.swap(b);
            s.maxnb = W;
            s.T.clear();
            s.sidx.clear();
        }
    }
    e = cudaStreamSynchronize(sm);
    if (e != cudaSuccess) return cuda_fail(c, e, "finalize sync");
    c->dev_final = true;
    return FEM_GPU_OK;
}

}  // namespace fem

extern "C" {

int32_t fem_gpu_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

fem_gpu_status fem_gpu_set_stream(fem_gpu_ctx* c, void* stream) {
    if (!c) return FEM_GPU_BAD_ARG;
    if (c->own_stream && c->stream) {
        cudaStreamSynchronize((cudaStream_t)c->stream);
        cudaStreamDestroy((cudaStream_t)c->stream);
    }
    c->stream = stream;
    c->own_stream = false;
    c->stream_set = true;
    return FEM_GPU_OK;
}

fem_gpu_status fem_gpu_finalize(fem_gpu_ctx* c) {
    if (!c) return FEM_GPU_BAD_ARG;
    fem_gpu_status st = fem_gpu_finalize_host(c);
    if (st != FEM_GPU_OK) return st;
    if (c->dev_final) return FEM_GPU_OK;
    st = device_finalize(c);
    if (st != FEM_GPU_OK) return st;
    // resolve the allocation-free solver's array on this device now, so that
    // loading its module (which reserves the array) happens here and not
    // inside a later fem_gpu_pcg_noalloc call
    return noalloc_prepare(c);
}

fem_gpu_status fem_gpu_build_graph(fem_gpu_ctx* c, int32_t* rowptr, int32_t* colidx, uint32_t flags) {
    if (!c || !rowptr || !colidx) return FEM_GPU_BAD_ARG;
    if (!c->host_final) return FEM_GPU_NOT_FINALIZED;
    const int64_t nad = c->num_used * c->dim;
    std::vector<int32_t> ci;
    int32_t* outc = colidx;
    const bool host = flags & FEM_GPU_HOST_BUFFERS;
    if (!host) {
        ci.resize(c->nnz);
        outc = ci.data();
    }
    for (int f = 0; f < c->dim; ++f)
        for (int64_t b = 0; b < c->num_used; ++b) {
            int32_t* o = outc + c->rowptr[f * c->num_used + b];
            const int32_t* u = c->ucols.data() + c->uoff[b];
            for (int g = 0; g < c->dim; ++g)
                for (int32_t k = 0; k < c->ulen[b]; ++k) *o++ = (int32_t)(g * c->num_used + u[k]);
        }
    if (host) {
        std::memcpy(rowptr, c->rowptr.data(), (nad + 1) * sizeof(int32_t));
        return FEM_GPU_OK;
    }
    fem_gpu_status st = ensure_device(c);
    if (st != FEM_GPU_OK) return st;
    cudaError_t e = cudaMemcpyAsync(rowptr, c->rowptr.data(), (nad + 1) * sizeof(int32_t), cudaMemcpyHostToDevice,
                                    stream_of(c));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(colidx, ci.data(), c->nnz * sizeof(int32_t), cudaMemcpyHostToDevice, stream_of(c));
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream_of(c));
    if (e != cudaSuccess) return cuda_fail(c, e, "graph upload");
    return FEM_GPU_OK;
}

fem_gpu_status fem_gpu_element_matrices(fem_gpu_ctx* c, int32_t set, int64_t first, int64_t count,
                                        const double* u, double* K, double* R, uint32_t flags) {
    if (!c || set < 0 || set >= (int32_t)c->sets.size() || count < 0) return FEM_GPU_BAD_ARG;
    if (!c->dev_final) return FEM_GPU_NOT_FINALIZED;
    SetData& s = c->sets[set];
    if (first < 0 || first + count > s.neq) return FEM_GPU_OOB_INDEX;
    if (count == 0) return FEM_GPU_OK;
    const int nmax = s.maxnb * c->dim * (s.kind == 2 ? 2 : 1);
    const bool host = flags & FEM_GPU_HOST_BUFFERS;
    const int64_t nad = c->num_used * c->dim;
    Staged su, sk, sr;
    fem_gpu_status st;
    if ((st = stage_in(c, u, nad * sizeof(double), host, su)) != FEM_GPU_OK) return st;
    if ((st = stage_out_alloc(c, K, (size_t)count * nmax * nmax * sizeof(double), host, sk)) != FEM_GPU_OK) return st;
    if ((st = stage_out_alloc(c, R, (size_t)count * nmax * sizeof(double), host, sr)) != FEM_GPU_OK) return st;
    cudaStream_t sm = stream_of(c);
    if (sk.dev) cudaMemsetAsync(sk.dev, 0, (size_t)count * nmax * nmax * sizeof(double), sm);
    if (sr.dev) cudaMemsetAsync(sr.dev, 0, (size_t)count * nmax * sizeof(double), sm);
    cudaMemsetAsync(c->d_status.p, 0, sizeof(int), sm);
    if (cluster_set(c, set))
        st = cluster_launch_set(c, set, MODE_ELEMENT, first, count, (const double*)su.dev, nullptr, nullptr,
                                (double*)sk.dev, (double*)sr.dev, nmax);
    else if (s.kind == 0)
        st = launch_bulk(c, set, MODE_ELEMENT, first, count, (const double*)su.dev, nullptr, nullptr,
                         (double*)sk.dev, (double*)sr.dev, nmax, nullptr, nullptr);
    else
        st = launch_side(c, set, MODE_ELEMENT, first, count, (const double*)su.dev, nullptr, nullptr,
                         (double*)sk.dev, (double*)sr.dev, nmax);
    if (st == FEM_GPU_OK) {
        cudaError_t e = cudaSuccess;
        if (host && K) e = cudaMemcpyAsync(K, sk.dev, (size_t)count * nmax * nmax * sizeof(double), cudaMemcpyDeviceToHost, sm);
        if (e == cudaSuccess && host && R)
            e = cudaMemcpyAsync(R, sr.dev, (size_t)count * nmax * sizeof(double), cudaMemcpyDeviceToHost, sm);
        if (e != cudaSuccess) st = cuda_fail(c, e, "element matrices copy");
    }
    release(c, su);
    release(c, sk);
    release(c, sr);
    if (st != FEM_GPU_OK) return st;
    return read_status(c);
}

fem_gpu_status fem_gpu_assemble(fem_gpu_ctx* c, const double* u, double* vals, double* rhs, uint32_t flags) {
    if (!c) return FEM_GPU_BAD_ARG;
    if (!c->dev_final) return FEM_GPU_NOT_FINALIZED;
    const bool host = flags & FEM_GPU_HOST_BUFFERS;
    const int64_t nad = c->num_used * c->dim;
    double* v = (flags & FEM_GPU_NO_JACOBIAN) ? nullptr : vals;
    double* r = (flags & FEM_GPU_NO_RESIDUAL) ? nullptr : rhs;
    if (!v && !r) return FEM_GPU_BAD_ARG;
    Staged su, sv, sr;
    fem_gpu_status st;
    if ((st = stage_in(c, u, nad * sizeof(double), host, su)) != FEM_GPU_OK) return st;
    const bool acc = flags & FEM_GPU_ACCUMULATE;
    if (acc) {
        if ((st = stage_in(c, v, c->nnz * sizeof(double), host, sv)) != FEM_GPU_OK) return st;
        if ((st = stage_in(c, r, nad * sizeof(double), host, sr)) != FEM_GPU_OK) return st;
    } else {
        if ((st = stage_out_alloc(c, v, c->nnz * sizeof(double), host, sv)) != FEM_GPU_OK) return st;
        if ((st = stage_out_alloc(c, r, nad * sizeof(double), host, sr)) != FEM_GPU_OK) return st;
    }
    cudaStream_t sm = stream_of(c);
    if (!acc) {
        if (sv.dev) cudaMemsetAsync(sv.dev, 0, c->nnz * sizeof(double), sm);
        if (sr.dev) cudaMemsetAsync(sr.dev, 0, nad * sizeof(double), sm);
    }
    cudaMemsetAsync(c->d_status.p, 0, sizeof(int), sm);
    auto run = [&](int k, int64_t first, int64_t count) {
        SetData& s = c->sets[k];
        if (cluster_set(c, k))
            return cluster_launch_set(c, k, MODE_ASSEMBLE, first, count, (const double*)su.dev, (double*)sv.dev,
                                      (double*)sr.dev, nullptr, nullptr, 0);
        if (s.kind == 0)
            return launch_bulk(c, k, MODE_ASSEMBLE, first, count, (const double*)su.dev, (double*)sv.dev,
                               (double*)sr.dev, nullptr, nullptr, 0, nullptr, nullptr);
        return launch_side(c, k, MODE_ASSEMBLE, first, count, (const double*)su.dev, (double*)sv.dev, (double*)sr.dev,
                           nullptr, nullptr, 0);
    };
    HostPipe* hp = (host && v) ? host_pipe(c) : nullptr;
    if (hp) {
        const int64_t nu = c->num_used;
        int64_t done_rank = 0;
        cudaError_t e = cudaSuccess;
        for (size_t w = 0; w < hp->set.size() && st == FEM_GPU_OK && e == cudaSuccess; ++w) {
            st = run(hp->set[w], hp->first[w], hp->count[w]);
            const int64_t fin = hp->final_rank[w];
            if (st != FEM_GPU_OK || fin <= done_rank) continue;
            e = cudaEventRecord(hp->done[w], sm);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(hp->copy, hp->done[w], 0);
            for (int f = 0; f < c->dim && e == cudaSuccess; ++f) {
                const int64_t lo = c->rowptr[f * nu + done_rank], hi = c->rowptr[f * nu + fin];
                e = cudaMemcpyAsync(v + lo, (double*)sv.dev + lo, (hi - lo) * sizeof(double), cudaMemcpyDeviceToHost,
                                    hp->copy);
            }
            done_rank = fin;
        }
        // the residual after the last chunk; the compute stream then waits for
        // the copy stream so that the staging release and the status read follow
        if (e == cudaSuccess && st == FEM_GPU_OK && r)
            e = cudaMemcpyAsync(r, sr.dev, nad * sizeof(double), cudaMemcpyDeviceToHost, sm);
        if (e == cudaSuccess) e = cudaEventRecord(hp->done.back(), hp->copy);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(sm, hp->done.back(), 0);
        if (e != cudaSuccess) st = cuda_fail(c, e, "assemble copy back");
    } else {
        for (int k = 0; k < (int)c->sets.size() && st == FEM_GPU_OK; ++k) st = run(k, 0, c->sets[k].neq);
        if (st == FEM_GPU_OK && host) {
            cudaError_t e = cudaSuccess;
            if (v) e = cudaMemcpyAsync(v, sv.dev, c->nnz * sizeof(double), cudaMemcpyDeviceToHost, sm);
            if (e == cudaSuccess && r) e = cudaMemcpyAsync(r, sr.dev, nad * sizeof(double), cudaMemcpyDeviceToHost, sm);
            if (e != cudaSuccess) st = cuda_fail(c, e, "assemble copy back");
        }
    }
    release(c, su);
    release(c, sv);
    release(c, sr);
    if (st != FEM_GPU_OK) return st;
    return read_status(c);
}

// nodal values of an adof field at the interpolation-mesh nodes through the
// node extraction rows (the values the reference's VIS output evaluates at
// the vertices, VIS::Output_Manager::write_field, FEM/VIS/src/
// cl_VIS_Output_Manager.cpp:679-785): out[f][node] = sum_k w_k u[f nu + rank_k]
fem_gpu_status fem_gpu_nodal_field(fem_gpu_ctx* c, const double* u, double* out) {
    if (!c || !u || !out) return FEM_GPU_BAD_ARG;
    if (!c->dev_final) return FEM_GPU_NOT_FINALIZED;
    const int64_t nn = c->num_nodes, nz = (int64_t)c->t_bases.size();
    std::vector<int32_t> rk(nz);
    for (int64_t k = 0; k < nz; ++k) rk[k] = (int32_t)c->basis_rank[c->t_bases[k]];
    int64_t* doff = nullptr;
    int32_t* drk = nullptr;
    double* dw = nullptr;
    cudaStream_t sm = stream_of(c);
    cudaError_t e = cudaMallocAsync(&doff, (nn + 1) * sizeof(int64_t), sm);
    if (e == cudaSuccess) e = cudaMallocAsync(&drk, std::max<int64_t>(nz, 1) * sizeof(int32_t), sm);
    if (e == cudaSuccess) e = cudaMallocAsync(&dw, std::max<int64_t>(nz, 1) * sizeof(double), sm);
    if (e == cudaSuccess) e = cudaMemcpyAsync(doff, c->t_off.data(), (nn + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, sm);
    if (e == cudaSuccess && nz) e = cudaMemcpyAsync(drk, rk.data(), nz * sizeof(int32_t), cudaMemcpyHostToDevice, sm);
    if (e == cudaSuccess && nz) e = cudaMemcpyAsync(dw, c->t_w.data(), nz * sizeof(double), cudaMemcpyHostToDevice, sm);
    if (e == cudaSuccess) {
        const int64_t n = nn * c->dim;
        fem_nodal::nodal_field_kernel<<<(unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 16), 256, 0, sm>>>(
            nn, c->dim, c->num_used, doff, drk, dw, u, out);
        ++c->launches;
        e = cudaGetLastError();
    }
    cudaFreeAsync(doff, sm);
    cudaFreeAsync(drk, sm);
    cudaFreeAsync(dw, sm);
    if (e == cudaSuccess) e = cudaStreamSynchronize(sm);
    return e == cudaSuccess ? FEM_GPU_OK : cuda_fail(c, e, "nodal field");
}

}  // extern "C"

namespace fem_flux {

// stress sigma = D eps(u) of one bulk equation object at an IP-parametric
// point (CM_Struc_Linear::flux, FEM/INT/src/CM/cl_FEM_CM_Struc_Linear.cpp:
// 280-302, strain by eval_strain_2d / _3d :349-498, D by CM_Struc_Linear_
// Isotropic :61-392), one thread per point; the element data of the points
// are gathered by the host, u_pdof = T u_adof in the kernel
template <int D>
__global__ void flux_kernel(int64_t n, int maxnb, int model, double nu_p, const double* xe, const double* T,
                            const int32_t* bases, const int32_t* nb, const double* E, const double* rho, double beta,
                            const double* xi, const double* u, int64_t nu, int ncomp, double* out) {
    constexpr int NPE = D == 2 ? 4 : 8;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        double N[NPE], dN[NPE * D];
        if (D == 2) Shape<0>::eval(xi + k * D, N, dN);
        else Shape<1>::eval(xi + k * D, N, dN);
        const double* X = xe + k * NPE * D;
        double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, Ji[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int i = 0; i < D; ++i)
            for (int j = 0; j < D; ++j)
                for (int a = 0; a < NPE; ++a) J[i][j] = fma(dN[i * NPE + a], X[a * D + j], J[i][j]);
        if (D == 2) {
            const double id = 1.0 / (J[0][0] * J[1][1] - J[0][1] * J[1][0]);
            Ji[0][0] = J[1][1] * id; Ji[0][1] = -J[0][1] * id; Ji[1][0] = -J[1][0] * id; Ji[1][1] = J[0][0] * id;
        } else {
            const double id = 1.0 / (J[0][0] * (J[1][1] * J[2][2] - J[2][1] * J[1][2]) -
                                     J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                                     J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]));
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
        // grad[f][i] = du_f / dx_i
        double grad[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int a = 0; a < NPE; ++a) {
            double g[3] = {0, 0, 0};
            for (int i = 0; i < D; ++i)
                for (int kk = 0; kk < D; ++kk) g[i] = fma(Ji[i][kk], dN[kk * NPE + a], g[i]);
            for (int f = 0; f < D; ++f) {
                double up = 0.0;
                for (int j = 0; j < nb[k]; ++j) {
                    const double t = T[(k * NPE + a) * maxnb + j];
                    if (fem_nonzero(t)) up = fma(t, u[f * nu + bases[k * maxnb + j]], up);
                }
                for (int i = 0; i < D; ++i) grad[f][i] = fma(g[i], up, grad[f][i]);
            }
        }
        double Ek = E[k];
        if (rho) {
            double r = 0.0;
            for (int a = 0; a < NPE; ++a) r = fma(N[a], rho[k * NPE + a], r);
            Ek *= beta == 3.0 ? r * r * r : pow(r, beta);
        }
        const double mu = Ek / (2.0 * (1.0 + nu_p));
        const double lam = model == FEM_GPU_MODEL_PLANE_STRESS ? Ek * nu_p / (1.0 - nu_p * nu_p)
                                                               : Ek * nu_p / ((1.0 + nu_p) * (1.0 - 2.0 * nu_p));
        double* o = out + k * ncomp;
        if (D == 3) {
            const double tr = grad[0][0] + grad[1][1] + grad[2][2];
            for (int i = 0; i < 3; ++i) o[i] = lam * tr + 2.0 * mu * grad[i][i];
            o[3] = mu * (grad[1][2] + grad[2][1]);
            o[4] = mu * (grad[0][2] + grad[2][0]);
            o[5] = mu * (grad[0][1] + grad[1][0]);
        } else {
            const double tr = grad[0][0] + grad[1][1];
            o[0] = lam * tr + 2.0 * mu * grad[0][0];
            o[1] = lam * tr + 2.0 * mu * grad[1][1];
            if (model == FEM_GPU_MODEL_PLANE_STRESS) {
                o[2] = mu * (grad[0][1] + grad[1][0]);
            } else {
                o[2] = lam * tr;
                o[3] = mu * (grad[0][1] + grad[1][0]);
            }
        }
    }
}

}  // namespace fem_flux

extern "C" {

fem_gpu_status fem_gpu_element_flux(fem_gpu_ctx* c, int32_t set, int64_t count, const int64_t* eq, const double* xi,
                                    const double* u, double* flux, int32_t* ncomp, uint32_t flags) {
    if (!c || count < 0 || (count > 0 && (!eq || !xi || !u || !flux))) return FEM_GPU_BAD_ARG;
    if (!c->dev_final) return FEM_GPU_NOT_FINALIZED;
    if (set < 0 || set >= (int32_t)c->sets.size() || c->sets[set].kind != 0)
        return fail(c, FEM_GPU_BAD_ARG, "element_flux: not a bulk set");
    const SetData& s = c->sets[set];
    const int D = c->dim, NPE = c->npe, model = s.bulk.model_type;
    const int nc = D == 3 ? 6 : (model == FEM_GPU_MODEL_PLANE_STRESS ? 3 : 4);
    if (ncomp) *ncomp = nc;
    if (count == 0) return FEM_GPU_OK;
    const int maxnb = s.maxnb;
    std::vector<double> xe((size_t)count * NPE * D), T((size_t)count * NPE * maxnb), E(count), rho;
    std::vector<int32_t> bs((size_t)count * maxnb), nbv(count);
    if (!s.rhoe.empty()) rho.resize((size_t)count * NPE);
    for (int64_t k = 0; k < count; ++k) {
        const int64_t e = eq[k];
        if (e < 0 || e >= s.neq) return fail(c, FEM_GPU_OOB_INDEX, "element_flux: equation object index");
        std::copy_n(s.xe.data() + e * NPE * D, NPE * D, xe.data() + k * NPE * D);
        std::copy_n(s.T.data() + e * NPE * maxnb, NPE * maxnb, T.data() + k * NPE * maxnb);
        std::copy_n(s.bases.data() + e * maxnb, maxnb, bs.data() + k * maxnb);
        nbv[k] = s.nb[e];
        // the stiffness modulus carries the Thickness property; the stress does not
        E[k] = s.E[e] / s.bulk_thickness;
        if (!rho.empty()) std::copy_n(s.rhoe.data() + e * NPE, NPE, rho.data() + k * NPE);
    }
    const bool host = flags & FEM_GPU_HOST_BUFFERS;
    const int64_t nad = c->num_used * c->dim;
    cudaStream_t sm = stream_of(c);
    Staged su, so, sxi, sxe, sT, sE, sb, snb, sr;
    fem_gpu_status st;
    if ((st = stage_in(c, u, nad * sizeof(double), host, su)) != FEM_GPU_OK) return st;
    if ((st = stage_out_alloc(c, flux, (size_t)count * nc * sizeof(double), host, so)) != FEM_GPU_OK) return st;
    if ((st = stage_in(c, xi, (size_t)count * D * sizeof(double), true, sxi)) != FEM_GPU_OK) return st;
    if ((st = stage_in(c, xe.data(), xe.size() * sizeof(double), true, sxe)) != FEM_GPU_OK) return st;
    if ((st = stage_in(c, T.data(), T.size() * sizeof(double), true, sT)) != FEM_GPU_OK) return st;
    if ((st = stage_in(c, E.data(), E.size() * sizeof(double), true, sE)) != FEM_GPU_OK) return st;
    if ((st = stage_in(c, bs.data(), bs.size() * sizeof(int32_t), true, sb)) != FEM_GPU_OK) return st;
    if ((st = stage_in(c, nbv.data(), nbv.size() * sizeof(int32_t), true, snb)) != FEM_GPU_OK) return st;
    if (!rho.empty() && (st = stage_in(c, rho.data(), rho.size() * sizeof(double), true, sr)) != FEM_GPU_OK)
        return st;
    const unsigned blocks = (unsigned)std::min<int64_t>((count + 127) / 128, (int64_t)sm_count() * 8);
    const double beta = s.bulk.density_exponent;
    if (D == 2)
        fem_flux::flux_kernel<2><<<blocks, 128, 0, sm>>>(count, maxnb, model, s.bulk.poisson_ratio, (double*)sxe.dev,
                                                         (double*)sT.dev, (int32_t*)sb.dev, (int32_t*)snb.dev,
                                                         (double*)sE.dev, (double*)sr.dev, beta, (double*)sxi.dev,
                                                         (double*)su.dev, c->num_used, nc, (double*)so.dev);
    else
        fem_flux::flux_kernel<3><<<blocks, 128, 0, sm>>>(count, maxnb, model, s.bulk.poisson_ratio, (double*)sxe.dev,
                                                         (double*)sT.dev, (int32_t*)sb.dev, (int32_t*)snb.dev,
                                                         (double*)sE.dev, (double*)sr.dev, beta, (double*)sxi.dev,
                                                         (double*)su.dev, c->num_used, nc, (double*)so.dev);
    ++c->launches;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && host)
        e = cudaMemcpyAsync(flux, so.dev, (size_t)count * nc * sizeof(double), cudaMemcpyDeviceToHost, sm);
    for (Staged* p : {&su, &so, &sxi, &sxe, &sT, &sE, &sb, &snb, &sr}) release(c, *p);
    if (e == cudaSuccess) e = cudaStreamSynchronize(sm);
    return e == cudaSuccess ? FEM_GPU_OK : cuda_fail(c, e, "element flux");
}

fem_gpu_status fem_gpu_check_status(fem_gpu_ctx* c) {
    if (!c) return FEM_GPU_BAD_ARG;
    if (!c->dev_final) return FEM_GPU_NOT_FINALIZED;
    fem_gpu_status st = read_status(c);
    cudaMemsetAsync(c->d_status.p, 0, sizeof(int), stream_of(c));
    return st;
}

fem_gpu_status fem_gpu_apply(fem_gpu_ctx* c, const double* x, double* y, uint32_t flags) {
    if (!c || !x || !y) return FEM_GPU_BAD_ARG;
    if (!c->dev_final) return FEM_GPU_NOT_FINALIZED;
    const bool host = flags & FEM_GPU_HOST_BUFFERS;
    const int64_t nad = c->num_used * c->dim;
    Staged sx, sy;
    fem_gpu_status st;
    if ((st = stage_in(c, x, nad * sizeof(double), host, sx)) != FEM_GPU_OK) return st;
    if ((st = stage_out_alloc(c, y, nad * sizeof(double), host, sy)) != FEM_GPU_OK) return st;
    cudaStream_t sm = stream_of(c);
    if (!(flags & FEM_GPU_ACCUMULATE)) cudaMemsetAsync(sy.dev, 0, nad * sizeof(double), sm);
    for (int k = 0; k < (int)c->sets.size() && st == FEM_GPU_OK; ++k) {
        SetData& s = c->sets[k];
        if (s.neq == 0) continue;
        if (s.kind != 0) {
            st = fail(c, FEM_GPU_UNSUPPORTED, "matrix-free apply covers bulk sets only");
            break;
        }
        st = launch_bulk(c, k, MODE_APPLY, 0, s.neq, nullptr, nullptr, nullptr, nullptr, nullptr, 0,
                         (const double*)sx.dev, (double*)sy.dev);
    }
    if (st == FEM_GPU_OK && host) {
        cudaError_t e = cudaMemcpyAsync(y, sy.dev, nad * sizeof(double), cudaMemcpyDeviceToHost, sm);
        if (e == cudaSuccess) e = cudaStreamSynchronize(sm);
        if (e != cudaSuccess) st = cuda_fail(c, e, "apply copy back");
    }
    release(c, sx);
    release(c, sy);
    return st;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// autotuner: per bulk set, time every kernel variant on the set's own elements
// (assembly into a scratch CSR) and keep the fastest.
extern "C" {

fem_gpu_status fem_gpu_autotune(fem_gpu_ctx* c, int64_t max_elements) {
    if (!c) return FEM_GPU_BAD_ARG;
    if (!c->dev_final) return FEM_GPU_NOT_FINALIZED;
    cudaStream_t sm = stream_of(c);
    const int64_t nad = c->num_used * c->dim;
    double *vals = nullptr, *rhs = nullptr, *u = nullptr;
    cudaError_t e = cudaMallocAsync(&vals, std::max<int64_t>(c->nnz, 1) * sizeof(double), sm);
    if (e == cudaSuccess) e = cudaMallocAsync(&rhs, nad * sizeof(double), sm);
    if (e == cudaSuccess) e = cudaMallocAsync(&u, nad * sizeof(double), sm);
    if (e != cudaSuccess) return cuda_fail(c, e, "autotune scratch");
    cudaMemsetAsync(vals, 0, c->nnz * sizeof(double), sm);
    cudaMemsetAsync(rhs, 0, nad * sizeof(double), sm);
    cudaMemsetAsync(u, 0, nad * sizeof(double), sm);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fem_gpu_status st = FEM_GPU_OK;
    for (int k = 0; k < (int)c->sets.size() && st == FEM_GPU_OK; ++k) {
        SetData& s = c->sets[k];
        if (s.kind != 0 || !s.ig_off.empty() || s.neq == 0) continue;
        const int64_t n = max_elements > 0 ? std::min(max_elements, s.neq) : s.neq;
        double best = 1e30;
        int bestv = s.variant;
        for (int v = 0; v < NUM_VARIANTS && st == FEM_GPU_OK; ++v) {
            // a variant that does not fit (shared memory / registers) is skipped
            st = launch_bulk(c, k, MODE_ASSEMBLE, 0, n, u, vals, rhs, nullptr, nullptr, 0, nullptr, nullptr, v);
            if (st == FEM_GPU_UNSUPPORTED) {
                st = FEM_GPU_OK;
                cudaGetLastError();
                continue;
            }
            if (st != FEM_GPU_OK) break;
            cudaEventRecord(e0, sm);
            const int reps = 3;
            for (int r = 0; r < reps && st == FEM_GPU_OK; ++r)
                st = launch_bulk(c, k, MODE_ASSEMBLE, 0, n, u, vals, rhs, nullptr, nullptr, 0, nullptr, nullptr, v);
            cudaEventRecord(e1, sm);
            e = cudaEventSynchronize(e1);
            if (e != cudaSuccess) {
                st = cuda_fail(c, e, "autotune run");
                break;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms / reps < best) {
                best = ms / reps;
                bestv = v;
            }
        }
        s.variant = bestv;
        s.tuned_ms = best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(vals, sm);
    cudaFreeAsync(rhs, sm);
    cudaFreeAsync(u, sm);
    cudaStreamSynchronize(sm);
    return st;
}

fem_gpu_status fem_gpu_get_variant(const fem_gpu_ctx* c, int32_t set, int32_t* variant, double* tuned_ms,
                                   const char** name) {
    if (!c || set < 0 || set >= (int32_t)c->sets.size()) return FEM_GPU_BAD_ARG;
    const SetData& s = c->sets[set];
    if (variant) *variant = s.variant;
    if (tuned_ms) *tuned_ms = s.tuned_ms;
    if (name) *name = (s.kind == 0 && s.variant >= 0 && s.variant < NUM_VARIANTS) ? kVariantNames[s.variant] : "";
    return FEM_GPU_OK;
}

fem_gpu_status fem_gpu_set_variant(fem_gpu_ctx* c, int32_t set, int32_t variant) {
    if (!c || set < 0 || set >= (int32_t)c->sets.size() || variant < 0 || variant >= NUM_VARIANTS)
        return FEM_GPU_BAD_ARG;
    c->sets[set].variant = variant;
    return FEM_GPU_OK;
}

}  // extern "C"
