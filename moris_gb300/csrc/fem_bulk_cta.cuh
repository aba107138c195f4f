// fem_bulk_cta.cuh -- bulk elasticity with one element per CTA.
//
// The element quantities of the warp-per-element kernel in fem_device.cu (Gram
// matrix of the physical gradients, isotropic K from it, sparse T^T K T, CSR
// scatter), with the phases of one element spread over NW warps and several
// CTAs per SM, so that the FP64 pipe sees enough independent warps to cover its
// latency.  The T^T K T stage works on the element adofs ordered by the nonzero
// count of their T column: every upper-triangle entry contracts over the
// sparser of its two columns, and entries of one count are contiguous, so the
// warps run uniform trip counts.  Elements come from a device counter, in order.
// Shared memory per CTA is sized so that 8 CTAs fit on one SM for the hex8 /
// quadratic B-spline element (the extraction T is staged in a region that the
// K T product overwrites once T is no longer needed).
//
// RECT (axis-aligned brick cells, the reference's CellShape::RECTANGULAR with
// its diagonal Jacobian): a trilinear map whose Jacobian is diagonal at every
// Gauss point is affine, so J is constant over the cell and the Gram matrix is
//   A[(i,a),(j,b)] = detJ / (J_ii J_jj) * G0[(i,a),(j,b)],
//   G0 = sum_q w_q dN_a/dxi_i dN_b/dxi_j          (per-rule table, p.g0),
// which replaces 27 FMAs per Gram entry by one multiply.  J_ii is half the
// edge length of the cell along axis i.
//
// MODE_APPLY (matrix-free Jacobian-vector product) forms the pdof K the same
// way and scatters T^T (K T x) without the K T / T^T K T stages.
//
// Uniform quadratic B-splines (3D HEX8, 27 bases): at the cell corners every
// basis is the tensor product of the 1D values (1/2, 1/2, 0) / (0, 1/2, 1/2),
// so T = 1/8 P with P the 0/1 pattern of nodes (x left/right) x (y) x (z).
// When an element's T is exactly that (checked per element: every nonzero
// 1/8, each column a tensor-product node set, all 27 present), K is formed
// as K/64 (exact: a power of two), K T / 8 = (K/64) P is summed axis by axis
// (8 node values -> 27 bases in three 2 -> 3 stages of additions) and
// T^T K T = P^T ((K/64) P) is a plain sum over each column's nodes: count - 1
// additions per entry instead of count FMAs.  Other elements take the general
// path.
#pragma once

// E0-relative SIMP factor rho(x_q)^beta with rho interpolated from the nodal
// densities by the IP-cell shape functions at Gauss point q
__device__ __forceinline__ double fem_density_power(const BulkArgs& p, const double* rho_nodes, int q) {
    constexpr int kMaxNodes = 8;
    double r = 0.0;
    const int npe = p.npe;
    for (int a = 0; a < npe && a < kMaxNodes; ++a) r = fma(__ldg(p.nq + q * npe + a), rho_nodes[a], r);
    return p.beta == 3.0 ? r * r * r : pow(r, p.beta);
}

// (included inside namespace fem of fem_device.cu)

// sum_k w[k] * base[tn[k] * stride] over the nonzeros of one T column; the
// counts of tensor-product B-spline extraction (1, 2, 4, 8) get fully unrolled
// bodies, so a warp of one count issues no predicated-off FMAs and all loads
// of the column up front
template <int N>
__device__ __forceinline__ double fem_tdot_n(const double* w, const uint8_t* tn, const double* base, int stride) {
    double v = 0.0;
#pragma unroll
    for (int k = 0; k < N; ++k) v = fma(w[k], base[tn[k] * stride], v);
    return v;
}
// sum of base[tn[k] * stride] over one column's nonzeros (columns whose
// weights are all equal, the weight folded elsewhere): count - 1 additions
template <int N>
__device__ __forceinline__ double fem_tsum_n(const uint8_t* tn, const double* base, int stride) {
    double v = base[tn[0] * stride];
#pragma unroll
    for (int k = 1; k < N; ++k) v += base[tn[k] * stride];
    return v;
}
__device__ __forceinline__ double fem_tsum(int cnt, const uint8_t* tn, const double* base, int stride) {
    switch (cnt) {
        case 1: return fem_tsum_n<1>(tn, base, stride);
        case 2: return fem_tsum_n<2>(tn, base, stride);
        case 4: return fem_tsum_n<4>(tn, base, stride);
        case 8: return fem_tsum_n<8>(tn, base, stride);
        default: {
            double v = 0.0;
            for (int k = 0; k < cnt; ++k) v += base[tn[k] * stride];
            return v;
        }
    }
}
__device__ __forceinline__ double fem_tdot(int cnt, const double* w, const uint8_t* tn, const double* base,
                                           int stride) {
    switch (cnt) {
        case 1: return fem_tdot_n<1>(w, tn, base, stride);
        case 2: return fem_tdot_n<2>(w, tn, base, stride);
        case 4: return fem_tdot_n<4>(w, tn, base, stride);
        case 8: return fem_tdot_n<8>(w, tn, base, stride);
        default: {
            double v = 0.0;
            for (int k = 0; k < cnt; ++k) v = fma(w[k], base[tn[k] * stride], v);
            return v;
        }
    }
}

template <int D, int NPE, int NGP, int NB, bool RECT>
struct CtaLayout {
    static constexpr int NPD = D * NPE;
    static constexpr int NAD = D * NB;
    static constexpr int NSYM = NPD * (NPD + 1) / 2;
    static constexpr int NTRI = NAD * (NAD + 1) / 2;       // upper triangle of the element matrix
    static constexpr int NKT = NB * D * D * NPE;           // K T entries (all field blocks)
    // R1 holds, until phase 3, the Gauss-point gradients g and w*g (general
    // cells) or the density Gram matrix A (rectangular cells, where g is not
    // formed), then the staged T; from phase 4 on, K T
    static constexpr bool A_IN_R1 = RECT && NPD * NPD <= 2 * NGP * NPD;
    static constexpr int GPR = A_IN_R1 ? NPD * NPD : 2 * NGP * NPD;
    static constexpr int R1 = (GPR + NPE * NB > NPD * NAD) ? GPR + NPE * NB : NPD * NAD;
    static constexpr int oX = 0;
    static constexpr int oR1 = oX + NPE * D;
    static constexpr int oT = oR1 + GPR;                           // inside R1
    static constexpr int oA = A_IN_R1 ? oR1 : oR1 + R1;
    static constexpr int oK = A_IN_R1 ? oR1 + R1 : oA + NPD * NPD;
    static constexpr int oTW = oK + NPD * NPD;                     // [slot][k] T weights in count order
    static constexpr int oU = oTW + NB * NPE;
    static constexpr int oUA = oU + NPD;
    static constexpr int oRP = oUA + NAD;
    static constexpr int oW = oRP + NPD;
    static constexpr int oCJ = oW + NGP;                           // RECT: detJ/(J_ii J_jj), i<=j
    static constexpr int oRHO = oCJ + 8;                           // nodal densities (SIMP sets)
    static constexpr int ND = oRHO + NPE;
    // ints: bases, CSR row starts [f][basis], row lengths, and the CSR row
    // base of count-ordered adof x for column field g
    static constexpr int iB = 0, iRB = iB + NB, iUL = iRB + NAD, iRG = iUL + NB, NI = iRG + NAD * D;
    // bytes: T row lists [slot][k], nonzero counts by basis / by slot, the
    // count order and its inverse, then the count-ordered scatter slots
    // [slot][slot] (u16)
    static constexpr int bTN = 0, bTC = bTN + NB * NPE, bTCP = bTC + NB, bCP = bTCP + NB, bCPI = bCP + NB;
    static constexpr int bS = ((bCPI + NB + 1) / 2) * 2;
    static constexpr int bNJ = bS + 2 * NB * NB;  // tensor-product elements: slot of natural basis code
    static constexpr int NBYTE = bNJ + NB;
    // uniform quadratic B-spline elements (sum-factorised K T)
    static constexpr bool kTQ2 = D == 3 && NPE == 8 && NB == 27;
    static constexpr size_t kBytes = ((size_t)ND * 8 + (size_t)NI * 4 + (size_t)NBYTE + 15) / 16 * 16;
    static_assert(NB <= 32 && D <= 3, "table packing: 5-bit slots, 2-bit fields");
    static_assert((D - 1) * NPE * NPD + D * NPE <= 1024 && NPD * NAD <= 8192, "K T table packing");
};

// Item tables of the K T and T^T K T phases (built on the host per basis width
// when a bulk set is uploaded, fem_device.cu): they replace per-entry index
// arithmetic by one load.
//   ktab[t]: slot | kbase << 6 | ktdst << 16, items slot-major so that the
//            lanes of a warp share one column (one trip count)
//            kbase = g*NPE*NPD + f*NPE + a, ktdst = (f*NPE + a)*NAD + slot*D + g
//   tri[t]:  sr | f << 5 | sc << 7 | g << 12 for the upper-triangle entry t
//            (row x = sr*D + f, column y = sc*D + g, x <= y) in row order

template <int D, int NPE, int NGP, int NB, bool RECT, int NW>
__global__ void __launch_bounds__(32 * NW) bulk_cta_kernel(BulkArgs p, int mode) {
    using L = CtaLayout<D, NPE, NGP, NB, RECT>;
    constexpr int NPD = L::NPD, NAD = L::NAD, NSYM = L::NSYM, NT = 32 * NW;
    extern __shared__ __align__(16) unsigned char smem[];
    double* sd = reinterpret_cast<double*>(smem);
    int32_t* si = reinterpret_cast<int32_t*>(sd + L::ND);
    unsigned char* sb = reinterpret_cast<unsigned char*>(si + L::NI);
    double* X = sd + L::oX;
    double* g = sd + L::oR1;
    double* wg = g + NGP * NPD;
    double* KT = sd + L::oR1;
    double* T = sd + L::oT;
    double* A = sd + L::oA;
    double* K = sd + L::oK;
    double* TW = sd + L::oTW;
    double* U = sd + L::oU;
    double* UA = sd + L::oUA;
    double* RP = sd + L::oRP;
    double* WS = sd + L::oW;
    double* CJ = sd + L::oCJ;
    double* RHO = sd + L::oRHO;
    int32_t* B = si + L::iB;
    int32_t* RB = si + L::iRB;
    int32_t* UL = si + L::iUL;
    int32_t* RG = si + L::iRG;
    uint8_t* TN = sb + L::bTN;
    uint8_t* TC = sb + L::bTC;
    uint8_t* TCP = sb + L::bTCP;
    uint8_t* CP = sb + L::bCP;
    uint8_t* CPI = sb + L::bCPI;
    uint16_t* S = reinterpret_cast<uint16_t*>(sb + L::bS);
    uint8_t* NJ = sb + L::bNJ;
    const int tid = threadIdx.x;
    const uint32_t* pairs = p.pairs;
    const bool assemble = mode == MODE_ASSEMBLE, apply = mode == MODE_APPLY;
    const bool want_r = (assemble && p.rhs) || (mode == MODE_ELEMENT && p.Rout);
    const bool want_k = (assemble && p.vals) || (mode == MODE_ELEMENT && p.Kout);
    const bool need_u = want_r || apply;
    const double* uin = apply ? p.x : p.u;
    const bool scatter_k = assemble && p.vals;
    constexpr int NSR = (NB * NB + NT - 1) / NT;  // scatter slots held per thread

    // elements are taken in order from a device counter (after each CTA's
    // first): CTAs cannot drift apart, so the CSR rows being scattered form one
    // compact front and most of the scatter stays in L2 even when the matrix is
    // many times larger than L2
    __shared__ int64_t s_next;
    __shared__ int s_tq2;
    for (int64_t e = blockIdx.x; e < p.ne; e = s_next) {
        const int nb = p.nb[e];
        const double E = p.E[e];
        // ---- phase 0: loads --------------------------------------------------
        for (int i = tid; i < NPE * D; i += NT) X[i] = p.xe[e * (NPE * D) + i];
        for (int i = tid; i < NPE * NB; i += NT) T[i] = p.T[e * (NPE * NB) + i];
        for (int i = tid; i < NB; i += NT) B[i] = p.bases[e * NB + i];
        if (p.rho)
            for (int i = tid; i < NPE; i += NT) RHO[i] = p.rho[e * NPE + i];
        // scatter slots [basis][basis] into registers now; they are stored in
        // count order once the order is known
        uint16_t sreg[NSR];
        if (scatter_k) {
            const uint16_t* sg = p.sidx + e * (NB * NB);
#pragma unroll
            for (int m = 0; m < NSR; ++m) {
                const int k = tid + m * NT;
                sreg[m] = k < NB * NB ? sg[k] : 0;
            }
        }
        __syncthreads();
        // ---- phase 1: adof values, T column counts, Gauss-point geometry ---------
        for (int r = tid; r < NAD; r += NT) {
            const int f = r / NB, i = r - f * NB;
            UA[r] = (uin && i < nb) ? uin[f * p.nu + B[i]] : 0.0;
            if (scatter_k) RB[r] = i < nb ? __ldg(p.rowptr + f * p.nu + B[i]) : 0;
        }
        if (scatter_k)
            for (int i = tid; i < NB; i += NT) UL[i] = i < nb ? __ldg(p.ulen + B[i]) : 0;
        // nonzero lists of the T rows (nodes), for the nodal values: weights in
        // the K region and basis indices + counts in the scatter-slot region,
        // both unused until phase 3; one warp per node, the lanes over the
        // bases, positions from a ballot (ascending basis order)
        double* NZW = K;
        uint8_t* NZJ = reinterpret_cast<uint8_t*>(S);
        static_assert(NPE * NB <= NPD * NPD && NPE * NB + NPE <= 2 * NB * NB, "node lists fit their regions");
        if (need_u) {
            const int lane = tid & 31;
            for (int a = tid >> 5; a < NPE; a += NW) {
                const double t = lane < NB ? T[a * NB + lane] : 0.0;
                const bool nz = lane < nb && fem_nonzero(t);
                const unsigned m = __ballot_sync(0xffffffffu, nz);
                if (nz) {
                    const int pos = __popc(m & ((1u << lane) - 1u));
                    NZJ[a * NB + pos] = (uint8_t)lane;
                    NZW[a * NB + pos] = t;
                }
                if (lane == 0) NZJ[NPE * NB + a] = (uint8_t)__popc(m);
            }
        }
        for (int i = tid; i < NB; i += NT) {
            int cnt = 0;
            if (i < nb)
                for (int a = 0; a < NPE; ++a) cnt += fem_nonzero(T[a * NB + i]);
            TC[i] = (uint8_t)cnt;
        }
        if (RECT) {
            // constant Jacobian of the brick: J_ii = half the edge length along
            // axis i (node 0 is at xi = (-1,...), nodes 1, 3, 4 are its
            // neighbours along xi_0, xi_1, xi_2 in the QUAD4 / HEX8 order), which
            // is the diagonal of sum_a dN_a/dxi x_a at any point of the cell;
            // CJ[i<=j] = detJ / (J_ii J_jj): off-diagonal factors are the
            // remaining J entry (3D) or 1 (2D), diagonal ones one division each
            if (tid < D) {
                constexpr int kNext[3] = {1, 3, 4};
                double jd[D];
#pragma unroll
                for (int i = 0; i < D; ++i) jd[i] = 0.5 * (X[kNext[i] * D + i] - X[i]);
                const double detJ = (D == 3) ? jd[1] * jd[0] * jd[2] : jd[0] * jd[1];
                // integration points with detJ below -1e-6 are skipped by the
                // reference element loop (cl_FEM_Element_Bulk.cpp:164)
                const bool skip = detJ < -1.0e-6;
                const int i = tid;
                double other = 1.0;  // product of the other diagonal entries
                for (int k = 0; k < D; ++k)
                    if (k != i) other *= jd[k];
                CJ[i * D - i * (i - 1) / 2] = skip ? 0.0 : other / jd[i];
                if (D == 3 && i == 0) {
                    CJ[1] = skip ? 0.0 : jd[2];   // (0,1)
                    CJ[2] = skip ? 0.0 : jd[1];   // (0,2)
                    CJ[4] = skip ? 0.0 : jd[0];   // (1,2)
                }
                if (D == 2 && i == 0) CJ[1] = skip ? 0.0 : 1.0;
            }
            // SIMP material: w_q E0 rho(x_q)^beta (the Jacobian factors stay in CJ)
            if (p.rho)
                for (int q = tid; q < NGP; q += NT) WS[q] = __ldg(p.w + q) * E * fem_density_power(p, RHO, q);
        } else
        for (int q = tid; q < NGP; q += NT) {
            const double* dn = p.dn + q * D * NPE;
            double detJ, Ji[D][D];
            if (RECT) {
                double jd[D];
                for (int i = 0; i < D; ++i) {
                    double s = 0.0;
                    for (int a = 0; a < NPE; ++a) s = fma(__ldg(dn + i * NPE + a), X[a * D + i], s);
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
                        for (int a = 0; a < NPE; ++a) s = fma(__ldg(dn + i * NPE + a), X[a * D + j], s);
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
            double ws = (detJ < -1.0e-6) ? 0.0 : __ldg(p.w + q) * detJ;
            if (p.rho) ws *= E * fem_density_power(p, RHO, q);
            WS[q] = ws;
            for (int i = 0; i < D; ++i)
                for (int a = 0; a < NPE; ++a) {
                    double s;
                    if (RECT) {
                        s = Ji[i][i] * __ldg(dn + i * NPE + a);
                    } else {
                        s = 0.0;
                        for (int k = 0; k < D; ++k) s = fma(Ji[i][k], __ldg(dn + k * NPE + a), s);
                    }
                    g[q * NPD + i * NPE + a] = s;
                    wg[q * NPD + i * NPE + a] = ws * s;
                }
        }
        __syncthreads();
        // ---- phase 2: count order, pdof values, (general cells) Gram matrix ----
        // CP[slot] = basis, stable in basis order; padding bases (count 0) first
        for (int j = tid; j < NB; j += NT) {
            const int cj = TC[j];
            int rank = 0;
            for (int k = 0; k < NB; ++k) {
                const int ck = TC[k];
                rank += (ck < cj) || (ck == cj && k < j);
            }
            CP[rank] = (uint8_t)j;
            CPI[j] = (uint8_t)rank;
        }
        if (L::kTQ2 && want_k && (tid >> 5) == 1) {
            // tensor-product check of T (second warp): lane j finds the nodes of
            // column j, their codes along x, y, z (0: left node only, 1: both,
            // 2: right only) and checks the set and the weights
            const int j = tid & 31;
            bool ok = true;
            unsigned code = 0u;
            if (j < NB) {
                unsigned mask = 0u;
                for (int a = 0; a < NPE; ++a) {
                    const long long tb = __double_as_longlong(T[a * NB + j]);
                    if (tb != 0ll) {
                        mask |= 1u << a;
                        ok &= tb == 0x3FC0000000000000ll;  // 0.125
                    }
                }
                // HEX8 nodes: x left {0,3,4,7}, right {1,2,5,6}; y left {0,1,4,5},
                // right {2,3,6,7}; z left {0..3}, right {4..7}
                const unsigned L3[3] = {0x99u, 0x33u, 0x0Fu}, R3[3] = {0x66u, 0xCCu, 0xF0u};
                unsigned expect = 0xFFu;
                int nat = 0, mul = 1;
                for (int d = 0; d < 3; ++d) {
                    const int c = (mask & L3[d]) ? ((mask & R3[d]) ? 1 : 0) : 2;
                    expect &= c == 0 ? L3[d] : c == 2 ? R3[d] : 0xFFu;
                    nat += c * mul;
                    mul *= 3;
                }
                ok &= j < nb && mask != 0u && mask == expect;
                code = 1u << nat;
                if (ok) NJ[nat] = (uint8_t)j;
            }
            const unsigned all = __reduce_or_sync(0xffffffffu, code);
            const bool allok = __all_sync(0xffffffffu, ok);
            if (j == 0) s_tq2 = allok && all == (1u << 27) - 1u;
        }
        if (need_u)  // on the last warp (the first one computes the count order)
            for (int r = tid - (NT - 32); r >= 0 && r < NPD; r += 32) {
                const int f = r / NPE, a = r - f * NPE, cnt = NZJ[NPE * NB + a];
                double s = 0.0;
                for (int k = 0; k < cnt; ++k) s = fma(NZW[a * NB + k], UA[f * NB + NZJ[a * NB + k]], s);
                U[r] = s;
            }
        if (RECT && p.rho) {
            // density-weighted reference Gram matrix of this element
            if (!L::A_IN_R1) {
                // the weighted gradients w_q E(x_q) dN_r(x_q) once per point, in the
                // region of the general-cell gradients (unused by bricks): one FMA
                // per Gram term instead of a multiply and an FMA
                double* WDN = g;
                for (int i = tid; i < NGP * NPD; i += NT) WDN[i] = WS[i / NPD] * __ldg(p.dn + i);
                __syncthreads();
                for (int k = tid; k < NSYM; k += NT) {
                    const uint32_t pc = __ldg(pairs + k);
                    const int r = pc >> 16, c = pc & 0xffff;
                    double s = 0.0;
#pragma unroll 4
                    for (int q = 0; q < NGP; ++q) s = fma(WDN[q * NPD + r], __ldg(p.dn + q * NPD + c), s);
                    A[r * NPD + c] = s;
                    A[c * NPD + r] = s;
                }
            } else {
                for (int k = tid; k < NSYM; k += NT) {
                    const uint32_t pc = __ldg(pairs + k);
                    const int r = pc >> 16, c = pc & 0xffff;
                    double s = 0.0;
                    for (int q = 0; q < NGP; ++q)
                        s = fma(WS[q] * __ldg(p.dn + q * NPD + r), __ldg(p.dn + q * NPD + c), s);
                    A[r * NPD + c] = s;
                    A[c * NPD + r] = s;
                }
            }
        }
        if (!RECT) {
            for (int k = tid; k < NSYM; k += NT) {
                const uint32_t pc = __ldg(pairs + k);
                const int r = pc >> 16, c = pc & 0xffff;
                double s0 = 0.0, s1 = 0.0, s2 = 0.0;
                int q = 0;
                for (; q + 2 < NGP; q += 3) {
                    s0 = fma(wg[q * NPD + r], g[q * NPD + c], s0);
                    s1 = fma(wg[(q + 1) * NPD + r], g[(q + 1) * NPD + c], s1);
                    s2 = fma(wg[(q + 2) * NPD + r], g[(q + 2) * NPD + c], s2);
                }
                for (; q < NGP; ++q) s0 = fma(wg[q * NPD + r], g[q * NPD + c], s0);
                const double s = s0 + s1 + s2;
                A[r * NPD + c] = s;
                A[c * NPD + r] = s;
            }
        }
        __syncthreads();
        // ---- phase 3: isotropic stiffness in pdof space, count-ordered data -------
        const bool tq2 = L::kTQ2 && NW >= 2 && want_k && s_tq2;  // the check runs on the second warp
        {
            // with a density field E(x_q) is already inside the Gram sums;
            // tensor-product elements form K / 64 (T^T K T = P^T (K / 64) P)
            const double escale = (p.rho ? 1.0 : E) * (tq2 ? 1.0 / 64.0 : 1.0);
            const double lam = escale * p.lam_c, mu = escale * p.mu_c;
            const double* G = p.rho ? A : p.g0;
            for (int k = tid; k < NSYM; k += NT) {
                const uint32_t pc = __ldg(pairs + k);
                const int r = pc >> 16, c = pc & 0xffff;
                const int f = r / NPE, a = r - f * NPE, gg = c / NPE, b = c - gg * NPE;
                double v;
                if (RECT) {
                    // A = c_ij G: c_fg (lam G[(f,a),(g,b)] + mu G[(g,a),(f,b)]) + mu tr
                    const int lo = f < gg ? f : gg, hi = f < gg ? gg : f;
                    const double cfg = CJ[lo * D - lo * (lo - 1) / 2 + (hi - lo)];
                    v = cfg * (lam * G[r * NPD + c] + mu * G[(gg * NPE + a) * NPD + f * NPE + b]);
                    if (f == gg) {
                        double tr = 0.0;
                        for (int kk = 0; kk < D; ++kk)
                            tr = fma(CJ[kk * D - kk * (kk - 1) / 2], G[(kk * NPE + a) * NPD + kk * NPE + b], tr);
                        v = fma(mu, tr, v);
                    }
                } else {
                    v = lam * A[r * NPD + c] + mu * A[(gg * NPE + a) * NPD + f * NPE + b];
                    if (f == gg) {
                        double tr = 0.0;
                        for (int kk = 0; kk < D; ++kk) tr += A[(kk * NPE + a) * NPD + kk * NPE + b];
                        v = fma(mu, tr, v);
                    }
                }
                K[r * NPD + c] = v;
                K[c * NPD + r] = v;
            }
        }
        // count-ordered element data: T lists by slot, CSR row bases and the
        // scatter slots of the count-ordered adofs
        for (int sl = tid; sl < NB; sl += NT) {
            const int j = CP[sl];
            int cnt = 0;
            for (int a = 0; a < NPE; ++a) {
                const double t = T[a * NB + j];
                if (fem_nonzero(t)) {
                    TN[sl * NPE + cnt] = (uint8_t)a;
                    TW[sl * NPE + cnt] = t;
                    ++cnt;
                }
            }
            TCP[sl] = (uint8_t)cnt;
        }
        // natural basis code -> count-ordered slot (in place)
        if (tq2 && tid < 27) NJ[tid] = CPI[NJ[tid]];
        if (scatter_k) {
            for (int x = tid; x < NAD; x += NT) {
                const int sl = x / D, f = x - sl * D, i = CP[sl];
                const int32_t rb = RB[f * NB + i], ul = UL[i];
                for (int gg = 0; gg < D; ++gg) RG[x * D + gg] = rb + gg * ul;
            }
#pragma unroll
            for (int m = 0; m < NSR; ++m) {
                const int k = tid + m * NT;
                if (k < NB * NB) {
                    const int i = k / NB, j = k - i * NB;
                    S[CPI[i] * NB + CPI[j]] = sreg[m];
                }
            }
        }
        __syncthreads();
        // ---- phase 4: pdof residual and K T ----------------------------------------
        if (need_u) {
            // K U with four lanes per row and a shuffle sum: dot chains a quarter
            // as long, spread over several warps (4 NPD is a multiple of 32, so a
            // warp takes part whole)
            static_assert((4 * NPD) % 32 == 0, "K U lanes fill whole warps");
            for (int t = tid; t < 4 * NPD; t += NT) {
                const int r = t >> 2, q = t & 3;
                double s = 0.0;
                for (int c = q; c < NPD; c += 4) s = fma(K[r * NPD + c], U[c], s);
                s += __shfl_xor_sync(0xffffffffu, s, 1);
                s += __shfl_xor_sync(0xffffffffu, s, 2);
                if (q == 0) RP[r] = tq2 ? 64.0 * s : s;  // K / 64 on tensor-product elements (exact)
            }
        }
        if (want_k && tq2) {
            // KT[(f,a)][slot(j) D + g] = sum over the nodes b of basis j of
            // (K/64)[(f,a),(g,b)]; thread (row r = (f,a), g, jy): the y stage for
            // its jy, then x and z, nine outputs.  K is read as K[(g,b),(f,a)]
            // (symmetric): the lanes take consecutive rows, consecutive words.
            for (int t = tid; t < NPD * 9; t += NT) {
                const int r = t % NPD, gj = t / NPD, gg = gj / 3, jy = gj - 3 * gg;
                double w[2][2];  // [bx][bz]: the y stage
#pragma unroll
                for (int bz = 0; bz < 2; ++bz)
#pragma unroll
                    for (int bx = 0; bx < 2; ++bx) {
                        // HEX8 node of (bx, by, bz): (0,0) 0, (1,0) 1, (1,1) 2, (0,1) 3 in a layer
                        const int b0 = 4 * bz + (bx ? 1 : 0), b1 = 4 * bz + (bx ? 2 : 3);
                        const double v0 = K[(gg * NPE + b0) * NPD + r], v1 = K[(gg * NPE + b1) * NPD + r];
                        w[bx][bz] = jy == 0 ? v0 : jy == 2 ? v1 : v0 + v1;
                    }
#pragma unroll
                for (int jx = 0; jx < 3; ++jx) {
                    const double u0 = jx == 0 ? w[0][0] : jx == 2 ? w[1][0] : w[0][0] + w[1][0];
                    const double u1 = jx == 0 ? w[0][1] : jx == 2 ? w[1][1] : w[0][1] + w[1][1];
                    const int nat = jx + 3 * jy;
                    KT[r * NAD + NJ[nat] * D + gg] = u0;
                    KT[r * NAD + NJ[nat + 9] * D + gg] = u0 + u1;
                    KT[r * NAD + NJ[nat + 18] * D + gg] = u1;
                }
            }
        } else if (want_k) {
            // KT[(f,a)][x], x = slot * D + g: K symmetric, K[(f,a),(g,b)] is read
            // as K[(g,b),(f,a)], consecutive words along a
            uint32_t nxt = tid < L::NKT ? __ldg(p.ktab + tid) : 0u;
            for (int t = tid; t < L::NKT; t += NT) {
                const uint32_t it = nxt;  // next item loaded one iteration ahead
                if (t + NT < L::NKT) nxt = __ldg(p.ktab + t + NT);
                const int sl = it & 63, kb = (it >> 6) & 1023, dst = it >> 16;
                KT[dst] = fem_tdot(TCP[sl], TW + sl * NPE, TN + sl * NPE, K + kb, NPD);
            }
        }
        __syncthreads();
        // ---- phase 5: residual scatter, T^T (K T) upper triangle and scatter --------
        if (tid == 0) s_next = (int64_t)gridDim.x + (int64_t)atomicAdd(p.queue, 1ull);
        if (need_u)
            for (int x = tid; x < NAD; x += NT) {
                // count order: the lanes of a warp share trip counts
                const int sl = x / D, f = x - sl * D, i = CP[sl];
                const double s = fem_tdot(TCP[sl], TW + sl * NPE, TN + sl * NPE, RP + f * NPE, 1);
                if (assemble) {
                    if (i < nb) atomicAdd(p.rhs + f * p.nu + B[i], s);
                } else if (apply) {
                    if (i < nb) atomicAdd(p.y + f * p.nu + B[i], s);
                } else if (i < p.kw) {
                    p.Rout[(e - p.first) * p.nmax + f * p.kw + i] = s;
                }
            }
        if (want_k) {
            // entry (x, y), x <= y, of the count-ordered adofs: the row has the
            // sparser T column, so the entry costs the smaller nonzero count, and
            // entries of one count are contiguous in t (uniform warp trip counts)
            bool bad = false;
            uint32_t nxt = tid < L::NTRI ? __ldg(p.tri + tid) : 0u;
            for (int t = tid; t < L::NTRI; t += NT) {
                const uint32_t it = nxt;  // next item loaded one iteration ahead
                if (t + NT < L::NTRI) nxt = __ldg(p.tri + t + NT);
                const int sr = it & 31, f = (it >> 5) & 3, sc = (it >> 7) & 31, gg = it >> 12;
                const int cnt = TCP[sr];
                if (cnt == 0) continue;  // padding (or all-zero) column: nothing to add
                const int x = sr * D + f, y = sc * D + gg;
                const double v = tq2 ? fem_tsum(cnt, TN + sr * NPE, KT + f * NPE * NAD + y, NAD)
                                     : fem_tdot(cnt, TW + sr * NPE, TN + sr * NPE, KT + f * NPE * NAD + y, NAD);
                bad |= !fem_finite(v);
                if (assemble) {
                    atomicAdd(p.vals + RG[x * D + gg] + S[sr * NB + sc], v);
                    if (x != y) atomicAdd(p.vals + RG[y * D + f] + S[sc * NB + sr], v);
                } else {
                    // rows and columns in the set's padding width (Kout's layout)
                    const int r = f * p.kw + CP[sr], c = gg * p.kw + CP[sc];
                    double* Ko = p.Kout + (e - p.first) * (int64_t)p.nmax * p.nmax;
                    Ko[r + (int64_t)c * p.nmax] = v;
                    Ko[c + (int64_t)r * p.nmax] = v;
                }
            }
            if (bad) atomicOr(p.status, 1);
        }
        __syncthreads();
    }
}
