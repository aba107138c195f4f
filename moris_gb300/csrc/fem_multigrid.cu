// fem_multigrid.cu -- geometric multigrid V-cycle for the assembled operator of
// a uniform linear-B-spline hex mesh (the config-5 SIMP solves).
//
// The reference offers a PETSc PCMG preconditioner (Preconditioner_PETSc::
// build_multigrid_preconditioner, SOL/DLA/src/cl_DLA_Preconditioner_PETSc.cpp:
// 77-345): a multiplicative V-cycle with Galerkin coarse operators
// A_(l+1) = P^T A_l P (PC_MG_GALERKIN_BOTH), prolongations from the B-spline
// two-scale relation (Geometric_Multigrid, SOL/DLA/src/cl_DLA_Geometric_
// Multigrid.cpp:47-121, HMR get_fine_basis_weights_of_basis), SOR smoothing
// and an LU coarse solve.  The same preconditioner, laid out for the GPU:
//
//   * levels l = 0..L of node grids n_l^3, n_(l+1) = (n_l - 1) / 2 + 1.  The
//     linear B-spline two-scale relation is trilinear interpolation: coarse
//     node I weighs fine node i by prod_d (1 - |i_d - 2 I_d| / 2);
//   * every operator is a 27-point block stencil S[k][f][g][node]
//     (tap k = (dx+1) + 3 (dy+1) + 9 (dz+1); f, g displacement components)
//     with the node index fastest, so a warp reads 32 consecutive nodes of one
//     coefficient; level 0 is scattered from the CSR, level l+1 = P^T S_l P is
//     formed on the device one axis at a time (P is a Kronecker product of
//     1D two-scale relations), each pass a thread per node and component pair;
//   * smoothing is Chebyshev-accelerated point Jacobi of degree `degree` on
//     [lo, hi] * lambda_max(D^-1 A) (lambda_max by power iteration): SOR is
//     sequential, a polynomial in D^-1 A is one stencil sweep per degree.  Pre-
//     and post-smoothing use the same polynomial, so the V-cycle is a
//     symmetric positive definite operator;
//   * the coarsest level (n_L <= coarse_max) is solved with its dense inverse,
//     formed by Gauss-Jordan elimination on the device (the operator is SPD,
//     so no pivoting; two launches per pivot, so a small coarsest grid);
//   * the finest fp32_levels levels smooth, restrict and prolong in FP32 (an
//     FP32 copy of the stencil, FP32 vectors): the FP64 stencil sweep is bound
//     by the FP64 pipe (243 FMAs per node), the FP32 one by HBM.  The V-cycle
//     is a preconditioner inside an FP64 Krylov method, whose true residual
//     decides convergence.
// Vectors are type-major like the adof vector: v[g n_l^3 + node].  All work
// is issued on the legacy default stream, like fem_gpu_fcg.
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "fem_internal.hpp"

using fem::fail;

namespace {

__host__ __device__ __forceinline__ int64_t sidx(int k, int f, int g, int64_t N, int64_t i) {
    return (int64_t)((k * 3 + f) * 3 + g) * N + i;
}

__device__ __forceinline__ double mg_warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ void mg_block_sum_add(double v, double* out) {
    __shared__ double red[32];
    v = mg_warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
        v = mg_warp_sum(v);
        if (lane == 0) atomicAdd(out, v);
    }
}

// level-0 stencil from the CSR of the assembled operator (one thread per row);
// err |= 1 for a column outside the 27-node neighbourhood
// One CTA per block of kCsRows consecutive rows: their nonzeros are one contiguous
// range of the CSR, loaded coalesced into shared memory; then kCsPart threads
// per row take its entries with stride kCsPart, the lanes of a warp on 32
// consecutive rows with the same part.  Consecutive rows are consecutive
// nodes, and interior rows have the same column pattern, so a warp's lanes
// write entry p of 32 neighbouring nodes: consecutive words of one tap.  A block whose range exceeds the
// staging space (rows longer than 27 x 3 entries, which are an error anyway)
// reads from global memory.
constexpr int kCsRows = 64, kCsPart = 8, kCsCap = kCsRows * 81;
constexpr size_t kCsSmem = (size_t)kCsCap * (sizeof(double) + sizeof(int32_t));
__global__ void __launch_bounds__(kCsPart * kCsRows) mg_csr_to_stencil(int n, const int32_t* __restrict__ rp,
                                                               const int32_t* __restrict__ ci,
                                                               const double* __restrict__ v,
                                                               double* __restrict__ S, int* err) {
    extern __shared__ __align__(16) unsigned char cs_smem[];
    double* sv = reinterpret_cast<double*>(cs_smem);
    int32_t* sc = reinterpret_cast<int32_t*>(sv + kCsCap);
    const int64_t N = (int64_t)n * n * n, rows = 3 * N;
    for (int64_t r0 = (int64_t)blockIdx.x * kCsRows; r0 < rows; r0 += (int64_t)gridDim.x * kCsRows) {
        const int64_t r1 = r0 + kCsRows < rows ? r0 + kCsRows : rows;
        const int64_t e0 = rp[r0], e1 = rp[r1];
        const bool staged = e1 - e0 <= kCsCap;
        if (staged)
            for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
                sv[e - e0] = v[e];
                sc[e - e0] = ci[e];
            }
        __syncthreads();
        const int64_t row = r0 + threadIdx.x % kCsRows;
        if (row < r1) {
            const int f = (int)(row / N);
            const int64_t i = row - f * N;
            const int ix = (int)(i % n), iy = (int)((i / n) % n), iz = (int)(i / ((int64_t)n * n));
            const int64_t b = rp[row + 1];
            const int64_t n2 = (int64_t)n * n;
            for (int64_t e = rp[row] + threadIdx.x / kCsRows; e < b; e += kCsPart) {
                const int64_t col = staged ? sc[e - e0] : ci[e];
                // component and node offset d = j - i without divisions: d =
                // dx + n dy + n^2 dz with |dx|, |dy|, |dz| <= 1 is split by
                // sign tests (n >= 3); any other column leaves |dx| > 1 or a
                // neighbour outside the grid and is flagged
                const int g = (int)(col >= N) + (int)(col >= 2 * N);
                int64_t d = col - g * N - i;
                const int dz = (int)(d > n2 / 2) - (int)(d < -(n2 / 2));
                d -= dz * n2;
                const int dy = (int)(d > n / 2) - (int)(d < -(n / 2));
                d -= (int64_t)dy * n;
                const int dx = (int)(d < -2 ? -2 : d > 2 ? 2 : d);
                if (col < 0 || col >= 3 * N || dx < -1 || dx > 1 || ix + dx < 0 || ix + dx >= n || iy + dy < 0 ||
                    iy + dy >= n || iz + dz < 0 || iz + dz >= n) {
                    atomicOr(err, 1);
                    continue;
                }
                S[sidx((dx + 1) + 3 * (dy + 1) + 9 * (dz + 1), f, g, N, i)] = staged ? sv[e - e0] : v[e];
            }
        }
        __syncthreads();
    }
}

__global__ void mg_diag_inv(int64_t N, const double* __restrict__ S, double* __restrict__ dinv) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < 3 * N; t += (int64_t)gridDim.x * blockDim.x) {
        const int f = (int)(t / N);
        const double d = S[sidx(13, f, f, N, t - f * N)];
        dinv[t] = d != 0.0 ? 1.0 / d : 0.0;
    }
}

// s[f] = sum_k sum_g S[k][f][g][i] x[g][i + off_k] for the three rows of node i,
// accumulated in the vector type TV (FP32 levels: FP32 FMAs)
template <typename TS, typename TV>
__device__ __forceinline__ void stencil_rows(int n, int64_t N, const TS* __restrict__ S, const TV* __restrict__ x,
                                             int64_t i, TV s[3]) {
    const int ix = (int)(i % n), iy = (int)((i / n) % n), iz = (int)(i / ((int64_t)n * n));
    s[0] = s[1] = s[2] = TV(0);
#pragma unroll
    for (int dz = -1; dz <= 1; ++dz) {
        if (iz + dz < 0 || iz + dz >= n) continue;
#pragma unroll
        for (int dy = -1; dy <= 1; ++dy) {
            if (iy + dy < 0 || iy + dy >= n) continue;
#pragma unroll
            for (int dx = -1; dx <= 1; ++dx) {
                if (ix + dx < 0 || ix + dx >= n) continue;
                const int k = (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1);
                const int64_t j = i + dx + (int64_t)n * (dy + (int64_t)n * dz);
#pragma unroll
                for (int g = 0; g < 3; ++g) {
                    const TV xg = __ldg(x + g * N + j);
#pragma unroll
                    for (int f = 0; f < 3; ++f) s[f] = fma((TV)__ldg(S + sidx(k, f, g, N, i)), xg, s[f]);
                }
            }
        }
    }
}

// power iteration step: y = D^-1 A (a x), a = 1 / sqrt(*xx) (1 without xx: x
// is the previous step's y, normalised here instead of in a pass of its own);
// dots[0] += y.y (in the level's precision)
template <typename TS, typename TV>
__global__ void mg_power(int n, const TS* __restrict__ S, const TV* __restrict__ dinv, const TV* __restrict__ x,
                         const double* __restrict__ xx, TV* __restrict__ y, double* dots) {
    const int64_t N = (int64_t)n * n * n;
    double a = 1.0;
    if (xx) {
        const double d = *xx;
        a = d > 0.0 ? 1.0 / sqrt(d) : 0.0;
    }
    const TV at = (TV)a;
    double acc = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        TV s[3];
        stencil_rows<TS, TV>(n, N, S, x, i, s);
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            const TV v = dinv[f * N + i] * s[f] * at;
            y[f * N + i] = v;
            acc += (double)v * (double)v;
        }
    }
    mg_block_sum_add(acc, dots);
}

template <typename TV>
__global__ void mg_sumsq(int64_t m, const TV* __restrict__ x, double* dots) {
    double acc = 0.0;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m; t += (int64_t)gridDim.x * blockDim.x)
        acc += (double)x[t] * (double)x[t];
    mg_block_sum_add(acc, dots);
}

template <typename TV>
__global__ void mg_scale(int64_t m, double a, const TV* __restrict__ y, TV* __restrict__ x) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m; t += (int64_t)gridDim.x * blockDim.x)
        x[t] = (TV)(a * (double)y[t]);
}
// splitmix64 uniform in [-0.5, 0.5): element t of the stream of `seed`
__global__ void mg_random(int64_t m, uint64_t seed, double* __restrict__ x) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m; t += (int64_t)gridDim.x * blockDim.x) {
        uint64_t z = seed + (uint64_t)(t + 1) * 0x9E3779B97F4A7C15ULL;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        z ^= z >> 31;
        x[t] = (double)(z >> 11) * (1.0 / 9007199254740992.0) - 0.5;
    }
}

template <typename TA, typename TB>
__global__ void mg_convert(int64_t m, const TA* __restrict__ a, TB* __restrict__ b) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m; t += (int64_t)gridDim.x * blockDim.x)
        b[t] = (TB)a[t];
}

// q = A p on an FP64 stencil and dot += p.q (the outer Krylov product)
__global__ void mg_apply_dot(int n, const double* __restrict__ S, const double* __restrict__ p, double* __restrict__ q,
                             double* dot) {
    const int64_t N = (int64_t)n * n * n;
    double acc = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        double s[3];
        stencil_rows<double, double>(n, N, S, p, i, s);
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            q[f * N + i] = s[f];
            acc = fma(p[f * N + i], s[f], acc);
        }
    }
    mg_block_sum_add(acc, dot);
}

// Chebyshev start with x = 0: r = b, d = D^-1 b / theta, x = d
template <typename TV>
__global__ void mg_cheb_init(int64_t m, const TV* __restrict__ b, const TV* __restrict__ dinv, TV inv_theta,
                             TV* __restrict__ r, TV* __restrict__ d, TV* __restrict__ x) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m; t += (int64_t)gridDim.x * blockDim.x) {
        const TV bt = b[t];
        const TV dt = dinv[t] * bt * inv_theta;
        r[t] = bt;
        d[t] = dt;
        x[t] = dt;
    }
}

// Chebyshev step: r -= A din; dout = c1 din + c2 D^-1 r; x += dout
template <typename TS, typename TV>
__global__ void mg_cheb_step(int n, const TS* __restrict__ S, const TV* __restrict__ din, TV* __restrict__ r,
                             const TV* __restrict__ dinv, TV c1, TV c2, TV* __restrict__ dout, TV* __restrict__ x) {
    const int64_t N = (int64_t)n * n * n;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        TV s[3];
        stencil_rows<TS, TV>(n, N, S, din, i, s);
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            const int64_t t = f * N + i;
            const TV rt = r[t] - s[f];
            const TV dt = fma(c1, din[t], c2 * dinv[t] * rt);
            r[t] = rt;
            dout[t] = dt;
            x[t] += dt;
        }
    }
}

// r -= A d
template <typename TS, typename TV>
__global__ void mg_residual_update(int n, const TS* __restrict__ S, const TV* __restrict__ d, TV* __restrict__ r) {
    const int64_t N = (int64_t)n * n * n;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        TV s[3];
        stencil_rows<TS, TV>(n, N, S, d, i, s);
#pragma unroll
        for (int f = 0; f < 3; ++f) r[f * N + i] -= s[f];
    }
}

// first post-smoothing step after the coarse correction e:
// r -= A e; d = D^-1 r / theta; x += e + d
template <typename TS, typename TV>
__global__ void mg_post_first(int n, const TS* __restrict__ S, const TV* __restrict__ e, TV* __restrict__ r,
                              const TV* __restrict__ dinv, TV inv_theta, TV* __restrict__ d, TV* __restrict__ x) {
    const int64_t N = (int64_t)n * n * n;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        TV s[3];
        stencil_rows<TS, TV>(n, N, S, e, i, s);
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            const int64_t t = f * N + i;
            const TV rt = r[t] - s[f];
            const TV dt = dinv[t] * rt * inv_theta;
            r[t] = rt;
            d[t] = dt;
            x[t] += e[t] + dt;
        }
    }
}

// full-weighting restriction bc = P^T r (fine grid nf = 2 (nc - 1) + 1)
template <typename TF, typename TC>
__global__ void mg_restrict(int nf, int nc, const TF* __restrict__ r, TC* __restrict__ bc) {
    const int64_t Nc = (int64_t)nc * nc * nc, Nf = (int64_t)nf * nf * nf;
    for (int64_t I = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; I < Nc; I += (int64_t)gridDim.x * blockDim.x) {
        const int X = (int)(I % nc), Y = (int)((I / nc) % nc), Z = (int)(I / ((int64_t)nc * nc));
        TF s[3] = {TF(0), TF(0), TF(0)};
        for (int az = -1; az <= 1; ++az) {
            const int z = 2 * Z + az;
            if (z < 0 || z >= nf) continue;
            for (int ay = -1; ay <= 1; ++ay) {
                const int y = 2 * Y + ay;
                if (y < 0 || y >= nf) continue;
                for (int ax = -1; ax <= 1; ++ax) {
                    const int x = 2 * X + ax;
                    if (x < 0 || x >= nf) continue;
                    const TF w = TF((ax ? 0.5 : 1.0) * (ay ? 0.5 : 1.0) * (az ? 0.5 : 1.0));
                    const int64_t i = x + (int64_t)nf * (y + (int64_t)nf * z);
                    for (int g = 0; g < 3; ++g) s[g] = fma(w, r[g * Nf + i], s[g]);
                }
            }
        }
        for (int g = 0; g < 3; ++g) bc[g * Nc + I] = (TC)s[g];
    }
}

// trilinear prolongation e = P xc
template <typename TC, typename TF>
__global__ void mg_prolong(int nf, int nc, const TC* __restrict__ xc, TF* __restrict__ e) {
    const int64_t Nc = (int64_t)nc * nc * nc, Nf = (int64_t)nf * nf * nf;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < Nf; i += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % nf), y = (int)((i / nf) % nf), z = (int)(i / ((int64_t)nf * nf));
        const int x0 = x >> 1, y0 = y >> 1, z0 = z >> 1;
        const int x1 = x0 + (x & 1), y1 = y0 + (y & 1), z1 = z0 + (z & 1);
        const TC wx = (x & 1) ? TC(0.5) : TC(1), wy = (y & 1) ? TC(0.5) : TC(1), wz = (z & 1) ? TC(0.5) : TC(1);
        for (int g = 0; g < 3; ++g) {
            const TC* c = xc + g * Nc;
            auto at = [&](int a, int b, int cc) { return c[a + (int64_t)nc * (b + (int64_t)nc * cc)]; };
            TC s = at(x0, y0, z0);
            if (x & 1) s += at(x1, y0, z0);
            if (y & 1) {
                TC t = at(x0, y1, z0);
                if (x & 1) t += at(x1, y1, z0);
                s += t;
            }
            if (z & 1) {
                TC t = at(x0, y0, z1);
                if (x & 1) t += at(x1, y0, z1);
                if (y & 1) {
                    TC u = at(x0, y1, z1);
                    if (x & 1) u += at(x1, y1, z1);
                    t += u;
                }
                s += t;
            }
            e[g * Nf + i] = (TF)(s * wx * wy * wz);
        }
    }
}

// 1D two-scale targets: fine offset sum s (a + b) reaches the coarse tap s / 2
// (weight 1) when even, the two taps (s -+ 1) / 2 (weight 1/2 each) when odd
__device__ __forceinline__ int ntarget(int s) { return (s & 1) ? 2 : 1; }
__device__ __forceinline__ int target(int s, int t) { return (s & 1) ? ((s - 1) >> 1) + t : (s >> 1); }

// err |= 2 where the level-0 operator is not symmetric (A_ij vs A_ji beyond
// the rounding of the assembly's atomic sums, relative to the entries and to
// the diagonals of rows i and j)
__global__ void mg_check_symmetric(int n, const double* __restrict__ S, int* err) {
    // one thread per node I: every tap k <= 13 and component pair (f, g) of row
    // I against the mirrored entry (26 - k, g, f) of the neighbour J; threads of
    // a warp are consecutive nodes, so both operands load coalesced.  An
    // element adds the same value to both entries in one scatter, so they are
    // usually equal to the bit: an integer comparison (finite values only)
    // settles a pair, and the tolerance test on the FP64 pipe runs only when a
    // lane of the warp needs it.  The loop bound is uniform per warp, so every
    // vote sees all 32 lanes (blockDim a multiple of 32).
    const int64_t N = (int64_t)n * n * n;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    bool bad = false;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < N; base += stride) {
        const int64_t I = base + (threadIdx.x & 31);
        const bool live = I < N;
        const int X = live ? (int)(I % n) : 0, Y = live ? (int)((I / n) % n) : 0,
                  Z = live ? (int)(I / ((int64_t)n * n)) : 0;
        for (int k = 0; k <= 13; ++k) {
            const int dx = k % 3 - 1, dy = (k / 3) % 3 - 1, dz = k / 9 - 1;
            const bool inside = live && X + dx >= 0 && X + dx < n && Y + dy >= 0 && Y + dy < n && Z + dz >= 0 &&
                                Z + dz < n;
            const int64_t J = I + dx + (int64_t)n * (dy + (int64_t)n * dz);
#pragma unroll
            for (int f = 0; f < 3; ++f)
#pragma unroll
                for (int g = 0; g < 3; ++g) {
                    double a = 0.0, b = 0.0;
                    if (inside) {
                        a = S[sidx(k, f, g, N, I)];
                        b = S[sidx(26 - k, g, f, N, J)];
                    }
                    const long long ab = __double_as_longlong(a);
                    const bool same = ab == __double_as_longlong(b) && ((ab >> 52) & 0x7ff) != 0x7ff;
                    if (__all_sync(0xffffffffu, same)) continue;
                    if (!same) {
                        // entries that cancel to near zero carry the rounding of
                        // their terms, which scales with the diagonals: measure the
                        // asymmetry against them too (in FP32: a square root on the
                        // FP64 pipe costs far more)
                        const float di = fabsf((float)S[sidx(13, f, f, N, I)]);
                        const float dj = fabsf((float)S[sidx(13, g, g, N, J)]);
                        const float tol = 1e-10f * (float)(fabs(a) + fabs(b)) + 1e-12f * sqrtf(di * dj);
                        bad |= !((float)fabs(a - b) <= tol);
                    }
                }
        }
    }
    if (bad) atomicOr(err, 2);
}

// One-axis Galerkin coarsening of a 27-point block stencil: P = P_z (x) P_y (x)
// P_x is separable, so P^T S P is three passes, each coarsening one axis of an
// (nx, ny, nz) node box with the 1D two-scale relation while the taps along
// the other two axes pass through.  One thread per output node and component
// pair; the 3 x 3 (a, b) pairs along the axis times the 9 taps across it are
// unrolled (117 FMAs for the 27 output taps).
__host__ __device__ __forceinline__ int tap_of(int AX, int along, int o1, int o2) {
    int d[3];
    d[AX] = along;
    d[(AX + 1) % 3] = o1;
    d[(AX + 2) % 3] = o2;
    return (d[0] + 1) + 3 * (d[1] + 1) + 9 * (d[2] + 1);
}

template <int AX>
__global__ void __launch_bounds__(128) mg_rap_axis(int3 din, int3 dout, const double* __restrict__ Sin,
                                                   double* __restrict__ Sout) {
    const int64_t Nin = (int64_t)din.x * din.y * din.z, Nout = (int64_t)dout.x * dout.y * dout.z;
    const int nin_ax = AX == 0 ? din.x : AX == 1 ? din.y : din.z;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < 9 * Nout;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int fg = (int)(t / Nout);
        const int64_t I = t - fg * Nout;
        const int f = fg / 3, g = fg % 3;
        int c[3] = {(int)(I % dout.x), (int)((I / dout.x) % dout.y), (int)(I / ((int64_t)dout.x * dout.y))};
        const int C = c[AX];
        double acc[27];
#pragma unroll
        for (int k = 0; k < 27; ++k) acc[k] = 0.0;
#pragma unroll
        for (int a = -1; a <= 1; ++a) {
            const int fc = 2 * C + a;
            if (fc < 0 || fc >= nin_ax) continue;
            int ci[3] = {c[0], c[1], c[2]};
            ci[AX] = fc;
            const int64_t i = ci[0] + (int64_t)din.x * (ci[1] + (int64_t)din.y * ci[2]);
            const double wa = a ? 0.5 : 1.0;
#pragma unroll
            for (int b = -1; b <= 1; ++b) {
                const int sm = a + b;
                const double pw = (sm & 1) ? 0.5 : 1.0;
#pragma unroll
                for (int o2 = -1; o2 <= 1; ++o2)
#pragma unroll
                    for (int o1 = -1; o1 <= 1; ++o1) {
                        const double v = wa * pw * __ldg(Sin + sidx(tap_of(AX, b, o1, o2), f, g, Nin, i));
#pragma unroll
                        for (int tt = 0; tt < 2; ++tt) {
                            if (tt >= ntarget(sm)) continue;
                            acc[tap_of(AX, target(sm, tt), o1, o2)] += v;
                        }
                    }
            }
        }
#pragma unroll
        for (int k = 0; k < 27; ++k) Sout[sidx(k, f, g, Nout, I)] = acc[k];
    }
}

// dense operator of the coarsest level, row-major m x m (m = 3 N)
__global__ void mg_dense(int n, const double* __restrict__ S, double* __restrict__ A) {
    const int64_t N = (int64_t)n * n * n, m = 3 * N;
    for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < m; row += (int64_t)gridDim.x * blockDim.x) {
        const int f = (int)(row / N);
        const int64_t i = row - f * N;
        const int ix = (int)(i % n), iy = (int)((i / n) % n), iz = (int)(i / ((int64_t)n * n));
        for (int k = 0; k < 27; ++k) {
            const int dx = k % 3 - 1, dy = (k / 3) % 3 - 1, dz = k / 9 - 1;
            if (ix + dx < 0 || ix + dx >= n || iy + dy < 0 || iy + dy >= n || iz + dz < 0 || iz + dz >= n) continue;
            const int64_t j = i + dx + (int64_t)n * (dy + (int64_t)n * dz);
            for (int g = 0; g < 3; ++g) A[row * m + g * N + j] = S[sidx(k, f, g, N, i)];
        }
    }
}

// Gauss-Jordan inversion in place, pivot k: stash row k and column k, then
// update every entry (a[k][k] > 0 for an SPD operator)
// Gauss-Jordan step k of the in-place inverse, from A to B (two buffers, so the
// pivot row and column are read from the previous step without a copy)
__global__ void mg_gj_step(int64_t m, const double* __restrict__ A, double* __restrict__ B, int64_t k) {
    const double inv = 1.0 / A[k * m + k];
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m * m; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / m, j = t - i * m;
        const double rk = (j == k ? 1.0 : A[k * m + j]) * inv;
        if (i == k) B[t] = rk;
        else B[t] = (j == k ? 0.0 : A[t]) - A[i * m + k] * rk;
    }
}

// x = Ainv b, one warp per row
__global__ void mg_gemv(int64_t m, const double* __restrict__ A, const double* __restrict__ b, double* __restrict__ x) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < m; row += warps) {
        double s = 0.0;
        for (int64_t j = lane; j < m; j += 32) s = fma(A[row * m + j], b[j], s);
        s = mg_warp_sum(s);
        if (lane == 0) x[row] = s;
    }
}

unsigned blocks_for(int64_t work, int tpb) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((work + tpb - 1) / tpb, (int64_t)fem::sm_count() * 32));
}

}  // namespace

struct fem_mg {
    struct Level {
        int n = 0;
        int64_t N = 0;
        bool fp32 = false;        // smoothing and vectors in FP32
        double* S = nullptr;      // FP64 stencil (Galerkin products, power iteration, FP64 smoothing)
        float* S32 = nullptr;     // FP32 copy of an FP32 level
        double* dinv = nullptr;
        float* dinv32 = nullptr;
        double lmax = 0.0;
        // vectors in the level's precision; level 0 of an FP64 hierarchy uses the caller's b and x
        void *x = nullptr, *b = nullptr, *r = nullptr, *d0 = nullptr, *d1 = nullptr;
    };
    std::vector<Level> lv;
    double* ainv = nullptr;  // dense inverse of the coarsest operator
    int64_t m = 0;
    fem_mg_opts o{};
    double setup_seconds = 0.0;
    double* dots = nullptr;
    double* pdots = nullptr;  // power-iteration norms (power_iters + 1)
    int* err = nullptr;
    std::vector<void*> bufs;
    ~fem_mg() {
        cudaDeviceSynchronize();
        for (void* p : bufs) cudaFree(p);
    }
    template <typename T>
    bool alloc(T** p, size_t count) {
        if (cudaMalloc((void**)p, count * sizeof(T)) != cudaSuccess) return false;
        bufs.push_back(*p);
        return true;
    }
    bool alloc_vec(void** p, size_t count, bool f32) {
        if (f32) return alloc((float**)p, count);
        return alloc((double**)p, count);
    }
};

namespace {

constexpr int kTpb = 256;

template <typename TV>
struct Cheb {
    TV inv_theta, delta, sigma;
    explicit Cheb(const fem_mg::Level& L, const fem_mg_opts& o) {
        const double lo = o.lo_frac * L.lmax, hi = o.hi_frac * L.lmax;
        const double theta = 0.5 * (hi + lo), dl = 0.5 * (hi - lo);
        inv_theta = (TV)(1.0 / theta);
        delta = (TV)dl;
        sigma = (TV)(theta / dl);
    }
};

// Chebyshev pre-smoothing from x = 0; on return r = b - A x
template <typename TS, typename TV>
void smooth_pre(const fem_mg::Level& L, const TS* S, const TV* dinv, const fem_mg_opts& o, const TV* b, TV* x) {
    const Cheb<double> c(L, o);
    const unsigned vb = blocks_for(3 * L.N, kTpb), nb = blocks_for(L.N, kTpb);
    TV *r = (TV*)L.r, *din = (TV*)L.d0, *dout = (TV*)L.d1;
    mg_cheb_init<TV><<<vb, kTpb>>>(3 * L.N, b, dinv, (TV)c.inv_theta, r, din, x);
    double rho = 1.0 / c.sigma;
    for (int k = 1; k < o.degree; ++k) {
        const double rn = 1.0 / (2.0 * c.sigma - rho);
        mg_cheb_step<TS, TV><<<nb, kTpb>>>(L.n, S, din, r, dinv, (TV)(rn * rho), (TV)(2.0 * rn / c.delta), dout, x);
        rho = rn;
        std::swap(din, dout);
    }
    mg_residual_update<TS, TV><<<nb, kTpb>>>(L.n, S, din, r);
}

// Chebyshev post-smoothing after the coarse correction e, which lives in d1:
// the first step reads it and writes d0, after which d1 is free for the ping-pong
template <typename TS, typename TV>
void smooth_post(const fem_mg::Level& L, const TS* S, const TV* dinv, const fem_mg_opts& o, const TV* e, TV* x) {
    const Cheb<double> c(L, o);
    const unsigned nb = blocks_for(L.N, kTpb);
    TV *r = (TV*)L.r, *din = (TV*)L.d0, *dout = (TV*)L.d1;
    mg_post_first<TS, TV><<<nb, kTpb>>>(L.n, S, e, r, dinv, (TV)c.inv_theta, din, x);
    double rho = 1.0 / c.sigma;
    for (int k = 1; k < o.degree; ++k) {
        const double rn = 1.0 / (2.0 * c.sigma - rho);
        mg_cheb_step<TS, TV><<<nb, kTpb>>>(L.n, S, din, r, dinv, (TV)(rn * rho), (TV)(2.0 * rn / c.delta), dout, x);
        rho = rn;
        std::swap(din, dout);
    }
}

void vcycle(fem_mg* g, size_t l, const void* b, void* x);

// smoothing, restriction, the coarser cycle, prolongation on a level of vector type TV
template <typename TV>
void level_cycle(fem_mg* g, size_t l, const TV* b, TV* x) {
    fem_mg::Level& L = g->lv[l];
    fem_mg::Level& C = g->lv[l + 1];
    const bool f32 = std::is_same<TV, float>::value;
    if (f32) smooth_pre(L, L.S32, L.dinv32, g->o, (const float*)b, (float*)x);
    else smooth_pre(L, L.S, L.dinv, g->o, (const double*)b, (double*)x);
    if (C.fp32) mg_restrict<TV, float><<<blocks_for(C.N, kTpb), kTpb>>>(L.n, C.n, (const TV*)L.r, (float*)C.b);
    else mg_restrict<TV, double><<<blocks_for(C.N, kTpb), kTpb>>>(L.n, C.n, (const TV*)L.r, (double*)C.b);
    vcycle(g, l + 1, C.b, C.x);
    TV* e = (TV*)L.d1;
    if (C.fp32) mg_prolong<float, TV><<<blocks_for(L.N, kTpb), kTpb>>>(L.n, C.n, (const float*)C.x, e);
    else mg_prolong<double, TV><<<blocks_for(L.N, kTpb), kTpb>>>(L.n, C.n, (const double*)C.x, e);
    if (f32) smooth_post(L, L.S32, L.dinv32, g->o, (const float*)e, (float*)x);
    else smooth_post(L, L.S, L.dinv, g->o, (const double*)e, (double*)x);
}

// x_l = V_l(b_l) in the level's precision
void vcycle(fem_mg* g, size_t l, const void* b, void* x) {
    if (l + 1 == g->lv.size()) {  // coarsest level: FP64 dense inverse
        mg_gemv<<<blocks_for(g->m * 32, kTpb), kTpb>>>(g->m, g->ainv, (const double*)b, (double*)x);
        return;
    }
    if (g->lv[l].fp32) level_cycle<float>(g, l, (const float*)b, (float*)x);
    else level_cycle<double>(g, l, (const double*)b, (double*)x);
}

// lambda_max(D^-1 A) of a level by power iteration from the seeded vector in
// px (FP64; converted for an FP32 level); px / py are finest-size scratch
template <typename TS, typename TV>
double power_lambda(fem_mg* g, const fem_mg::Level& L, const TS* S, const TV* dinv, double* px, double* py, int iters) {
    const unsigned vb = blocks_for(3 * L.N, kTpb);
    TV *x = (TV*)px, *y = (TV*)py;
    if (!std::is_same<TV, double>::value) {
        mg_convert<double, TV><<<vb, kTpb>>>(3 * L.N, px, y);
        mg_scale<TV><<<vb, kTpb>>>(3 * L.N, 1.0, y, x);
    }
    // squared norms on the device: pd[0] = |x0|^2, pd[it + 1] = |y_it|^2 with
    // y_it = D^-1 A x_it and x_(it+1) = y_it / |y_it|, the normalisation done by
    // the next step as it reads y_it; the host reads the norms once at the end
    double* pd = g->pdots;
    cudaMemset(pd, 0, (iters + 1) * sizeof(double));
    mg_sumsq<TV><<<vb, kTpb>>>(3 * L.N, x, pd);
    for (int it = 0; it < iters; ++it) {
        mg_power<TS, TV><<<blocks_for(L.N, kTpb), kTpb>>>(L.n, S, dinv, x, it ? pd + it : nullptr, y, pd + it + 1);
        std::swap(x, y);
    }
    std::vector<double> h(iters + 1, 0.0);
    cudaMemcpy(h.data(), pd, (iters + 1) * sizeof(double), cudaMemcpyDeviceToHost);
    double xn = std::sqrt(h[0]), lam = 0.0;
    for (int it = 0; it < iters; ++it) {
        const double yn = std::sqrt(h[it + 1]);
        lam = yn / xn;
        if (!(yn > 0.0)) break;
        xn = 1.0;
    }
    return lam;
}

}  // namespace

bool mg_operator(fem_mg* g, const double* p, double* q, double* dot) {
    if (!g) return false;
    const fem_mg::Level& L = g->lv[0];
    mg_apply_dot<<<blocks_for(L.N, kTpb), kTpb>>>(L.n, L.S, p, q, dot);
    return cudaGetLastError() == cudaSuccess;
}

bool mg_vcycle(fem_mg* g, const double* r, double* z) {
    if (!g) return false;
    fem_mg::Level& L = g->lv[0];
    if (L.fp32) {
        const unsigned vb = blocks_for(3 * L.N, kTpb);
        mg_convert<double, float><<<vb, kTpb>>>(3 * L.N, r, (float*)L.b);
        vcycle(g, 0, L.b, L.x);
        mg_convert<float, double><<<vb, kTpb>>>(3 * L.N, (const float*)L.x, z);
    } else {
        vcycle(g, 0, r, z);
    }
    return cudaGetLastError() == cudaSuccess;
}

extern "C" {

fem_gpu_status fem_mg_default_opts(fem_mg_opts* o) {
    if (!o) return FEM_GPU_BAD_ARG;
    o->coarse_max = 5;
    o->degree = 2;
    o->lo_frac = 0.1;
    o->hi_frac = 1.1;
    o->power_iters = 12;
    o->fp32_levels = 8;
    return FEM_GPU_OK;
}

fem_gpu_status fem_mg_create(fem_gpu_ctx* c, const int32_t* rowptr, const int32_t* colidx, const double* vals,
                             const fem_mg_opts* opts, fem_mg** out) {
    if (!c || !rowptr || !colidx || !vals || !out) return FEM_GPU_BAD_ARG;
    *out = nullptr;
    if (!c->host_final) return FEM_GPU_NOT_FINALIZED;
    fem_mg_opts o;
    fem_mg_default_opts(&o);
    if (opts) o = *opts;
    if (o.degree < 1 || o.degree > 8 || !(o.lo_frac > 0.0) || !(o.hi_frac > o.lo_frac) || o.power_iters < 1 ||
        o.coarse_max < 3 || o.coarse_max > 9 || o.fp32_levels < 0)
        return fail(c, FEM_GPU_BAD_ARG, "multigrid: options out of range");
    const int64_t nu = c->num_used;
    const int nf = (int)std::llround(std::cbrt((double)nu));
    if (c->dim != 3 || (int64_t)nf * nf * nf != nu)
        return fail(c, FEM_GPU_BAD_ARG, "multigrid: needs a 3D model on a cubic node grid");
    std::vector<int> ns{nf};
    while (ns.back() > o.coarse_max) {
        const int n = ns.back();
        if ((n - 1) % 2) return fail(c, FEM_GPU_BAD_ARG, "multigrid: node grid edge - 1 must halve down to coarse_max");
        ns.push_back((n - 1) / 2 + 1);
    }
    if (ns.size() < 2) return fail(c, FEM_GPU_BAD_ARG, "multigrid: grid already at or below coarse_max");
    const auto t0 = std::chrono::steady_clock::now();
    fem_mg* g = new fem_mg();
    g->o = o;
    g->lv.resize(ns.size());
    bool ok = g->alloc(&g->dots, 4) && g->alloc(&g->pdots, (size_t)std::max(o.power_iters, 1) + 1) &&
              g->alloc(&g->err, 1);
    for (size_t l = 0; ok && l < ns.size(); ++l) {
        fem_mg::Level& L = g->lv[l];
        L.n = ns[l];
        L.N = (int64_t)L.n * L.n * L.n;
        L.fp32 = (int)l < o.fp32_levels && l + 1 < ns.size();
        ok = g->alloc(&L.S, 243 * L.N) && g->alloc(&L.dinv, 3 * L.N) && g->alloc_vec(&L.r, 3 * L.N, L.fp32) &&
             g->alloc_vec(&L.d0, 3 * L.N, L.fp32) && g->alloc_vec(&L.d1, 3 * L.N, L.fp32);
        if (ok && (l > 0 || L.fp32)) ok = g->alloc_vec(&L.x, 3 * L.N, L.fp32) && g->alloc_vec(&L.b, 3 * L.N, L.fp32);
        if (ok && L.fp32) ok = g->alloc(&L.S32, 243 * L.N) && g->alloc(&L.dinv32, 3 * L.N);
    }
    g->m = 3 * g->lv.back().N;
    double* ainv2 = nullptr;
    if (ok) ok = g->alloc(&g->ainv, g->m * g->m) && g->alloc(&ainv2, g->m * g->m);
    if (!ok) {
        delete g;
        return fail(c, FEM_GPU_OUT_OF_MEMORY, "multigrid hierarchy");
    }
    // level 0 from the CSR, then the Galerkin products
    fem_mg::Level& L0 = g->lv[0];
    cudaMemset(L0.S, 0, 243 * L0.N * sizeof(double));
    cudaMemset(g->err, 0, sizeof(int));
    cudaFuncSetAttribute(mg_csr_to_stencil, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCsSmem);
    mg_csr_to_stencil<<<blocks_for(3 * L0.N, kCsRows), kCsPart * kCsRows, kCsSmem>>>(L0.n, rowptr, colidx, vals,
                                                                                    L0.S, g->err);
    mg_check_symmetric<<<blocks_for(L0.N, kTpb), kTpb>>>(L0.n, L0.S, g->err);
    {
        // Galerkin products axis by axis through two scratch boxes (freed after setup)
        const int64_t n0 = L0.n, n1 = (n0 - 1) / 2 + 1;
        double *t1 = nullptr, *t2 = nullptr;
        if (cudaMalloc(&t1, 243 * n0 * n0 * n1 * sizeof(double)) != cudaSuccess ||
            cudaMalloc(&t2, 243 * n0 * n1 * n1 * sizeof(double)) != cudaSuccess) {
            cudaFree(t1);
            delete g;
            return fail(c, FEM_GPU_OUT_OF_MEMORY, "multigrid Galerkin scratch");
        }
        for (size_t l = 0; l + 1 < g->lv.size(); ++l) {
            const int nf = g->lv[l].n, ncs = g->lv[l + 1].n;
            const int3 a{nf, nf, nf}, b{nf, nf, ncs}, cc{nf, ncs, ncs}, d{ncs, ncs, ncs};
            mg_rap_axis<2><<<blocks_for(9 * (int64_t)b.x * b.y * b.z, 128), 128>>>(a, b, g->lv[l].S, t1);
            mg_rap_axis<1><<<blocks_for(9 * (int64_t)cc.x * cc.y * cc.z, 128), 128>>>(b, cc, t1, t2);
            mg_rap_axis<0><<<blocks_for(9 * (int64_t)d.x * d.y * d.z, 128), 128>>>(cc, d, t2, g->lv[l + 1].S);
        }
        cudaDeviceSynchronize();
        cudaFree(t1);
        cudaFree(t2);
    }
    int herr = 0;
    cudaMemcpy(&herr, g->err, sizeof(int), cudaMemcpyDeviceToHost);
    if (herr) {
        delete g;
        return fail(c, FEM_GPU_BAD_ARG, (herr & 1) ? "multigrid: operator is not a 27-point nodal stencil on the node grid"
                                                   : "multigrid: operator is not symmetric");
    }
    // smoother data: diagonal, FP32 copies, lambda_max(D^-1 A) by power iteration
    // (FP64, in two scratch vectors of the finest size)
    double *px = nullptr, *py = nullptr;
    if (!g->alloc(&px, 3 * L0.N) || !g->alloc(&py, 3 * L0.N)) {
        delete g;
        return fail(c, FEM_GPU_OUT_OF_MEMORY, "multigrid hierarchy");
    }
    for (size_t l = 0; l + 1 < g->lv.size(); ++l) {
        fem_mg::Level& L = g->lv[l];
        const unsigned vb = blocks_for(3 * L.N, kTpb);
        mg_diag_inv<<<blocks_for(3 * L.N, kTpb), kTpb>>>(L.N, L.S, L.dinv);
        if (L.fp32) {
            mg_convert<double, float><<<blocks_for(243 * L.N, kTpb), kTpb>>>(243 * L.N, L.S, L.S32);
            mg_convert<double, float><<<vb, kTpb>>>(3 * L.N, L.dinv, L.dinv32);
        }
        mg_random<<<vb, kTpb>>>(3 * L.N, 0x5EEDULL + l, px);
        // FP64 levels iterate on the FP64 stencil; FP32 levels on their FP32 copy
        // (the smoothing interval needs lambda_max to a few digits only)
        double lam = L.fp32 ? power_lambda<float, float>(g, L, L.S32, L.dinv32, px, py, o.power_iters)
                            : power_lambda<double, double>(g, L, L.S, L.dinv, px, py, o.power_iters);
        L.lmax = lam;
        if (!(lam > 0.0) || !std::isfinite(lam)) {
            delete g;
            return fail(c, FEM_GPU_NONFINITE, "multigrid: power iteration gave no positive lambda_max");
        }
    }
    // coarsest level: dense inverse
    fem_mg::Level& LC = g->lv.back();
    cudaMemset(g->ainv, 0, g->m * g->m * sizeof(double));
    mg_dense<<<blocks_for(g->m, kTpb), kTpb>>>(LC.n, LC.S, g->ainv);
    for (int64_t k = 0; k < g->m; ++k) {
        mg_gj_step<<<blocks_for(g->m * g->m, kTpb), kTpb>>>(g->m, g->ainv, ainv2, k);
        std::swap(g->ainv, ainv2);
    }
    if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess) {
        delete g;
        return fail(c, FEM_GPU_CUDA_ERROR, "multigrid setup");
    }
    g->setup_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    *out = g;
    return FEM_GPU_OK;
}

fem_gpu_status fem_mg_destroy(fem_mg* g) {
    delete g;
    return FEM_GPU_OK;
}

int32_t fem_mg_num_levels(const fem_mg* g) { return g ? (int32_t)g->lv.size() : 0; }

double fem_mg_setup_seconds(const fem_mg* g) { return g ? g->setup_seconds : 0.0; }

fem_gpu_status fem_mg_level_info(const fem_mg* g, int32_t level, int32_t* n, double* lambda_max) {
    if (!g || level < 0 || level >= (int32_t)g->lv.size()) return FEM_GPU_BAD_ARG;
    if (n) *n = g->lv[level].n;
    if (lambda_max) *lambda_max = g->lv[level].lmax;
    return FEM_GPU_OK;
}

fem_gpu_status fem_mg_get_stencil(const fem_mg* g, int32_t level, double* host_out) {
    if (!g || !host_out || level < 0 || level >= (int32_t)g->lv.size()) return FEM_GPU_BAD_ARG;
    const fem_mg::Level& L = g->lv[level];
    return cudaMemcpy(host_out, L.S, 243 * L.N * sizeof(double), cudaMemcpyDeviceToHost) == cudaSuccess
               ? FEM_GPU_OK
               : FEM_GPU_CUDA_ERROR;
}

fem_gpu_status fem_mg_apply(fem_mg* g, const double* r, double* z) {
    if (!g || !r || !z) return FEM_GPU_BAD_ARG;
    return mg_vcycle(g, r, z) ? FEM_GPU_OK : FEM_GPU_CUDA_ERROR;
}

}  // extern "C"
