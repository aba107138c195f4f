// fem_hmr_device.cu -- element T matrices and node rows of refined
// (hierarchical) HMR B-spline meshes on the GPU.
//
// The same rules as the host's fem_hmr.cpp, one thread per element:
//  * the hierarchy: the refined elements of every level as sorted packed keys
//    (binary search), padding and existence as BSpline_Mesh / Background_Mesh
//    define them (HMR/src/cl_HMR_Background_Element_Base.hpp:225-249);
//  * basis states (BSpline_Mesh::determine_basis_state,
//    cl_HMR_BSpline_Mesh.hpp:738-807);
//  * untruncated element T (T_Matrix_Base::calculate_untruncated_t_matrix,
//    cl_HMR_T_Matrix_Base.cpp:58-126): the column of an active basis m of level
//    lev on the level-l element is the product over the axes of the 1-D
//    coefficients of m's level-l expansion by the two-scale relation (children
//    2m - p + t, weights 2^-p C(p + 1, t)) -- the same numbers as the host's
//    chain of child matrices, since B-splines are locally linearly independent;
//  * truncated element T (calculate_truncated_t_matrix, :127-248): the
//    element's active bases, and the active bases of the parent element
//    restricted to the children that are deactivated.
// Every weight is a dyadic fraction with few bits, so the T entries are exact
// in FP64 whatever the order of the sums: the device matrices equal the
// host's bit for bit.  The node rows (T_Matrix_Base::evaluate, :306-457) use
// the host's operations in the host's order, with explicitly rounded
// operations (no contraction), so they are equal bit for bit too.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "fem_internal.hpp"

namespace {

constexpr int kBits = 20;       // per direction in a packed key
constexpr int kMaxList = 24;    // 1-D expansion window

struct HmrArgs {
    int dim, p, pad, nloc, levels;
    long long ne[3];
    int local[fem::kHmrMaxLocal][3];
    int inv[fem::kHmrMaxLocal];  // local offset (ox + (p+1)(oy + (p+1) oz)) -> local basis index
    double w1[5];                // 2^-p C(p + 1, t), t = 0 .. p + 1
    const unsigned long long* keys;
    const long long* koff;
};

struct Ix {
    long long v[3];
};

__device__ __forceinline__ unsigned long long pack(const Ix& e) {
    return (unsigned long long)e.v[0] | ((unsigned long long)e.v[1] << kBits) |
           ((unsigned long long)e.v[2] << (2 * kBits));
}

__device__ bool is_refined(const HmrArgs& h, int l, const Ix& e) {
    if (l < 0 || l >= h.levels) return false;
    const unsigned long long key = pack(e);
    long long lo = h.koff[l], hi = h.koff[l + 1];
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        const unsigned long long k = h.keys[mid];
        if (k == key) return true;
        if (k < key) lo = mid + 1;
        else hi = mid;
    }
    return false;
}

__device__ bool inside(const HmrArgs& h, int l, const Ix& e) {
    for (int k = 0; k < h.dim; ++k)
        if (e.v[k] < 0 || e.v[k] >= ((h.ne[k] + 2 * h.pad) << l)) return false;
    return true;
}

__device__ Ix parent(const HmrArgs& h, const Ix& e) {
    Ix q{{0, 0, 0}};
    for (int k = 0; k < h.dim; ++k) q.v[k] = e.v[k] >> 1;
    return q;
}

__device__ bool exists(const HmrArgs& h, int l, const Ix& e) {
    return inside(h, l, e) && (l == 0 || is_refined(h, l - 1, parent(h, e)));
}

__device__ bool padding(const HmrArgs& h, int l, const Ix& e) {
    for (int k = 0; k < h.dim; ++k)
        if (e.v[k] < ((long long)h.pad << l) || e.v[k] >= ((h.pad + h.ne[k]) << l)) return true;
    return false;
}

__device__ bool active(const HmrArgs& h, int l, const Ix& e) {
    return exists(h, l, e) && !is_refined(h, l, e) && !padding(h, l, e);
}

// 0 deactivated, 1 active, 2 refined
__device__ int basis_state(const HmrArgs& h, int l, const Ix& m) {
    int tot = 1;
    for (int k = 0; k < h.dim; ++k) tot *= h.p + 1;
    bool any_active = false;
    for (int c = 0; c < tot; ++c) {
        Ix e{{0, 0, 0}};
        int rem = c;
        for (int k = 0; k < h.dim; ++k) {
            e.v[k] = m.v[k] - rem % (h.p + 1);
            rem /= h.p + 1;
        }
        if (!exists(h, l, e)) return 0;
        any_active |= active(h, l, e);
    }
    return any_active ? 1 : 2;
}

__device__ Ix local_basis(const HmrArgs& h, const Ix& e, int b) {
    Ix m{{0, 0, 0}};
    for (int k = 0; k < h.dim; ++k) m.v[k] = e.v[k] + h.local[b][k];
    return m;
}

// the coefficient of level-(lev + r) basis j in the expansion of level-lev
// basis m by r refinements (1-D): the children of the current window, kept
// while their support can still reach j's
__device__ double coef1(const HmrArgs& h, int r, long long m, long long j) {
    if (r == 0) return m == j ? 1.0 : 0.0;
    long long idx[kMaxList], nidx[kMaxList];
    double w[kMaxList], nw[kMaxList];
    int n = 1;
    idx[0] = m;
    w[0] = 1.0;
    for (int s = 1; s <= r; ++s) {
        const long long scale = 1ll << (r - s);  // level-(lev + s) units -> level-(lev + r) units
        int nn = 0;
        for (int a = 0; a < n; ++a)
            for (int t = 0; t <= h.p + 1; ++t) {
                const long long c = 2 * idx[a] - h.p + t;
                // supports [c - p, c + 1) (scaled) and [j - p, j + 1) must overlap
                if ((c + 1) * scale <= j - h.p || (c - h.p) * scale >= j + 1) continue;
                const double cw = w[a] * h.w1[t];
                int q = 0;
                while (q < nn && nidx[q] != c) ++q;
                if (q == nn) {
                    if (nn == kMaxList) return 0.0;  // cannot happen for p <= 3 (window <= 2 p + 2)
                    nidx[nn] = c;
                    nw[nn] = 0.0;
                    ++nn;
                }
                nw[q] += cw;
            }
        n = nn;
        for (int a = 0; a < n; ++a) {
            idx[a] = nidx[a];
            w[a] = nw[a];
        }
    }
    for (int a = 0; a < n; ++a)
        if (idx[a] == j) return w[a];
    return 0.0;
}

// element T of element e (level l): ndof, and with T != nullptr the columns
// (nloc each) and the dofs (level, m0, m1, m2)
__device__ int element_t(const HmrArgs& h, int l, const Ix& e, bool truncate, double* T, long long* dofs) {
    const int B = h.nloc;
    int nd = 0;
    if (!truncate) {
        Ix el = e;
        for (int lev = l; lev >= 0; --lev) {
            for (int k = 0; k < B; ++k) {
                const Ix m = local_basis(h, el, k);
                if (basis_state(h, lev, m) != 1) continue;
                if (T) {
                    for (int b = 0; b < B; ++b) {
                        const Ix jb = local_basis(h, e, b);
                        double v = 1.0;
                        for (int d = 0; d < h.dim && v != 0.0; ++d) v *= coef1(h, l - lev, m.v[d], jb.v[d]);
                        T[(size_t)nd * B + b] = v;
                    }
                    dofs[nd * 4 + 0] = lev;
                    for (int d = 0; d < 3; ++d) dofs[nd * 4 + 1 + d] = m.v[d];
                }
                ++nd;
            }
            if (lev > 0) el = parent(h, el);
        }
        return nd;
    }
    for (int k = 0; k < B; ++k) {
        const Ix m = local_basis(h, e, k);
        if (basis_state(h, l, m) != 1) continue;
        if (T) {
            for (int b = 0; b < B; ++b) T[(size_t)nd * B + b] = b == k ? 1.0 : 0.0;
            dofs[nd * 4 + 0] = l;
            for (int d = 0; d < 3; ++d) dofs[nd * 4 + 1 + d] = m.v[d];
        }
        ++nd;
    }
    if (l == 0) return nd;
    const Ix par = parent(h, e);
    const int n1 = h.p + 2, P1 = h.p + 1;
    int tot = 1;
    for (int d = 0; d < h.dim; ++d) tot *= n1;
    double col[fem::kHmrMaxLocal];
    for (int k = 0; k < B; ++k) {
        const Ix m = local_basis(h, par, k);
        if (basis_state(h, l - 1, m) != 1) continue;
        for (int b = 0; b < B; ++b) col[b] = 0.0;
        for (int c = 0; c < tot; ++c) {
            Ix ch{{0, 0, 0}};
            double w = 1.0;
            int rem = c, off = 0, stride = 1;
            bool local = true;
            for (int d = 0; d < h.dim; ++d) {
                const int t = rem % n1;
                rem /= n1;
                ch.v[d] = 2 * m.v[d] - h.p + t;
                w *= h.w1[t];
                const long long o = ch.v[d] - e.v[d];
                local &= o >= 0 && o <= h.p;
                off += (int)(local ? o : 0) * stride;
                stride *= P1;
            }
            if (local && basis_state(h, l, ch) == 0) col[h.inv[off]] += w;
        }
        double lo = 0.0, hi = 0.0;
        for (int b = 0; b < B; ++b) {
            lo = fmin(lo, col[b]);
            hi = fmax(hi, col[b]);
        }
        if (lo < -1e-12 || hi > 1e-12) {
            if (T) {
                for (int b = 0; b < B; ++b) T[(size_t)nd * B + b] = col[b];
                dofs[nd * 4 + 0] = l - 1;
                for (int d = 0; d < 3; ++d) dofs[nd * 4 + 1 + d] = m.v[d];
            }
            ++nd;
        }
    }
    return nd;
}

__global__ void hmr_count_kernel(HmrArgs h, int truncate, long long count, const int* level, const long long* idx,
                                 int* ndof) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        const Ix e{{idx[i * 3], idx[i * 3 + 1], idx[i * 3 + 2]}};
        ndof[i] = element_t(h, level[i], e, truncate != 0, nullptr, nullptr);
    }
}

__global__ void hmr_fill_kernel(HmrArgs h, int truncate, long long count, const int* level, const long long* idx,
                                const long long* toff, double* T, long long* dofs, int* ndof) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        const Ix e{{idx[i * 3], idx[i * 3 + 1], idx[i * 3 + 2]}};
        const long long o = toff[i];
        // the dof slots of element i start at o / nloc
        const int nd = element_t(h, level[i], e, truncate != 0, T + o, dofs + (o / h.nloc) * 4);
        if (nd != ndof[i]) ndof[i] = -1;  // the two passes disagree: reported by the host
    }
}

// uniform cardinal B-spline of degree p on [0, p + 1], the host's recursion
// with explicitly rounded operations
__device__ double cardinal(int p, double t) {
    if (p == 0) return (t >= 0.0 && t < 1.0) ? 1.0 : 0.0;
    const double a = __dmul_rn(t, cardinal(p - 1, t));
    const double b = __dmul_rn(__dsub_rn((double)(p + 1), t), cardinal(p - 1, __dsub_rn(t, 1.0)));
    return __ddiv_rn(__dadd_rn(a, b), (double)p);
}

__global__ void hmr_rows_kernel(HmrArgs h, const double* len, long long nfirst, const long long* elem,
                                const double* x, const int* level, const long long* idx, const int* ndof,
                                const long long* toff, const double* T, const long long* roff, double* rows) {
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nfirst;
         k += (long long)gridDim.x * blockDim.x) {
        const long long i = elem[k];
        const int l = level[i], B = h.nloc, nd = ndof[i];
        const Ix e{{idx[i * 3], idx[i * 3 + 1], idx[i * 3 + 2]}};
        double lag[fem::kHmrMaxLocal];
        for (int b = 0; b < B; ++b) {
            const Ix mb = local_basis(h, e, b);
            double v = 1.0;
            for (int d = 0; d < h.dim; ++d) {
                const double ne = (double)h.ne[d];
                // hl = len / ne / 2^l; t = (x + pad len / ne) / hl - (m - p)
                const double hl = __ddiv_rn(__ddiv_rn(len[d], ne), (double)(1ll << l));
                const double shift = __ddiv_rn(__dmul_rn((double)h.pad, len[d]), ne);
                const double t = __dsub_rn(__ddiv_rn(__dadd_rn(x[k * h.dim + d], shift), hl), (double)(mb.v[d] - h.p));
                v = __dmul_rn(v, cardinal(h.p, t));
            }
            lag[b] = v;
        }
        const double* Ti = T + toff[i];
        for (int j = 0; j < nd; ++j) {
            double s = 0.0;
            for (int b = 0; b < B; ++b) s = __dadd_rn(s, __dmul_rn(lag[b], Ti[(size_t)j * B + b]));
            rows[roff[k] + j] = s;
        }
    }
}

HmrArgs make_args(const fem::HmrDevice& h, const unsigned long long* keys, const long long* koff) {
    HmrArgs a{};
    a.dim = h.dim;
    a.p = h.p;
    a.pad = h.pad;
    a.nloc = h.nloc;
    a.levels = h.levels;
    for (int k = 0; k < 3; ++k) a.ne[k] = h.ne[k];
    for (int b = 0; b < h.nloc; ++b) {
        int off = 0, stride = 1;
        for (int k = 0; k < 3; ++k) {
            a.local[b][k] = h.local[b][k];
            if (k < h.dim) {
                off += h.local[b][k] * stride;
                stride *= h.p + 1;
            }
        }
        a.inv[off] = b;
    }
    for (int t = 0; t <= h.p + 1; ++t) {
        double c = 1.0;  // C(p + 1, t)
        for (int i = 1; i <= t; ++i) c = c * (h.p + 2 - i) / i;
        double pw = 1.0;
        for (int i = 0; i < h.p; ++i) pw *= 2.0;
        a.w1[t] = c / pw;
    }
    a.keys = keys;
    a.koff = koff;
    return a;
}

// device buffers of one call, freed on every exit
struct Bufs {
    std::vector<void*> p;
    cudaError_t e = cudaSuccess;
    template <class T>
    T* up(const T* host, size_t n) {
        void* d = nullptr;
        if (e == cudaSuccess) e = cudaMalloc(&d, std::max<size_t>(n, 1) * sizeof(T));
        if (e == cudaSuccess) p.push_back(d);
        if (e == cudaSuccess && host && n) e = cudaMemcpy(d, host, n * sizeof(T), cudaMemcpyHostToDevice);
        return (T*)d;
    }
    template <class T>
    T* alloc(size_t n) {
        return up<T>(nullptr, n);
    }
    ~Bufs() {
        for (void* q : p) cudaFree(q);
    }
};

unsigned grid_for(long long n) {
    return (unsigned)std::max<long long>(1, std::min<long long>((n + 127) / 128, (long long)fem::sm_count() * 8));
}

}  // namespace

namespace fem {

fem_gpu_status hmr_element_t_device(const HmrDevice& h, bool truncate, int64_t count, const int32_t* level,
                                    const int64_t* idx, int32_t* ndof, const int64_t* toff, double* T,
                                    int64_t* dofs) {
    if (count <= 0) return FEM_GPU_OK;
    if (h.nloc > kHmrMaxLocal || h.dim < 2 || h.dim > 3 || h.p < 1 || h.p > 3) return FEM_GPU_BAD_ARG;
    Bufs b;
    auto* dk = b.up(reinterpret_cast<const unsigned long long*>(h.keys.data()), h.keys.size());
    auto* dko = b.up(reinterpret_cast<const long long*>(h.koff.data()), h.koff.size());
    auto* dl = b.up(level, (size_t)count);
    auto* di = b.up(reinterpret_cast<const long long*>(idx), (size_t)count * 3);
    auto* dn = b.alloc<int>((size_t)count);
    if (b.e != cudaSuccess) return FEM_GPU_CUDA_ERROR;
    const HmrArgs a = make_args(h, dk, dko);
    if (!T) {
        hmr_count_kernel<<<grid_for(count), 128>>>(a, truncate, count, dl, di, dn);
    } else {
        const long long total = toff[count];
        auto* dt = b.alloc<double>((size_t)total);
        auto* dof = b.alloc<long long>((size_t)(total / std::max(h.nloc, 1)) * 4);
        auto* dto = b.up(reinterpret_cast<const long long*>(toff), (size_t)count + 1);
        if (b.e == cudaSuccess) b.e = cudaMemcpy(dn, ndof, (size_t)count * sizeof(int), cudaMemcpyHostToDevice);
        if (b.e != cudaSuccess) return FEM_GPU_CUDA_ERROR;
        hmr_fill_kernel<<<grid_for(count), 128>>>(a, truncate, count, dl, di, dto, dt, dof, dn);
        if (cudaDeviceSynchronize() != cudaSuccess) return FEM_GPU_CUDA_ERROR;
        if (cudaMemcpy(T, dt, (size_t)total * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(dofs, dof, (size_t)(total / h.nloc) * 4 * sizeof(long long), cudaMemcpyDeviceToHost) !=
                cudaSuccess)
            return FEM_GPU_CUDA_ERROR;
    }
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return FEM_GPU_CUDA_ERROR;
    if (cudaMemcpy(ndof, dn, (size_t)count * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        return FEM_GPU_CUDA_ERROR;
    for (int64_t i = 0; i < count; ++i)
        if (ndof[i] < 0) return FEM_GPU_CUDA_ERROR;
    return FEM_GPU_OK;
}

fem_gpu_status hmr_node_rows_device(const HmrDevice& h, const double* len, int64_t nfirst, const int64_t* elem,
                                    const double* x, const int32_t* level, const int64_t* idx, const int32_t* ndof,
                                    const int64_t* toff, const double* T, const int64_t* roff, double* rows) {
    if (nfirst <= 0) return FEM_GPU_OK;
    int64_t ne = 0;
    for (int64_t k = 0; k < nfirst; ++k) ne = std::max<int64_t>(ne, elem[k] + 1);
    Bufs b;
    auto* dk = b.up(reinterpret_cast<const unsigned long long*>(h.keys.data()), h.keys.size());
    auto* dko = b.up(reinterpret_cast<const long long*>(h.koff.data()), h.koff.size());
    auto* dlen = b.up(len, 3);
    auto* del = b.up(reinterpret_cast<const long long*>(elem), (size_t)nfirst);
    auto* dx = b.up(x, (size_t)nfirst * h.dim);
    auto* dl = b.up(level, (size_t)ne);
    auto* di = b.up(reinterpret_cast<const long long*>(idx), (size_t)ne * 3);
    auto* dn = b.up(ndof, (size_t)ne);
    auto* dto = b.up(reinterpret_cast<const long long*>(toff), (size_t)ne + 1);
    auto* dt = b.up(T, (size_t)toff[ne]);
    auto* dro = b.up(reinterpret_cast<const long long*>(roff), (size_t)nfirst + 1);
    auto* dr = b.alloc<double>((size_t)roff[nfirst]);
    if (b.e != cudaSuccess) return FEM_GPU_CUDA_ERROR;
    const HmrArgs a = make_args(h, dk, dko);
    hmr_rows_kernel<<<grid_for(nfirst), 128>>>(a, dlen, nfirst, del, dx, dl, di, dn, dto, dt, dro, dr);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return FEM_GPU_CUDA_ERROR;
    if (cudaMemcpy(rows, dr, (size_t)roff[nfirst] * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
        return FEM_GPU_CUDA_ERROR;
    return FEM_GPU_OK;
}

}  // namespace fem
