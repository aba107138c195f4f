// fem_solver.cu -- preconditioned conjugate gradients on the assembled CSR
// operator (the reference delegates this to Trilinos AztecOO AZ_cg with
// AZ_Jacobi, SOL/DLA/src/cl_DLA_Linear_Solver_Aztec.cpp:260-355).
//
// One iteration is four launches on the context stream:
//   k1  q = A p and the partial sums of p.q            (4 lanes per CSR row)
//   k2  alpha = rz/pq; x += alpha p; r -= alpha q; z = M^-1 r; sums of r.z, r.r
//   k3  convergence test; beta = rz'/rz; p = z + beta p
//   k4  (one thread) advance the iteration counter
// Scalars live in a device ring indexed by the iteration counter, so the
// launches carry no host-side values and a chunk of iterations is captured
// once into a CUDA graph and replayed.  The host reads the done flag once
// per chunk; iterations after convergence return immediately on the device.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "fem_internal.hpp"
#include "fem_spmv.cuh"

namespace {

struct CgState {
    int it;          // current iteration
    int done;        // 1 converged, 2 breakdown
    int converged_at;
    int pad;
    double thresh2;  // (rtol * ||b||)^2
    double bn2;
    // ring of per-iteration scalars: [slot][0]=pq, [1]=rz, [2]=rr
    double ring[4][4];
};

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// block reduction of one double into *out (atomic)
__device__ __forceinline__ void block_add(double v, double* out) {
    __shared__ double red[32];
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
        v = warp_sum(v);
        if (lane == 0) atomicAdd(out, v);
    }
}

__global__ void k_diag_inv(int64_t n, const int32_t* rp, const int32_t* ci, const double* v, double* dinv,
                           int jacobi) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double d = 1.0;
    if (jacobi) {
        int lo = rp[i], hi = rp[i + 1] - 1;
        while (lo <= hi) {  // columns ascending
            const int mid = (lo + hi) >> 1;
            if (ci[mid] == i) {
                d = v[mid];
                break;
            }
            if (ci[mid] < i) lo = mid + 1;
            else hi = mid - 1;
        }
        d = (d != 0.0) ? 1.0 / d : 1.0;
    }
    dinv[i] = d;
}

// r = b - A x ; z = M^-1 r ; p = z ; accumulate r.z, r.r, b.b into slot 0
__global__ void k_init(int64_t n, const int32_t* rp, const int32_t* ci, const double* v, const double* b,
                       const double* x, double* r, double* z, double* p, const double* dinv, CgState* st) {
    const int sub = threadIdx.x % fem::kLanesPerRow;
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / fem::kLanesPerRow;
    double rz = 0.0, rr = 0.0, bb = 0.0;
    const double s = fem::csr_row_dot(n, rp, ci, v, x, row, sub);
    if (row < n) {
        if (sub == 0) {
            const double ri = b[row] - s, zi = dinv[row] * ri;
            r[row] = ri;
            z[row] = zi;
            p[row] = zi;
            rz = ri * zi;
            rr = ri * ri;
            bb = b[row] * b[row];
        }
    }
    block_add(rz, &st->ring[0][1]);
    __syncthreads();
    block_add(rr, &st->ring[0][2]);
    __syncthreads();
    block_add(bb, &st->bn2);
}

// q = A p (warp per row, grid-stride over rows so that each block adds its
// share of p.q with one atomic) and p.q into the ring
__global__ void k_spmv_pq(int64_t n, const int32_t* rp, const int32_t* ci, const double* v, const double* p,
                          double* q, CgState* st) {
    if (st->done) return;
    const int slot = st->it & 3;
    const int sub = threadIdx.x % fem::kLanesPerRow;
    const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / fem::kLanesPerRow;
    // the warp's first row; the trip count is uniform over the warp (the row
    // reduction shuffles need all 32 lanes)
    const int64_t first = ((int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31)) / fem::kLanesPerRow;
    double pq = 0.0;
    for (int64_t base = first; base < n; base += groups) {
        const int64_t row = base + (threadIdx.x & 31) / fem::kLanesPerRow;
        const double s = fem::csr_row_dot(n, rp, ci, v, p, row, sub);
        if (sub == 0 && row < n) {
            q[row] = s;
            pq = fma(s, p[row], pq);
        }
    }
    block_add(pq, &st->ring[slot][0]);
}

__global__ void k_update_xr(int64_t n, double* x, double* r, double* z, const double* p, const double* q,
                            const double* dinv, CgState* st) {
    if (st->done) return;
    const int slot = st->it & 3, nxt = (st->it + 1) & 3;
    const double alpha = st->ring[slot][1] / st->ring[slot][0];
    double rz = 0.0, rr = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] = fma(alpha, p[i], x[i]);
        const double ri = fma(-alpha, q[i], r[i]);
        r[i] = ri;
        const double zi = dinv[i] * ri;
        z[i] = zi;
        rz = fma(ri, zi, rz);
        rr = fma(ri, ri, rr);
    }
    block_add(rz, &st->ring[nxt][1]);
    __syncthreads();
    block_add(rr, &st->ring[nxt][2]);
}

__global__ void k_update_p(int64_t n, double* p, const double* z, CgState* st) {
    if (st->done) return;
    const int slot = st->it & 3, nxt = (st->it + 1) & 3;
    if (st->ring[nxt][2] <= st->thresh2) return;  // k4 records convergence
    const double beta = st->ring[nxt][1] / st->ring[slot][1];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = fma(beta, p[i], z[i]);
}

__global__ void k_advance(CgState* st, int max_iter) {
    if (st->done) return;
    const int slot = st->it & 3, nxt = (st->it + 1) & 3, nn = (st->it + 2) & 3;
    st->it += 1;
    if (st->ring[nxt][2] <= st->thresh2) {
        st->done = 1;
        st->converged_at = st->it;
    } else if (!(st->ring[nxt][1] == st->ring[nxt][1]) || st->ring[slot][0] == 0.0) {
        st->done = 2;  // breakdown (NaN or p.Ap == 0)
    } else if (st->it >= max_iter) {
        st->done = 3;
    }
    for (int k = 0; k < 4; ++k) st->ring[nn][k] = 0.0;
    (void)slot;
}

__global__ void k_set_thresh(CgState* st, double rtol) {
    const double bn2 = st->bn2 > 0.0 ? st->bn2 : 1.0;
    st->bn2 = bn2;
    st->thresh2 = rtol * rtol * bn2;
    if (st->ring[0][2] <= st->thresh2) {
        st->done = 1;
        st->converged_at = 0;
    }
}

}  // namespace

using namespace fem;

extern "C" fem_gpu_status fem_gpu_pcg(fem_gpu_ctx* c, const int32_t* rowptr, const int32_t* colidx,
                                      const double* vals, const double* b, double* x, const fem_gpu_pcg_opts* opts,
                                      fem_gpu_pcg_report* rep, uint32_t flags) {
    if (!c || !rowptr || !colidx || !vals || !b || !x || !opts) return FEM_GPU_BAD_ARG;
    if (flags & FEM_GPU_HOST_BUFFERS) return fail(c, FEM_GPU_UNSUPPORTED, "pcg takes device buffers");
    if (!c->host_final) return FEM_GPU_NOT_FINALIZED;
    if (!(opts->rel_tol > 0.0) || opts->max_iter < 1) return FEM_GPU_BAD_ARG;
    if (!c->stream && !c->stream_set) {
        cudaStream_t s;
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
            return fail(c, FEM_GPU_CUDA_ERROR, "stream create");
        c->stream = s;
        c->own_stream = true;
    }
    // stream capture needs a non-default stream: on the legacy default stream
    // the solve runs on a private stream after the default stream's work
    cudaStream_t sm = (cudaStream_t)c->stream;
    cudaStream_t own = nullptr;
    if (!sm) {
        if (cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking) != cudaSuccess)
            return fail(c, FEM_GPU_CUDA_ERROR, "stream create");
        cudaStreamSynchronize(nullptr);
        sm = own;
    }
    const int64_t n = c->num_used * c->dim;
    const auto t0 = std::chrono::steady_clock::now();
    double *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *dinv = nullptr;
    CgState* st = nullptr;
    cudaError_t e = cudaMallocAsync(&r, 5 * n * sizeof(double), sm);
    if (e == cudaSuccess) e = cudaMallocAsync(&st, sizeof(CgState), sm);
    if (e != cudaSuccess) return fail(c, FEM_GPU_OUT_OF_MEMORY, "pcg workspace");
    z = r + n;
    p = z + n;
    q = p + n;
    dinv = q + n;
    cudaMemsetAsync(st, 0, sizeof(CgState), sm);
    const int tpb = 256;
    const unsigned row_blocks = (unsigned)((n * fem::kLanesPerRow + tpb - 1) / tpb);
    const unsigned spmv_blocks = (unsigned)std::min<int64_t>(row_blocks, (int64_t)sm_count() * 16);
    const unsigned vec_blocks = (unsigned)std::min<int64_t>((n + tpb - 1) / tpb, (int64_t)sm_count() * 16);
    k_diag_inv<<<(unsigned)((n + tpb - 1) / tpb), tpb, 0, sm>>>(n, rowptr, colidx, vals, dinv,
                                                                opts->preconditioner == 1);
    k_init<<<row_blocks, tpb, 0, sm>>>(n, rowptr, colidx, vals, b, x, r, z, p, dinv, st);
    k_set_thresh<<<1, 1, 0, sm>>>(st, opts->rel_tol);
    c->launches += 3;
    // capture a chunk of iterations into a graph
    const int chunk = 32;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    e = cudaStreamBeginCapture(sm, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        for (int k = 0; k < chunk; ++k) {
            k_spmv_pq<<<spmv_blocks, tpb, 0, sm>>>(n, rowptr, colidx, vals, p, q, st);
            k_update_xr<<<vec_blocks, tpb, 0, sm>>>(n, x, r, z, p, q, dinv, st);
            k_update_p<<<vec_blocks, tpb, 0, sm>>>(n, p, z, st);
            k_advance<<<1, 1, 0, sm>>>(st, opts->max_iter);
        }
        e = cudaStreamEndCapture(sm, &graph);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    CgState hs{};
    fem_gpu_status result = FEM_GPU_OK;
    if (e == cudaSuccess) {
        for (int launched = 0; launched < opts->max_iter + chunk; launched += chunk) {
            e = cudaGraphLaunch(exec, sm);
            if (e != cudaSuccess) break;
            c->launches += 4 * chunk;
            e = cudaMemcpyAsync(&hs, st, sizeof(CgState), cudaMemcpyDeviceToHost, sm);
            if (e == cudaSuccess) e = cudaStreamSynchronize(sm);
            if (e != cudaSuccess || hs.done) break;
        }
    }
    if (e != cudaSuccess) result = fail(c, FEM_GPU_CUDA_ERROR, std::string("pcg: ") + cudaGetErrorString(e));
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    cudaFreeAsync(r, sm);
    cudaFreeAsync(st, sm);
    cudaStreamSynchronize(sm);
    if (own) cudaStreamDestroy(own);
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (rep) {
        rep->iterations = hs.done == 1 ? hs.converged_at : hs.it;
        rep->converged = hs.done == 1;
        const int slot = hs.it & 3;
        rep->rel_residual = std::sqrt(hs.ring[slot][2] / (hs.bn2 > 0 ? hs.bn2 : 1.0));
        rep->seconds = secs;
    }
    if (result != FEM_GPU_OK) return result;
    if (hs.done == 2) return fail(c, FEM_GPU_NONFINITE, "pcg breakdown");
    if (hs.done != 1) return fail(c, FEM_GPU_NOT_CONVERGED, "pcg hit max_iter");
    return FEM_GPU_OK;
}

// ---------------------------------------------------------------------------
// PCG without device allocation.
//
// Some callers cannot allocate device memory while they solve: code that runs
// inside a host callback, a signal-safe or real-time section, or a framework
// that owns a fixed device memory budget and forbids cudaMalloc/cudaFree (and
// any allocating library call) after start-up.  For them the Jacobi-PCG work
// vectors live in one file-scope device array of fixed size instead of
// stream-ordered allocations, and the iterations are launched directly (no
// graph instantiation).  The array holds the solver state (first 256 bytes)
// and the five work vectors r, z, p, q and 1/diag(A), so systems up to
// kNoAllocMaxRows rows are accepted; larger ones are rejected with
// FEM_GPU_BAD_ARG.  Every GPU that loads the library keeps this array
// (about 5.2 MB) until the process exits.  The array comes with this file's
// module, which CUDA loads lazily: fem_gpu_finalize resolves the array's
// address on the current device (noalloc_prepare), so the module is loaded
// there; after fem_gpu_finalize_host alone the first fem_gpu_pcg_noalloc call
// on a device does it.
namespace {

constexpr int64_t kNoAllocMaxRows = 131072;
constexpr int64_t kNoAllocStateDoubles = 32;  // 256 bytes for CgState
static_assert(sizeof(CgState) <= kNoAllocStateDoubles * sizeof(double), "CgState fits the state slot");

static __device__ __align__(256) double g_pcg_noalloc_scratch[kNoAllocStateDoubles + 5 * kNoAllocMaxRows];

// device address of the scratch array, resolved once per device with that
// device current (the host-side symbol is only a stand-in, never a device
// address)
constexpr int kMaxDevices = 64;
double* g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mutex;

fem_gpu_status noalloc_scratch(fem_gpu_ctx* c, double** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return fail(c, FEM_GPU_NO_DEVICE, "pcg_noalloc: no current CUDA device");
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_pcg_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(c, FEM_GPU_CUDA_ERROR, std::string("pcg_noalloc: scratch address: ") + cudaGetErrorString(e));
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return FEM_GPU_OK;
}

}  // namespace

namespace fem {
fem_gpu_status noalloc_prepare(fem_gpu_ctx* c) {
    double* p = nullptr;
    fem_gpu_status st = noalloc_scratch(c, &p);
    if (st != FEM_GPU_OK) return st;
    // with lazy loading a kernel's code is loaded at its first launch; reading
    // the attributes of the solver's kernels loads them now
    const void* kernels[] = {(const void*)k_diag_inv, (const void*)k_init,     (const void*)k_set_thresh,
                             (const void*)k_spmv_pq,  (const void*)k_update_xr, (const void*)k_update_p,
                             (const void*)k_advance};
    for (const void* k : kernels) {
        cudaFuncAttributes a;
        const cudaError_t e = cudaFuncGetAttributes(&a, k);
        if (e != cudaSuccess)
            return fail(c, FEM_GPU_CUDA_ERROR, std::string("pcg_noalloc: kernel load: ") + cudaGetErrorString(e));
    }
    return FEM_GPU_OK;
}
}  // namespace fem

extern "C" fem_gpu_status fem_gpu_pcg_noalloc(fem_gpu_ctx* c, const int32_t* rowptr, const int32_t* colidx,
                                              const double* vals, const double* b, double* x,
                                              const fem_gpu_pcg_opts* opts, fem_gpu_pcg_report* rep,
                                              uint32_t flags) {
    if (!c || !rowptr || !colidx || !vals || !b || !x || !opts) return FEM_GPU_BAD_ARG;
    if (flags & FEM_GPU_HOST_BUFFERS) return fail(c, FEM_GPU_UNSUPPORTED, "pcg_noalloc takes device buffers");
    if (!c->host_final) return FEM_GPU_NOT_FINALIZED;
    if (!(opts->rel_tol > 0.0) || opts->max_iter < 1) return FEM_GPU_BAD_ARG;
    const int64_t n = c->num_used * c->dim;
    if (n > kNoAllocMaxRows)
        return fail(c, FEM_GPU_BAD_ARG,
                    "pcg_noalloc: " + std::to_string(n) + " rows exceed the fixed scratch limit of " +
                        std::to_string(kNoAllocMaxRows) + " rows; use fem_gpu_pcg");
    double* base = nullptr;
    fem_gpu_status st = noalloc_scratch(c, &base);
    if (st != FEM_GPU_OK) return st;
    // the caller's stream, or the legacy default stream when none was set
    cudaStream_t sm = (cudaStream_t)c->stream;
    const auto t0 = std::chrono::steady_clock::now();
    CgState* cs = reinterpret_cast<CgState*>(base);
    double* r = base + kNoAllocStateDoubles;
    double* z = r + n;
    double* p = z + n;
    double* q = p + n;
    double* dinv = q + n;
    // the array keeps the previous call's contents: the state must start at zero
    cudaError_t e = cudaMemsetAsync(cs, 0, sizeof(CgState), sm);
    if (e != cudaSuccess) return fail(c, FEM_GPU_CUDA_ERROR, std::string("pcg_noalloc: ") + cudaGetErrorString(e));
    const int tpb = 256;
    const unsigned row_blocks = (unsigned)((n * fem::kLanesPerRow + tpb - 1) / tpb);
    const unsigned vec_blocks = (unsigned)std::min<int64_t>((n + tpb - 1) / tpb, (int64_t)sm_count() * 16);
    k_diag_inv<<<(unsigned)((n + tpb - 1) / tpb), tpb, 0, sm>>>(n, rowptr, colidx, vals, dinv,
                                                                opts->preconditioner == 1);
    k_init<<<row_blocks, tpb, 0, sm>>>(n, rowptr, colidx, vals, b, x, r, z, p, dinv, cs);
    k_set_thresh<<<1, 1, 0, sm>>>(cs, opts->rel_tol);
    c->launches += 3;
    CgState hs{};
    const int chunk = 32;
    for (int launched = 0; launched < opts->max_iter + chunk; launched += chunk) {
        for (int k = 0; k < chunk; ++k) {
            k_spmv_pq<<<row_blocks, tpb, 0, sm>>>(n, rowptr, colidx, vals, p, q, cs);
            k_update_xr<<<vec_blocks, tpb, 0, sm>>>(n, x, r, z, p, q, dinv, cs);
            k_update_p<<<vec_blocks, tpb, 0, sm>>>(n, p, z, cs);
            k_advance<<<1, 1, 0, sm>>>(cs, opts->max_iter);
        }
        c->launches += 4 * chunk;
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, cs, sizeof(CgState), cudaMemcpyDeviceToHost, sm);
        if (e == cudaSuccess) e = cudaStreamSynchronize(sm);
        if (e != cudaSuccess) return fail(c, FEM_GPU_CUDA_ERROR, std::string("pcg_noalloc: ") + cudaGetErrorString(e));
        if (hs.done) break;
    }
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (rep) {
        rep->iterations = hs.done == 1 ? hs.converged_at : hs.it;
        rep->converged = hs.done == 1;
        rep->rel_residual = std::sqrt(hs.ring[hs.it & 3][2] / (hs.bn2 > 0 ? hs.bn2 : 1.0));
        rep->seconds = secs;
    }
    if (hs.done == 2) return fail(c, FEM_GPU_NONFINITE, "pcg_noalloc breakdown");
    if (hs.done != 1) return fail(c, FEM_GPU_NOT_CONVERGED, "pcg_noalloc hit max_iter");
    return FEM_GPU_OK;
}

// ---------------------------------------------------------------------------
// Jacobi-PCG that also records its iterates: x after every `every`
// iterations is copied into snaps[j * n ...] (device, max_snaps slots).  The
// residual/error pairs of the learned preconditioner's training set come from
// these iterates of the solver itself.
extern "C" fem_gpu_status fem_gpu_pcg_snapshots(fem_gpu_ctx* c, const int32_t* rowptr, const int32_t* colidx,
                                                const double* vals, const double* b, double* x,
                                                const fem_gpu_pcg_opts* opts, fem_gpu_pcg_report* rep, int32_t every,
                                                double* snaps, int32_t max_snaps, int32_t* n_snaps) {
    if (!c || !rowptr || !colidx || !vals || !b || !x || !opts || every < 1 || !snaps || max_snaps < 1 || !n_snaps)
        return FEM_GPU_BAD_ARG;
    if (!c->host_final) return FEM_GPU_NOT_FINALIZED;
    if (!(opts->rel_tol > 0.0) || opts->max_iter < 1) return FEM_GPU_BAD_ARG;
    const int64_t n = c->num_used * c->dim;
    cudaStream_t sm = nullptr;
    if (cudaStreamCreateWithFlags(&sm, cudaStreamNonBlocking) != cudaSuccess)
        return fail(c, FEM_GPU_CUDA_ERROR, "stream create");
    cudaDeviceSynchronize();
    const auto t0 = std::chrono::steady_clock::now();
    double* r = nullptr;
    CgState* st = nullptr;
    cudaError_t e = cudaMallocAsync(&r, 5 * n * sizeof(double), sm);
    if (e == cudaSuccess) e = cudaMallocAsync(&st, sizeof(CgState), sm);
    if (e != cudaSuccess) {
        cudaStreamDestroy(sm);
        return fail(c, FEM_GPU_OUT_OF_MEMORY, "pcg workspace");
    }
    double *z = r + n, *p = z + n, *q = p + n, *dinv = q + n;
    cudaMemsetAsync(st, 0, sizeof(CgState), sm);
    const int tpb = 256;
    const unsigned row_blocks = (unsigned)((n * fem::kLanesPerRow + tpb - 1) / tpb);
    const unsigned spmv_blocks = (unsigned)std::min<int64_t>(row_blocks, (int64_t)sm_count() * 16);
    const unsigned vec_blocks = (unsigned)std::min<int64_t>((n + tpb - 1) / tpb, (int64_t)sm_count() * 16);
    k_diag_inv<<<(unsigned)((n + tpb - 1) / tpb), tpb, 0, sm>>>(n, rowptr, colidx, vals, dinv, opts->preconditioner == 1);
    k_init<<<row_blocks, tpb, 0, sm>>>(n, rowptr, colidx, vals, b, x, r, z, p, dinv, st);
    k_set_thresh<<<1, 1, 0, sm>>>(st, opts->rel_tol);
    CgState hs{};
    int taken = 0;
    for (int done_it = 0; done_it < opts->max_iter; done_it += every) {
        for (int k = 0; k < every; ++k) {
            k_spmv_pq<<<spmv_blocks, tpb, 0, sm>>>(n, rowptr, colidx, vals, p, q, st);
            k_update_xr<<<vec_blocks, tpb, 0, sm>>>(n, x, r, z, p, q, dinv, st);
            k_update_p<<<vec_blocks, tpb, 0, sm>>>(n, p, z, st);
            k_advance<<<1, 1, 0, sm>>>(st, opts->max_iter);
        }
        c->launches += 4 * every;
        e = cudaMemcpyAsync(&hs, st, sizeof(CgState), cudaMemcpyDeviceToHost, sm);
        if (e == cudaSuccess) e = cudaStreamSynchronize(sm);
        if (e != cudaSuccess) break;
        if (hs.done) break;
        if (taken < max_snaps) {
            e = cudaMemcpyAsync(snaps + (int64_t)taken * n, x, n * sizeof(double), cudaMemcpyDeviceToDevice, sm);
            if (e != cudaSuccess) break;
            ++taken;
        }
    }
    cudaFreeAsync(r, sm);
    cudaFreeAsync(st, sm);
    cudaStreamSynchronize(sm);
    cudaStreamDestroy(sm);
    *n_snaps = taken;
    if (rep) {
        rep->iterations = hs.done == 1 ? hs.converged_at : hs.it;
        rep->converged = hs.done == 1;
        rep->rel_residual = std::sqrt(hs.ring[hs.it & 3][2] / (hs.bn2 > 0 ? hs.bn2 : 1.0));
        rep->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    if (e != cudaSuccess) return fail(c, FEM_GPU_CUDA_ERROR, std::string("pcg snapshots: ") + cudaGetErrorString(e));
    if (hs.done == 2) return fail(c, FEM_GPU_NONFINITE, "pcg breakdown");
    if (hs.done != 1) return fail(c, FEM_GPU_NOT_CONVERGED, "pcg hit max_iter");
    return FEM_GPU_OK;
}
