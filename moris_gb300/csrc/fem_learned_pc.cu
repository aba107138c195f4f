// fem_learned_pc.cu -- learned coarse-grid correction for PCG (config 5).
//
// The preconditioner is M(r) = D^-1 r + P f_theta(R r / s) * s,  s = ||R r||:
//   R, P  trilinear restriction / prolongation between the (n+1)^3 node grid
//         of a uniform linear-B-spline hex mesh and a grid coarsened by F
//         (P interpolates coarse node values, R = P^T), per displacement
//         component of the type-major adof vector;
//   f     a 4-layer 3D convolution net on the coarse grid: channels
//         4 (3 residual components + log10 density / 3) -> 32 -> 32 -> 32 -> 3,
//         3x3x3 taps, zero padding, ReLU between layers, no biases (so f is
//         positively homogeneous and the scaling by s is exact).
// Weights are kept as FP32 masters and used as BF16; activations are BF16,
// accumulation FP32.  Forward and data-gradient convolutions are implicit
// GEMMs on the 5th-generation tensor cores (tcgen05.mma with TMEM
// accumulators and TMA-fed operand tiles, fem_conv_umma.cuh): M = 128 voxels,
// N = output channels, K = 27 taps x input channels.  The warp-level
// mma.sync m16n8k16 kernel below stays as the reference of the tensor-core
// path in the tests (FEM_CNN_CONV_KERNEL selects it).  The weight gradient is
// an FP32 reduction over voxels.  Training (Adam) runs on the GPU; the
// flexible CG that uses the net is fem_gpu_fcg.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <chrono>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include <mutex>

#include "fem_conv_umma.cuh"
#include "fem_internal.hpp"
#include "fem_spmv.cuh"

namespace {

constexpr int kLayers = 4;
constexpr int kCin[kLayers] = {4, 32, 32, 32};
constexpr int kCout[kLayers] = {32, 32, 32, 3};
constexpr int kPad = 16;  // every channel dimension is padded to a multiple of 16

__host__ __device__ constexpr int pad16(int c) { return (c + 15) / 16 * 16; }

int64_t layer_weights(int l) { return 27LL * kCin[l] * kCout[l]; }

// ---------------------------------------------------------------------------
// tensor-core implicit-GEMM convolution
struct ConvArgs {
    int nb;                       // samples
    int n;                        // grid edge (n^3 voxels per sample)
    int cin, cout;                // padded channel counts (multiples of 16)
    const __nv_bfloat16* in;      // [nb*V][cin]
    const __nv_bfloat16* w;       // [27][cout][cin]
    int sign;                     // +1: in[v + off_k] (forward); -1: in[v - off_k] (data gradient)
    int relu;                     // ReLU on the output
    const __nv_bfloat16* mask;    // [nb*V][cout]: output *= (mask > 0) (nullable)
    __nv_bfloat16* out_bf;        // [nb*V][cout] (nullable)
    float* out_f;                 // [nb*V][cout] (nullable)
};

__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, const uint32_t* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// one warp: 16 voxels x all output channels (cout <= 32 -> up to 4 n-tiles)
__global__ void conv_mma_kernel(ConvArgs p) {
    const int64_t V = (int64_t)p.n * p.n * p.n;
    const int64_t total = (int64_t)p.nb * V;
    const int64_t tile = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (tile * 16 >= total) return;
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    int64_t vrow[2] = {tile * 16 + g, tile * 16 + g + 8};
    int xyz[2][3], sample[2];
    bool live[2];
    for (int h = 0; h < 2; ++h) {
        live[h] = vrow[h] < total;
        const int64_t v = live[h] ? vrow[h] : 0;
        sample[h] = (int)(v / V);
        const int64_t loc = v - (int64_t)sample[h] * V;
        xyz[h][0] = (int)(loc % p.n);
        xyz[h][1] = (int)((loc / p.n) % p.n);
        xyz[h][2] = (int)(loc / ((int64_t)p.n * p.n));
    }
    const int ntiles = p.cout / 8;
    float acc[4][4];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    for (int k = 0; k < 27; ++k) {
        const int off[3] = {(k % 3 - 1) * p.sign, ((k / 3) % 3 - 1) * p.sign, (k / 9 - 1) * p.sign};
        int64_t nbr[2];
        bool ok[2];
        for (int h = 0; h < 2; ++h) {
            const int x = xyz[h][0] + off[0], y = xyz[h][1] + off[1], z = xyz[h][2] + off[2];
            ok[h] = live[h] && x >= 0 && y >= 0 && z >= 0 && x < p.n && y < p.n && z < p.n;
            nbr[h] = ok[h] ? (int64_t)sample[h] * V + x + (int64_t)p.n * (y + (int64_t)p.n * z) : 0;
        }
        for (int kc = 0; kc < p.cin; kc += 16) {
            uint32_t a[4];
            const uint32_t* r0 = reinterpret_cast<const uint32_t*>(p.in + nbr[0] * p.cin + kc);
            const uint32_t* r1 = reinterpret_cast<const uint32_t*>(p.in + nbr[1] * p.cin + kc);
            a[0] = ok[0] ? r0[t] : 0u;
            a[1] = ok[1] ? r1[t] : 0u;
            a[2] = ok[0] ? r0[t + 4] : 0u;
            a[3] = ok[1] ? r1[t + 4] : 0u;
            for (int nt = 0; nt < ntiles; ++nt) {
                const uint32_t* wr = reinterpret_cast<const uint32_t*>(p.w + ((int64_t)k * p.cout + nt * 8 + g) * p.cin + kc);
                uint32_t b[2] = {__ldg(wr + t), __ldg(wr + t + 4)};
                mma_bf16(acc[nt], a, b);
            }
        }
    }
    for (int nt = 0; nt < ntiles; ++nt)
        for (int h = 0; h < 2; ++h) {
            if (!live[h]) continue;
            const int c = nt * 8 + t * 2;
            float v0 = acc[nt][2 * h], v1 = acc[nt][2 * h + 1];
            if (p.relu) {
                v0 = fmaxf(v0, 0.f);
                v1 = fmaxf(v1, 0.f);
            }
            const int64_t o = vrow[h] * p.cout + c;
            if (p.mask) {
                if (!(__bfloat162float(p.mask[o]) > 0.f)) v0 = 0.f;
                if (!(__bfloat162float(p.mask[o + 1]) > 0.f)) v1 = 0.f;
            }
            if (p.out_bf) {
                p.out_bf[o] = __float2bfloat16(v0);
                p.out_bf[o + 1] = __float2bfloat16(v1);
            }
            if (p.out_f) {
                p.out_f[o] = v0;
                p.out_f[o + 1] = v1;
            }
        }
}

// dW[k][co][ci] += sum_v g[v][co] * in[v + off_k][ci]   (FP32 reduction)
constexpr int kWgChunk = 64;
__global__ void conv_wgrad_kernel(int nb, int n, int cin, int cout, int cin_real, int cout_real,
                                  const __nv_bfloat16* in, const __nv_bfloat16* gout, float* dw, int voxels_per_block) {
    const int k = blockIdx.y;
    const int64_t V = (int64_t)n * n * n, total = (int64_t)nb * V;
    const int off[3] = {k % 3 - 1, (k / 3) % 3 - 1, k / 9 - 1};
    __shared__ float gs[kWgChunk][32];
    __shared__ float is[kWgChunk][33];
    const int tid = threadIdx.x;
    // thread -> (co, 4 consecutive ci)
    const int co = tid / 8, ci0 = (tid % 8) * 4;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    const int64_t v_begin = (int64_t)blockIdx.x * voxels_per_block;
    const int64_t v_end = min(total, v_begin + voxels_per_block);
    for (int64_t v0 = v_begin; v0 < v_end; v0 += kWgChunk) {
        for (int i = tid; i < kWgChunk * 32; i += blockDim.x) {
            const int r = i / 32, c = i % 32;
            const int64_t v = v0 + r;
            float gv = 0.f, iv = 0.f;
            if (v < v_end) {
                if (c < cout) gv = __bfloat162float(gout[v * cout + c]);
                const int s = (int)(v / V);
                const int64_t loc = v - (int64_t)s * V;
                const int x = (int)(loc % n) + off[0], y = (int)((loc / n) % n) + off[1],
                          z = (int)(loc / ((int64_t)n * n)) + off[2];
                if (c < cin && x >= 0 && y >= 0 && z >= 0 && x < n && y < n && z < n)
                    iv = __bfloat162float(in[((int64_t)s * V + x + (int64_t)n * (y + (int64_t)n * z)) * cin + c]);
            }
            gs[r][c] = gv;
            is[r][c] = iv;
        }
        __syncthreads();
        for (int r = 0; r < kWgChunk; ++r) {
            const float gv = gs[r][co];
            for (int j = 0; j < 4; ++j) acc[j] = fmaf(gv, is[r][ci0 + j], acc[j]);
        }
        __syncthreads();
    }
    if (co < cout_real)
        for (int j = 0; j < 4; ++j)
            if (ci0 + j < cin_real) atomicAdd(dw + ((int64_t)k * cout_real + co) * cin_real + ci0 + j, acc[j]);
}

// master FP32 [27][cout][cin] -> BF16 padded forward [27][coutp][cinp] and
// data-gradient [27][cinp][coutp] (transposed)
__global__ void pack_weights_kernel(const float* wm, int cin, int cout, __nv_bfloat16* wf, __nv_bfloat16* wt) {
    const int cinp = pad16(cin), coutp = pad16(cout);
    const int64_t total = 27LL * cinp * coutp;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(i / ((int64_t)cinp * coutp));
        const int rem = (int)(i % ((int64_t)cinp * coutp));
        const int co = rem / cinp, ci = rem % cinp;
        const float v = (co < cout && ci < cin) ? wm[((int64_t)k * cout + co) * cin + ci] : 0.f;
        wf[((int64_t)k * coutp + co) * cinp + ci] = __float2bfloat16(v);
        wt[((int64_t)k * cinp + ci) * coutp + co] = __float2bfloat16(v);
    }
}

__global__ void adam_kernel(int64_t n, float* w, const float* g, float* m, float* v, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// MSE loss over the 3 output channels and its gradient (BF16, padded)
__global__ void loss_kernel(int64_t voxels, int coutp, const float* y, const float* target, __nv_bfloat16* dy,
                            float scale, double* loss) {
    double acc = 0.0;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < voxels; v += (int64_t)gridDim.x * blockDim.x) {
        for (int c = 0; c < coutp; ++c) {
            float d = 0.f;
            if (c < 3) {
                d = y[v * coutp + c] - target[v * 3 + c];
                acc += (double)d * d;
            }
            dy[v * coutp + c] = __float2bfloat16(2.f * scale * d);
        }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc * scale);
}

// FP32 channels-last input [V][4] -> BF16 [V][16]
__global__ void pack_input_kernel(int64_t voxels, const float* in4, __nv_bfloat16* out) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < voxels; v += (int64_t)gridDim.x * blockDim.x)
        for (int c = 0; c < kPad; ++c) out[v * kPad + c] = __float2bfloat16(c < 4 ? in4[v * 4 + c] : 0.f);
}

}  // namespace

// ===========================================================================
struct fem_cnn {
    int n = 0, nb_max = 0;
    int64_t V = 0;
    std::vector<float> host_master;
    float* wm = nullptr;      // master weights, all layers concatenated
    float* gw = nullptr;      // gradients
    float* am = nullptr;      // Adam moments
    float* av = nullptr;
    int64_t off[kLayers + 1] = {0};
    __nv_bfloat16* wf[kLayers] = {nullptr};
    __nv_bfloat16* wt[kLayers] = {nullptr};
    __nv_bfloat16* act[kLayers + 1] = {nullptr};  // act[0] = packed input, act[1..3] hidden
    __nv_bfloat16* grad[kLayers + 1] = {nullptr};
    float* y = nullptr;       // [nb*V][16]
    double* loss = nullptr;
    int64_t step = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ready = nullptr;  // joins the net's stream to the legacy default stream
    int* d_status = nullptr;  // bounded waits of the tensor-core convolution (bit 2)
    int conv_kernel = 0;      // 0 tcgen05 (default), 1 mma.sync
    bool dirty = true;        // bf16 copies need refresh
    double out_scale = 1.0;   // the correction applied by fem_gpu_fcg is out_scale * f
};

namespace {

fem_gpu_status cnn_pack(fem_cnn* c) {
    for (int l = 0; l < kLayers; ++l)
        pack_weights_kernel<<<64, 256, 0, c->stream>>>(c->wm + c->off[l], kCin[l], kCout[l], c->wf[l], c->wt[l]);
    c->dirty = false;
    return cudaGetLastError() == cudaSuccess ? FEM_GPU_OK : FEM_GPU_CUDA_ERROR;
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// dependency on the driver library)
EncodeTiled encode_tiled() {
    static EncodeTiled fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(f);
        cudaGetLastError();
    });
    return fn;
}

// the channels-last tensor (C, x, y, z, sample) of one activation buffer and
// the box of a tile's halo block, all C channels of 16 x 10 x 3 voxels; one
// voxel's channels are one 64-byte (C = 32) or 32-byte (C = 16) row, written
// with the matching TMA swizzle (the tensor cores read the same pattern)
bool conv_tensor_map(CUtensorMap* map, const __nv_bfloat16* in, int nb, int n, int C) {
    EncodeTiled enc = encode_tiled();
    if (!enc || (C != 16 && C != 32)) return false;
    const cuuint64_t e = 2;  // bytes per BF16
    const cuuint64_t dims[5] = {(cuuint64_t)C, (cuuint64_t)n, (cuuint64_t)n, (cuuint64_t)n, (cuuint64_t)nb};
    const cuuint64_t strides[4] = {C * e, (cuuint64_t)n * C * e, (cuuint64_t)n * n * C * e,
                                   (cuuint64_t)n * n * n * C * e};
    const cuuint32_t box[5] = {(cuuint32_t)C, fem_umma::kHx, fem_umma::kHy, 3, 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<__nv_bfloat16*>(in), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, C == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// one pipeline instance per (input chunks, output channels); one CTA per SM
// (the weights and a four-block halo ring fill shared memory), persistent
// over the tiles
template <int NCHK, int COUT>
bool launch_umma_inst(const CUtensorMap& map, const fem_umma::UmmaConvArgs& a, cudaStream_t st) {
    auto kern = fem_umma::conv_umma_pipe_kernel<NCHK, COUT>;
    const size_t smem = fem_umma::pipe_smem_bytes(8 * NCHK, COUT);
    static std::once_flag attr;
    std::call_once(attr, [&] { cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); });
    const int64_t grid = std::min<int64_t>(fem_umma::num_tiles(a.nb, a.n), (int64_t)fem::sm_count());
    kern<<<(unsigned)grid, fem_umma::kPipeThreads, smem, st>>>(map, a);
    return cudaGetLastError() == cudaSuccess;
}

bool launch_umma(const CUtensorMap& map, const fem_umma::UmmaConvArgs& a, cudaStream_t st) {
    if ((a.cin != 16 && a.cin != 32) || (a.cout != 16 && a.cout != 32) || (a.sign != 1 && a.sign != -1) ||
        fem_umma::num_tiles(a.nb, a.n) >= (1ll << 31))
        return false;
    if (a.cin == 16) return a.cout == 16 ? launch_umma_inst<2, 16>(map, a, st) : launch_umma_inst<2, 32>(map, a, st);
    return a.cout == 16 ? launch_umma_inst<4, 16>(map, a, st) : launch_umma_inst<4, 32>(map, a, st);
}

bool conv(fem_cnn* c, int nb, const __nv_bfloat16* in, int cin, int cout, const __nv_bfloat16* w, int sign, int relu,
          const __nv_bfloat16* mask, __nv_bfloat16* out_bf, float* out_f) {
    if (c->conv_kernel == 1) {
        ConvArgs a{nb, c->n, cin, cout, in, w, sign, relu, mask, out_bf, out_f};
        const int64_t tiles = ((int64_t)nb * c->V + 15) / 16;
        const int threads = 128;
        const unsigned blocks = (unsigned)((tiles * 32 + threads - 1) / threads);
        conv_mma_kernel<<<blocks, threads, 0, c->stream>>>(a);
        return cudaGetLastError() == cudaSuccess;
    }
    CUtensorMap map;
    if (!conv_tensor_map(&map, in, nb, c->n, cin)) return false;
    fem_umma::UmmaConvArgs a{nb, c->n, cin, cout, sign, relu, w, mask, out_bf, out_f, c->d_status};
    return launch_umma(map, a, c->stream);
}

// forward of nb samples already packed in act[0]
bool cnn_forward(fem_cnn* c, int nb) {
    bool ok = true;
    for (int l = 0; l < kLayers; ++l) {
        const bool last = l == kLayers - 1;
        ok &= conv(c, nb, c->act[l], pad16(kCin[l]), pad16(kCout[l]), c->wf[l], +1, last ? 0 : 1, nullptr,
                   last ? nullptr : c->act[l + 1], last ? c->y : nullptr);
    }
    return ok;
}

bool cnn_backward(fem_cnn* c, int nb) {
    bool ok = true;
    // grad[kLayers] holds dL/dy (bf16, 16 channels)
    cudaMemsetAsync(c->gw, 0, sizeof(float) * c->off[kLayers], c->stream);
    const int64_t total = (int64_t)nb * c->V;
    const int vpb = 4096;
    for (int l = kLayers - 1; l >= 0; --l) {
        dim3 grid((unsigned)((total + vpb - 1) / vpb), 27);
        conv_wgrad_kernel<<<grid, 256, 0, c->stream>>>(nb, c->n, pad16(kCin[l]), pad16(kCout[l]), kCin[l], kCout[l],
                                                       c->act[l], c->grad[l + 1], c->gw + c->off[l], vpb);
        if (l > 0)  // data gradient, masked by the ReLU of layer l-1's output
            ok &= conv(c, nb, c->grad[l + 1], pad16(kCout[l]), pad16(kCin[l]), c->wt[l], -1, 0, c->act[l],
                       c->grad[l], nullptr);
    }
    return ok;
}

// the end of a net call: a launch that failed, a CUDA error, or a bounded
// wait of the tensor-core convolution that expired (status bit 2)
fem_gpu_status cnn_finish(fem_cnn* c, cudaError_t e, bool launched) {
    if (!launched) return FEM_GPU_CUDA_ERROR;
    int st = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&st, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return FEM_GPU_CUDA_ERROR;
    if (st) {
        cudaMemset(c->d_status, 0, sizeof(int));
        return FEM_GPU_TIMEOUT;
    }
    return FEM_GPU_OK;
}

// the net runs on its own stream; its inputs are produced on the legacy default
// stream (torch's default, the solver kernels): wait for that work first
void after_default_stream(fem_cnn* c) {
    cudaEventRecord(c->ready, 0);
    cudaStreamWaitEvent(c->stream, c->ready, 0);
}

}  // namespace

// ===========================================================================
using namespace fem;

extern "C" {

fem_gpu_status fem_cnn_destroy(fem_cnn* c);

int64_t fem_cnn_num_weights(void) {
    int64_t s = 0;
    for (int l = 0; l < kLayers; ++l) s += layer_weights(l);
    return s;
}

fem_gpu_status fem_cnn_create(int32_t n, int32_t batch_max, uint64_t seed, fem_cnn** out) {
    if (!out || n < 2 || batch_max < 1) return FEM_GPU_BAD_ARG;
    auto* c = new fem_cnn;
    c->n = n;
    c->nb_max = batch_max;
    c->V = (int64_t)n * n * n;
    for (int l = 0; l < kLayers; ++l) c->off[l + 1] = c->off[l] + layer_weights(l);
    // He initialisation from a seeded splitmix64 / Box-Muller stream
    c->host_master.resize(c->off[kLayers]);
    uint64_t s = seed;
    auto next = [&]() {
        s += 0x9E3779B97F4A7C15ULL;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return (double)((z ^ (z >> 31)) >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < kLayers; ++l) {
        const double stdv = std::sqrt(2.0 / (27.0 * kCin[l])) * (l == kLayers - 1 ? 0.1 : 1.0);
        for (int64_t i = c->off[l]; i < c->off[l + 1]; ++i) {
            const double u1 = std::max(next(), 1e-300), u2 = next();
            c->host_master[i] = (float)(stdv * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
        }
    }
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ready, cudaEventDisableTiming);
    const int64_t nw = c->off[kLayers];
    const int64_t vox = (int64_t)batch_max * c->V;
    if (e == cudaSuccess) e = cudaMalloc(&c->wm, nw * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&c->gw, nw * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&c->am, nw * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&c->av, nw * sizeof(float));
    for (int l = 0; l < kLayers && e == cudaSuccess; ++l) {
        const int64_t pw = 27LL * pad16(kCin[l]) * pad16(kCout[l]);
        e = cudaMalloc(&c->wf[l], pw * sizeof(__nv_bfloat16));
        if (e == cudaSuccess) e = cudaMalloc(&c->wt[l], pw * sizeof(__nv_bfloat16));
    }
    for (int l = 0; l <= kLayers && e == cudaSuccess; ++l) {
        const int ch = l == 0 ? kPad : (l == kLayers ? kPad : 32);
        e = cudaMalloc(&c->act[l], vox * ch * sizeof(__nv_bfloat16));
        if (e == cudaSuccess) e = cudaMalloc(&c->grad[l], vox * ch * sizeof(__nv_bfloat16));
    }
    if (e == cudaSuccess) e = cudaMalloc(&c->y, vox * kPad * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&c->loss, sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&c->d_status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(c->d_status, 0, sizeof(int));
    {
        // FEM_CNN_CONV_KERNEL=mma selects the warp-level mma.sync convolution
        const char* k = std::getenv("FEM_CNN_CONV_KERNEL");
        c->conv_kernel = (k && std::string(k) == "mma") ? 1 : 0;
    }
    if (e == cudaSuccess) e = cudaMemcpy(c->wm, c->host_master.data(), nw * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(c->am, 0, nw * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(c->av, 0, nw * sizeof(float));
    if (e != cudaSuccess) {
        fem_cnn_destroy(c);
        *out = nullptr;
        return e == cudaErrorMemoryAllocation ? FEM_GPU_OUT_OF_MEMORY : FEM_GPU_CUDA_ERROR;
    }
    *out = c;
    return cnn_pack(c);
}

fem_gpu_status fem_cnn_destroy(fem_cnn* c) {
    if (!c) return FEM_GPU_BAD_ARG;
    if (c->stream) cudaStreamSynchronize(c->stream);
    cudaFree(c->wm);
    cudaFree(c->gw);
    cudaFree(c->am);
    cudaFree(c->av);
    for (int l = 0; l < kLayers; ++l) {
        cudaFree(c->wf[l]);
        cudaFree(c->wt[l]);
    }
    for (int l = 0; l <= kLayers; ++l) {
        cudaFree(c->act[l]);
        cudaFree(c->grad[l]);
    }
    cudaFree(c->y);
    cudaFree(c->loss);
    cudaFree(c->d_status);
    if (c->ready) cudaEventDestroy(c->ready);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return FEM_GPU_OK;
}

// weights: host FP32, layers concatenated, each [27][cout][cin]
fem_gpu_status fem_cnn_set_weights(fem_cnn* c, const float* w) {
    if (!c || !w) return FEM_GPU_BAD_ARG;
    const int64_t nw = c->off[kLayers];
    if (cudaMemcpy(c->wm, w, nw * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) return FEM_GPU_CUDA_ERROR;
    cudaMemset(c->am, 0, nw * sizeof(float));
    cudaMemset(c->av, 0, nw * sizeof(float));
    c->step = 0;
    return cnn_pack(c);
}

fem_gpu_status fem_cnn_set_output_scale(fem_cnn* c, double scale) {
    if (!c || !(scale > 0.0) || !std::isfinite(scale)) return FEM_GPU_BAD_ARG;
    c->out_scale = scale;
    return FEM_GPU_OK;
}

double fem_cnn_get_output_scale(const fem_cnn* c) { return c ? c->out_scale : 0.0; }

fem_gpu_status fem_cnn_get_weights(const fem_cnn* c, float* w) {
    if (!c || !w) return FEM_GPU_BAD_ARG;
    cudaStreamSynchronize(c->stream);
    return cudaMemcpy(w, c->wm, c->off[kLayers] * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess
               ? FEM_GPU_OK
               : FEM_GPU_CUDA_ERROR;
}

// forward of nb samples: in4 [nb*V][4] FP32 device, y3 [nb*V][3] FP32 device
fem_gpu_status fem_cnn_forward(fem_cnn* c, const float* in4, int32_t nb, float* y3) {
    if (!c || !in4 || !y3 || nb < 1 || nb > c->nb_max) return FEM_GPU_BAD_ARG;
    if (c->dirty) cnn_pack(c);
    const int64_t vox = (int64_t)nb * c->V;
    after_default_stream(c);
    pack_input_kernel<<<256, 256, 0, c->stream>>>(vox, in4, c->act[0]);
    const bool ok = cnn_forward(c, nb);
    cudaError_t e = cudaMemcpy2DAsync(y3, 3 * sizeof(float), c->y, kPad * sizeof(float), 3 * sizeof(float), vox,
                                      cudaMemcpyDeviceToDevice, c->stream);
    return cnn_finish(c, e, ok);
}

// loss = sum (y - target)^2 / (nb*V*3) and its weight gradient (no update);
// grad: host FP32 buffer of fem_cnn_num_weights() floats (nullable)
fem_gpu_status fem_cnn_loss_grad(fem_cnn* c, const float* in4, const float* target3, int32_t nb, double* loss,
                                 float* grad) {
    if (!c || !in4 || !target3 || nb < 1 || nb > c->nb_max) return FEM_GPU_BAD_ARG;
    if (c->dirty) cnn_pack(c);
    const int64_t vox = (int64_t)nb * c->V;
    after_default_stream(c);
    pack_input_kernel<<<256, 256, 0, c->stream>>>(vox, in4, c->act[0]);
    bool ok = cnn_forward(c, nb);
    cudaMemsetAsync(c->loss, 0, sizeof(double), c->stream);
    const float scale = 1.f / (float)(vox * 3);
    loss_kernel<<<512, 256, 0, c->stream>>>(vox, kPad, c->y, target3, c->grad[kLayers], scale, c->loss);
    ok &= cnn_backward(c, nb);
    cudaError_t e = cudaSuccess;
    if (loss) e = cudaMemcpyAsync(loss, c->loss, sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && grad)
        e = cudaMemcpyAsync(grad, c->gw, c->off[kLayers] * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    return cnn_finish(c, e, ok);
}

// one Adam step on a batch
fem_gpu_status fem_cnn_train_step(fem_cnn* c, const float* in4, const float* target3, int32_t nb, float lr,
                                  double* loss) {
    if (!c || !in4 || !target3 || nb < 1 || nb > c->nb_max || !(lr > 0.f)) return FEM_GPU_BAD_ARG;
    if (c->dirty) cnn_pack(c);
    const int64_t vox = (int64_t)nb * c->V;
    after_default_stream(c);
    pack_input_kernel<<<256, 256, 0, c->stream>>>(vox, in4, c->act[0]);
    bool ok = cnn_forward(c, nb);
    cudaMemsetAsync(c->loss, 0, sizeof(double), c->stream);
    const float scale = 1.f / (float)(vox * 3);
    loss_kernel<<<512, 256, 0, c->stream>>>(vox, kPad, c->y, target3, c->grad[kLayers], scale, c->loss);
    ok &= cnn_backward(c, nb);
    c->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)c->step), c2 = 1.f - std::pow(b2, (float)c->step);
    adam_kernel<<<128, 256, 0, c->stream>>>(c->off[kLayers], c->wm, c->gw, c->am, c->av, lr, b1, b2, 1e-8f, c1, c2);
    cnn_pack(c);
    cudaError_t e = cudaSuccess;
    if (loss) e = cudaMemcpyAsync(loss, c->loss, sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    return cnn_finish(c, e, ok);
}

// device time of each forward convolution (ms per call, averaged over reps
// calls, CUDA events on the net's stream) on the current contents of the
// activation buffers; ms[kLayers + l - 1] gets the data gradient of layer l
// (l = 1..3)
fem_gpu_status fem_cnn_profile(fem_cnn* c, int32_t nb, int32_t reps, double* ms) {
    if (!c || !ms || nb < 1 || nb > c->nb_max || reps < 1) return FEM_GPU_BAD_ARG;
    if (c->dirty) cnn_pack(c);
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess) return FEM_GPU_CUDA_ERROR;
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return FEM_GPU_CUDA_ERROR;
    }
    bool ok = cnn_forward(c, nb);  // warm-up
    for (int l = 0; l < 2 * kLayers - 1; ++l) {
        const bool fwd = l < kLayers;
        const int L = fwd ? l : l - kLayers + 1;
        const bool last = L == kLayers - 1;
        cudaEventRecord(e0, c->stream);
        for (int r = 0; r < reps; ++r) {
            if (fwd)
                ok &= conv(c, nb, c->act[L], pad16(kCin[L]), pad16(kCout[L]), c->wf[L], +1, last ? 0 : 1, nullptr,
                           last ? nullptr : c->act[L + 1], last ? c->y : nullptr);
            else
                ok &= conv(c, nb, c->grad[L + 1], pad16(kCout[L]), pad16(kCin[L]), c->wt[L], -1, 0, c->act[L],
                           c->grad[L], nullptr);
        }
        cudaEventRecord(e1, c->stream);
        cudaEventSynchronize(e1);
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        ms[l] = t / reps;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return cnn_finish(c, cudaGetLastError(), ok);
}

}  // extern "C"

// ===========================================================================
// grid transfer between the fine node grid (nf^3, type-major 3-component adof
// vector) and the coarse grid (nc^3, nf - 1 = F (nc - 1)): P = trilinear
// interpolation of coarse node values, R = P^T.
namespace {

unsigned lpc_grid(int64_t work) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((work + 255) / 256, (int64_t)sm_count() * 32));
}

__device__ __forceinline__ float hat(int d, int F) {
    const int a = d < 0 ? -d : d;
    return a >= F ? 0.f : 1.f - (float)a / (float)F;
}

// coarse channels-last [Vc][ch]: channels 0..2 = (R r) * inv_scale, the others untouched
__global__ void restrict_kernel(int nf, int nc, int F, const double* r, float* coarse, int ch, double inv_scale) {
    const int64_t Vc = (int64_t)nc * nc * nc, Vf = (int64_t)nf * nf * nf;
    for (int64_t I = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; I < Vc * 3; I += (int64_t)gridDim.x * blockDim.x) {
        const int comp = (int)(I / Vc);
        const int64_t v = I - comp * Vc;
        const int cx = (int)(v % nc), cy = (int)((v / nc) % nc), cz = (int)(v / ((int64_t)nc * nc));
        const int fx = cx * F, fy = cy * F, fz = cz * F;
        double s = 0.0;
        for (int dz = -F + 1; dz < F; ++dz) {
            const int z = fz + dz;
            if (z < 0 || z >= nf) continue;
            const float wz = hat(dz, F);
            for (int dy = -F + 1; dy < F; ++dy) {
                const int y = fy + dy;
                if (y < 0 || y >= nf) continue;
                const float wyz = wz * hat(dy, F);
                const double* row = r + comp * Vf + (int64_t)nf * (y + (int64_t)nf * z);
                for (int dx = -F + 1; dx < F; ++dx) {
                    const int x = fx + dx;
                    if (x < 0 || x >= nf) continue;
                    s += (double)(wyz * hat(dx, F)) * row[x];
                }
            }
        }
        coarse[v * ch + comp] = (float)(s * inv_scale);
    }
}

// sum of squares of channels 0..2 of a [Vc][4] coarse input
__device__ double g_lpc_sumsq;
__global__ void lpc_sumsq_kernel(int64_t Vc, const float* __restrict__ c4) {
    double acc = 0.0;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < Vc * 3; t += (int64_t)gridDim.x * blockDim.x) {
        const double v = c4[(t / 3) * 4 + t % 3];
        acc = fma(v, v, acc);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&g_lpc_sumsq, acc);
}
__global__ void lpc_scale_kernel(int64_t Vc, float* __restrict__ c4, float a) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < Vc * 3; t += (int64_t)gridDim.x * blockDim.x)
        c4[(t / 3) * 4 + t % 3] *= a;
}

// z[fine] += scale * P c   (c: coarse channels-last [Vc][3])
__global__ void prolong_add_kernel(int nf, int nc, int F, const float* c, double scale, double* z) {
    const int64_t Vf = (int64_t)nf * nf * nf;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < Vf * 3; i += (int64_t)gridDim.x * blockDim.x) {
        const int comp = (int)(i / Vf);
        const int64_t v = i - comp * Vf;
        const int x = (int)(v % nf), y = (int)((v / nf) % nf), zz = (int)(v / ((int64_t)nf * nf));
        const int X = min(x / F, nc - 2), Y = min(y / F, nc - 2), Z = min(zz / F, nc - 2);
        const float tx = (float)(x - X * F) / F, ty = (float)(y - Y * F) / F, tz = (float)(zz - Z * F) / F;
        double s = 0.0;
        for (int k = 0; k < 8; ++k) {
            const int ox = k & 1, oy = (k >> 1) & 1, oz = k >> 2;
            const float w = (ox ? tx : 1.f - tx) * (oy ? ty : 1.f - ty) * (oz ? tz : 1.f - tz);
            s += (double)w * c[((X + ox) + (int64_t)nc * ((Y + oy) + (int64_t)nc * (Z + oz))) * 3 + comp];
        }
        z[i] += scale * s;
    }
}

// coarse density channel: log10 of the normalised restriction of the nodal
// density, / 3, into channel 3 of the coarse input
__global__ void density_channel_kernel(int nf, int nc, int F, const double* rho, float* coarse) {
    const int64_t Vc = (int64_t)nc * nc * nc;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < Vc; v += (int64_t)gridDim.x * blockDim.x) {
        const int cx = (int)(v % nc), cy = (int)((v / nc) % nc), cz = (int)(v / ((int64_t)nc * nc));
        double s = 0.0, ws = 0.0;
        for (int dz = -F + 1; dz < F; ++dz)
            for (int dy = -F + 1; dy < F; ++dy)
                for (int dx = -F + 1; dx < F; ++dx) {
                    const int x = cx * F + dx, y = cy * F + dy, z = cz * F + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= nf || y >= nf || z >= nf) continue;
                    const double w = (double)hat(dx, F) * hat(dy, F) * hat(dz, F);
                    s += w * rho[x + (int64_t)nf * (y + (int64_t)nf * z)];
                    ws += w;
                }
        coarse[v * 4 + 3] = (float)(log10(fmax(s / ws, 1e-30)) / 3.0);
    }
}

// ---- flexible CG building blocks -------------------------------------------
__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ void block_sum_add(double v, double* out) {
    __shared__ double red[32];
    v = warp_sum_d(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
        v = warp_sum_d(v);
        if (lane == 0) atomicAdd(out, v);
    }
}

__global__ void fcg_spmv_dot(int64_t n, const int32_t* rp, const int32_t* ci, const double* v, const double* p,
                             double* q, double* dot) {
    const int sub = threadIdx.x % fem::kLanesPerRow;
    const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / fem::kLanesPerRow;
    const int64_t first = ((int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31)) / fem::kLanesPerRow;
    double acc = 0.0;
    for (int64_t base = first; base < n; base += groups) {  // uniform trip count per warp
        const int64_t row = base + (threadIdx.x & 31) / fem::kLanesPerRow;
        const double s = fem::csr_row_dot(n, rp, ci, v, p, row, sub);
        if (sub == 0 && row < n) {
            q[row] = s;
            acc = fma(s, p[row], acc);
        }
    }
    block_sum_add(acc, dot);
}


__global__ void csr_spmv_kernel(int64_t n, const int32_t* rp, const int32_t* ci, const double* v, const double* x,
                                double* y) {
    const int sub = threadIdx.x % fem::kLanesPerRow;
    const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / fem::kLanesPerRow;
    const int64_t first = ((int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31)) / fem::kLanesPerRow;
    for (int64_t base = first; base < n; base += groups) {
        const int64_t row = base + (threadIdx.x & 31) / fem::kLanesPerRow;
        const double s = fem::csr_row_dot(n, rp, ci, v, x, row, sub);
        if (sub == 0 && row < n) y[row] = s;
    }
}

// z = dinv r (the Jacobi part of the preconditioner)
__global__ void fcg_jacobi(int64_t n, const double* dinv, const double* r, double* z) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        z[i] = dinv[i] * r[i];
}



__global__ void fcg_diag_inv(int64_t n, const int32_t* rp, const int32_t* ci, const double* v, double* dinv) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double d = 1.0;
    int lo = rp[i], hi = rp[i + 1] - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        if (ci[mid] == i) {
            d = v[mid];
            break;
        }
        if (ci[mid] < i) lo = mid + 1;
        else hi = mid - 1;
    }
    dinv[i] = d != 0.0 ? 1.0 / d : 1.0;
}

__global__ void fcg_residual(int64_t n, const int32_t* rp, const int32_t* ci, const double* v, const double* b,
                             const double* x, double* r, double* dots) {
    const int sub = threadIdx.x % fem::kLanesPerRow;
    const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / fem::kLanesPerRow;
    const int64_t first = ((int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31)) / fem::kLanesPerRow;
    double rr = 0.0, bb = 0.0;
    for (int64_t base = first; base < n; base += groups) {
        const int64_t row = base + (threadIdx.x & 31) / fem::kLanesPerRow;
        const double s = fem::csr_row_dot(n, rp, ci, v, x, row, sub);
        if (sub == 0 && row < n) {
            const double ri = b[row] - s;
            r[row] = ri;
            rr = fma(ri, ri, rr);
            bb = fma(b[row], b[row], bb);
        }
    }
    block_sum_add(rr, dots);
    block_sum_add(bb, dots + 1);
}

constexpr int kMaxM = 16;
struct VecSet {
    const double* v[kMaxM];
};

// dots[j] += z . q_j for j < m
__global__ void fcg_multi_dot(int64_t n, const double* z, VecSet q, int m, double* dots) {
    double acc[kMaxM];
    for (int j = 0; j < kMaxM; ++j) acc[j] = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double zi = z[i];
        for (int j = 0; j < m; ++j) acc[j] = fma(zi, q.v[j][i], acc[j]);
    }
    for (int j = 0; j < m; ++j) block_sum_add(acc[j], dots + j);
}

// p = z - sum_j c_j p_j ; dots[0] += p . r (alpha numerator)
struct Coef {
    double c[kMaxM];
};
__global__ void fcg_orthogonalize(int64_t n, const double* z, VecSet pj, Coef c, int m, const double* r, double* p,
                                  double* dots) {
    double pr = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double v = z[i];
        for (int j = 0; j < m; ++j) v = fma(-c.c[j], pj.v[j][i], v);
        p[i] = v;
        pr = fma(v, r[i], pr);
    }
    block_sum_add(pr, dots);
}

// x += a p; r -= a q; dots[0] += r.r
__global__ void fcg_step(int64_t n, double a, double* x, const double* p, double* r, const double* q, double* dots) {
    double rr = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] = fma(a, p[i], x[i]);
        const double rn = fma(-a, q[i], r[i]);
        r[i] = rn;
        rr = fma(rn, rn, rr);
    }
    block_sum_add(rr, dots);
}

}  // namespace

extern "C" {

// coarse input of the net for a fine residual r: channels 0..2 = R r / ||R r||,
// channel 3 = log10(restricted density) / 3.  Returns the scale ||R r||.
fem_gpu_status fem_lpc_restrict(int32_t nf, int32_t factor, const double* r_dev, const double* rho_dev,
                                 float* coarse_dev, double* scale) {
    if (!r_dev || !coarse_dev || factor < 1 || nf < 2 || (nf - 1) % factor) return FEM_GPU_BAD_ARG;
    const int nc = (nf - 1) / factor + 1;
    const int64_t Vc = (int64_t)nc * nc * nc;
    restrict_kernel<<<lpc_grid(Vc * 3), 256>>>(nf, nc, factor, r_dev, coarse_dev, 4, 1.0);
    if (rho_dev) density_channel_kernel<<<lpc_grid(Vc), 256>>>(nf, nc, factor, rho_dev, coarse_dev);
    // the norm on the device (one double back); the library-wide accumulator
    // makes concurrent calls race, like the rest of the net's entry points
    const double zero = 0.0;
    double s2 = 0.0;
    if (cudaMemcpyToSymbol(g_lpc_sumsq, &zero, sizeof(double)) != cudaSuccess) return FEM_GPU_CUDA_ERROR;
    lpc_sumsq_kernel<<<256, 256>>>(Vc, coarse_dev);
    if (cudaMemcpyFromSymbol(&s2, g_lpc_sumsq, sizeof(double)) != cudaSuccess) return FEM_GPU_CUDA_ERROR;
    const double s = std::sqrt(s2);
    if (s > 0) lpc_scale_kernel<<<256, 256>>>(Vc, coarse_dev, (float)(1.0 / s));
    if (scale) *scale = s;
    return cudaGetLastError() == cudaSuccess ? FEM_GPU_OK : FEM_GPU_CUDA_ERROR;
}

// injection of a fine 3-component field at the coarse nodes, / scale,
// channels-last [Vc][3] (training targets)
fem_gpu_status fem_lpc_inject(int32_t nf, int32_t factor, const double* e_dev, double scale, float* target_dev) {
    if (!e_dev || !target_dev || factor < 1 || nf < 2 || (nf - 1) % factor || !(scale > 0)) return FEM_GPU_BAD_ARG;
    const int nc = (nf - 1) / factor + 1;
    const int64_t Vc = (int64_t)nc * nc * nc, Vf = (int64_t)nf * nf * nf;
    std::vector<double> e(Vf * 3);
    if (cudaMemcpy(e.data(), e_dev, Vf * 3 * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
        return FEM_GPU_CUDA_ERROR;
    std::vector<float> t(Vc * 3);
    for (int64_t v = 0; v < Vc; ++v) {
        const int64_t cx = v % nc, cy = (v / nc) % nc, cz = v / ((int64_t)nc * nc);
        const int64_t f = cx * factor + nf * (cy * factor + (int64_t)nf * cz * factor);
        for (int c = 0; c < 3; ++c) t[v * 3 + c] = (float)(e[c * Vf + f] / scale);
    }
    return cudaMemcpy(target_dev, t.data(), t.size() * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess
               ? FEM_GPU_OK
               : FEM_GPU_CUDA_ERROR;
}

// z += scale * P c (c: coarse channels-last [Vc][3])
fem_gpu_status fem_lpc_prolong_add(int32_t nf, int32_t factor, const float* coarse3, double scale, double* z) {
    if (!coarse3 || !z || factor < 1 || nf < 2 || (nf - 1) % factor) return FEM_GPU_BAD_ARG;
    prolong_add_kernel<<<lpc_grid(3 * (int64_t)nf * nf * nf), 256>>>(nf, (nf - 1) / factor + 1, factor, coarse3, scale,
                                                                    z);
    return cudaGetLastError() == cudaSuccess ? FEM_GPU_OK : FEM_GPU_CUDA_ERROR;
}

// coarse3 = scale * P^T fine, channels-last [Vc][3]
fem_gpu_status fem_lpc_prolong_transpose(int32_t nf, int32_t factor, const double* fine, double scale,
                                         float* coarse3) {
    if (!coarse3 || !fine || factor < 1 || nf < 2 || (nf - 1) % factor) return FEM_GPU_BAD_ARG;
    const int64_t nc3 = (int64_t)((nf - 1) / factor + 1) * ((nf - 1) / factor + 1) * ((nf - 1) / factor + 1);
    restrict_kernel<<<lpc_grid(3 * nc3), 256>>>(nf, (nf - 1) / factor + 1, factor, fine, coarse3, 3, scale);
    return cudaGetLastError() == cudaSuccess ? FEM_GPU_OK : FEM_GPU_CUDA_ERROR;
}

// y = A x for a CSR operator with n rows (device buffers; legacy default stream)
fem_gpu_status fem_gpu_spmv(int64_t n, const int32_t* rowptr, const int32_t* colidx, const double* vals,
                            const double* x, double* y) {
    if (n < 1 || !rowptr || !colidx || !vals || !x || !y) return FEM_GPU_BAD_ARG;
    const unsigned blocks = (unsigned)std::min<int64_t>((n * fem::kLanesPerRow + 255) / 256, (int64_t)sm_count() * 16);
    csr_spmv_kernel<<<blocks, 256>>>(n, rowptr, colidx, vals, x, y);
    return cudaGetLastError() == cudaSuccess ? FEM_GPU_OK : FEM_GPU_CUDA_ERROR;
}

static int g_fcg_depth = 8, g_fcg_window = 200;

fem_gpu_status fem_gpu_fcg_config(int32_t depth, int32_t window) {
    if (depth < 1 || depth > kMaxM - 1 || window < 1) return FEM_GPU_BAD_ARG;
    g_fcg_depth = depth;
    g_fcg_window = window;
    return FEM_GPU_OK;
}

/* Truncated flexible CG, FCG(m) (Y. Notay, SIAM J. Sci. Comput. 22 (2000)),
   with M(r) = B r + P sigma f(R r / s) s, B = D^-1 (fem_gpu_fcg) or one
   multigrid V-cycle (fem_gpu_fcg_mg): each preconditioned residual is
   A-orthogonalised against the last m search directions, so the energy norm
   of the error decreases monotonically for any correction f (for a fixed
   SPD M the method is PCG).  Plain Jacobi-PCG is the fallback: on breakdown
   (non-positive p.Ap, NaN) or stagnation (no 10 % residual reduction within
   `window` iterations) the solve continues with fem_gpu_pcg from the current
   iterate; the final relative residual is recomputed from b - A x.
   cnn == NULL runs the same loop with M = B.  With the V-cycle as B, a
   stalled learned correction (4 iterations without a 10 % reduction) is
   switched off and the solve continues with M = B before any Jacobi-PCG
   fallback.  *used_fallback: 0 none, 1 Jacobi-PCG fallback, 2 the learned
   correction was switched off.  m and window: fem_gpu_fcg_config. */
static fem_gpu_status fcg_run(fem_gpu_ctx* c, const int32_t* rowptr, const int32_t* colidx, const double* vals,
                              const double* b, double* x, fem_mg* mg, fem_cnn* cnn, int32_t factor,
                              const double* node_density, const fem_gpu_pcg_opts* opts, fem_gpu_pcg_report* rep,
                              int32_t* used_fallback) {
    if (!c || !rowptr || !colidx || !vals || !b || !x || !opts) return FEM_GPU_BAD_ARG;
    if (!c->host_final) return FEM_GPU_NOT_FINALIZED;
    const int64_t n = c->num_used * c->dim;
    const int64_t nu = c->num_used;
    const int nf = (int)std::llround(std::cbrt((double)nu));
    if (cnn) {
        if (c->dim != 3 || (int64_t)nf * nf * nf != nu || factor < 1 || (nf - 1) % factor ||
            (nf - 1) / factor + 1 != cnn->n)
            return fail(c, FEM_GPU_BAD_ARG, "fcg: learned correction needs a cubic node grid matching the net");
    }
    if (mg) {
        int32_t n0 = 0;
        if (fem_mg_level_info(mg, 0, &n0, nullptr) != FEM_GPU_OK || (int64_t)n0 * n0 * n0 != nu || c->dim != 3)
            return fail(c, FEM_GPU_BAD_ARG, "fcg: multigrid hierarchy does not match the model");
    }
    const int M = g_fcg_depth;  // truncation depth
    const auto t0 = std::chrono::steady_clock::now();
    double *r, *z, *dinv, *dots, *P, *Q;
    float *cin = nullptr, *cout = nullptr;
    std::vector<void*> bufs;
    auto alloc = [&](void** ptr, size_t bytes) {
        cudaError_t e = cudaMalloc(ptr, bytes);
        if (e == cudaSuccess) bufs.push_back(*ptr);
        return e;
    };
    cudaError_t e = alloc((void**)&r, n * 8);
    if (e == cudaSuccess) e = alloc((void**)&z, n * 8);
    if (e == cudaSuccess) e = alloc((void**)&dinv, n * 8);
    if (e == cudaSuccess) e = alloc((void**)&dots, kMaxM * 8);
    if (e == cudaSuccess) e = alloc((void**)&P, (size_t)(M + 1) * n * 8);
    if (e == cudaSuccess) e = alloc((void**)&Q, (size_t)(M + 1) * n * 8);
    if (cnn && e == cudaSuccess) {
        e = alloc((void**)&cin, cnn->V * 4 * sizeof(float));
        if (e == cudaSuccess) e = cudaMemset(cin, 0, cnn->V * 4 * sizeof(float));
        if (e == cudaSuccess) e = alloc((void**)&cout, cnn->V * 3 * sizeof(float));
    }
    auto cleanup = [&]() {
        cudaDeviceSynchronize();
        for (void* ptr : bufs) cudaFree(ptr);
    };
    if (e != cudaSuccess) {
        cleanup();
        return fail(c, FEM_GPU_OUT_OF_MEMORY, "fcg workspace");
    }
    const int tpb = 256;
    const unsigned rb = (unsigned)std::min<int64_t>((n * fem::kLanesPerRow + tpb - 1) / tpb, (int64_t)sm_count() * 16);
    const unsigned vb = (unsigned)std::min<int64_t>((n + tpb - 1) / tpb, (int64_t)sm_count() * 16);
    double hd[kMaxM];
    auto readn = [&](int k) {
        cudaMemcpy(hd, dots, k * sizeof(double), cudaMemcpyDeviceToHost);
        cudaMemset(dots, 0, kMaxM * 8);
    };
    const int nc = cnn ? cnn->n : 0;
    // with the V-cycle as base, a stalled learned correction is switched off
    // after kNetWindow iterations without a 10 % residual reduction and the
    // solve continues (directions restarted) with the V-cycle alone
    constexpr int kNetWindow = 4;
    bool net_on = cnn != nullptr;
    int net_dropped = 0;
    auto apply_m = [&]() -> bool {
        if (mg) {
            if (!mg_vcycle(mg, r, z)) return false;
        } else {
            fcg_jacobi<<<vb, tpb>>>(n, dinv, r, z);
        }
        if (!net_on) return true;
        double s = 0.0;
        // the density channel of cin was written once before the loop
        if (fem_lpc_restrict(nf, factor, r, nullptr, cin, &s) != FEM_GPU_OK) return false;
        if (s > 0.0) {
            if (fem_cnn_forward(cnn, cin, 1, cout) != FEM_GPU_OK) return false;
            prolong_add_kernel<<<lpc_grid(3 * (int64_t)nf * nf * nf), 256>>>(nf, nc, factor, cout, s * cnn->out_scale,
                                                                           z);
        }
        return cudaGetLastError() == cudaSuccess;
    };
    if (cnn && node_density) density_channel_kernel<<<lpc_grid((int64_t)nc * nc * nc), 256>>>(nf, nc, factor,
                                                                                                node_density, cin);
    cudaMemset(dots, 0, kMaxM * 8);
    fcg_diag_inv<<<(unsigned)((n + tpb - 1) / tpb), tpb>>>(n, rowptr, colidx, vals, dinv);
    fcg_residual<<<rb, tpb>>>(n, rowptr, colidx, vals, b, x, r, dots);
    readn(2);
    const double bn = std::sqrt(hd[1] > 0 ? hd[1] : 1.0);
    double rn = std::sqrt(hd[0]);
    const double tol = opts->rel_tol * bn;
    std::vector<double> pq(M + 1, 1.0);
    int it = 0, fallback = 0, stored = 0;
    bool ok = true;
    double best = rn;
    int since_best = 0;
    while (rn > tol && it < opts->max_iter) {
        ok = apply_m();
        if (!ok) break;
        // A-orthogonalise z against the last min(stored, M) directions
        const int m = std::min(stored, M);
        VecSet qs{}, ps{};
        Coef cf{};
        for (int j = 0; j < m; ++j) {
            const int slot = (it - 1 - j + (M + 1) * 4) % (M + 1);
            qs.v[j] = Q + (int64_t)slot * n;
            ps.v[j] = P + (int64_t)slot * n;
        }
        if (m > 0) {
            fcg_multi_dot<<<vb, tpb>>>(n, z, qs, m, dots);
            readn(m);
            for (int j = 0; j < m; ++j) {
                const int slot = (it - 1 - j + (M + 1) * 4) % (M + 1);
                cf.c[j] = hd[j] / pq[slot];
            }
        }
        const int cur = it % (M + 1);
        double* p = P + (int64_t)cur * n;
        double* q = Q + (int64_t)cur * n;
        fcg_orthogonalize<<<vb, tpb>>>(n, z, ps, cf, m, r, p, dots);
        readn(1);
        const double pr = hd[0];
        if (mg) {
            // the level-0 stencil of the hierarchy is the CSR's operator without indices
            if (!mg_operator(mg, p, q, dots)) {
                ok = false;
                break;
            }
        } else {
            fcg_spmv_dot<<<rb, tpb>>>(n, rowptr, colidx, vals, p, q, dots);
        }
        readn(1);
        const double pAp = hd[0];
        if (!(pAp > 0.0) || !std::isfinite(pr)) {
            fallback = 1;
            break;
        }
        pq[cur] = pAp;
        const double alpha = pr / pAp;
        fcg_step<<<vb, tpb>>>(n, alpha, x, p, r, q, dots);
        readn(1);
        rn = std::sqrt(hd[0]);
        ++it;
        ++stored;
        if (rn < 0.9 * best) {
            best = rn;
            since_best = 0;
        } else if (mg && net_on && ++since_best > kNetWindow) {
            net_on = false;
            net_dropped = 1;
            stored = 0;
            best = rn;
            since_best = 0;
        } else if (++since_best > g_fcg_window) {
            fallback = 1;
            break;
        }
    }
    if (!ok) {
        cleanup();
        return fail(c, FEM_GPU_CUDA_ERROR, "fcg: preconditioner application failed");
    }
    fem_gpu_status st = FEM_GPU_OK;
    int fb_iters = 0;
    if (fallback) {
        fem_gpu_pcg_opts o = *opts;
        o.preconditioner = 1;
        o.max_iter = std::max(1, opts->max_iter - it);
        fem_gpu_pcg_report pr{};
        cudaDeviceSynchronize();
        st = fem_gpu_pcg(c, rowptr, colidx, vals, b, x, &o, &pr, 0);
        fb_iters = pr.iterations;
    }
    // convergence test: the true residual of the final iterate
    cudaMemset(dots, 0, kMaxM * 8);
    fcg_residual<<<rb, tpb>>>(n, rowptr, colidx, vals, b, x, r, dots);
    readn(2);
    const double true_rel = std::sqrt(hd[0]) / bn;
    cleanup();
    if (rep) {
        rep->iterations = it + fb_iters;
        rep->converged = true_rel <= opts->rel_tol * 1.0001;
        rep->rel_residual = true_rel;
        rep->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    if (used_fallback) *used_fallback = fallback ? 1 : (net_dropped ? 2 : 0);
    if (st != FEM_GPU_OK && st != FEM_GPU_NOT_CONVERGED) return st;
    return true_rel <= opts->rel_tol * 1.0001 ? FEM_GPU_OK : fail(c, FEM_GPU_NOT_CONVERGED, "fcg: not converged");
}

fem_gpu_status fem_gpu_fcg(fem_gpu_ctx* c, const int32_t* rowptr, const int32_t* colidx, const double* vals,
                           const double* b, double* x, fem_cnn* cnn, int32_t factor, const double* node_density,
                           const fem_gpu_pcg_opts* opts, fem_gpu_pcg_report* rep, int32_t* used_fallback) {
    return fcg_run(c, rowptr, colidx, vals, b, x, nullptr, cnn, factor, node_density, opts, rep, used_fallback);
}

fem_gpu_status fem_gpu_fcg_mg(fem_gpu_ctx* c, const int32_t* rowptr, const int32_t* colidx, const double* vals,
                              const double* b, double* x, fem_mg* mg, fem_cnn* cnn, int32_t factor,
                              const double* node_density, const fem_gpu_pcg_opts* opts, fem_gpu_pcg_report* rep,
                              int32_t* used_fallback) {
    if (!mg) return fail(c, FEM_GPU_BAD_ARG, "fcg_mg: no multigrid hierarchy");
    return fcg_run(c, rowptr, colidx, vals, b, x, mg, cnn, factor, node_density, opts, rep, used_fallback);
}

}  // extern "C"
