// fem_conv_umma.cuh -- 3x3x3 convolution on the 5th-generation tensor cores.
//
// out[v][co] = sum_k sum_ci in[v + s*off_k][ci] * w[k][co][ci]   (s = +1 forward,
// -1 for the data gradient with the transposed weights), channels-last BF16
// activations, FP32 accumulation, as an implicit GEMM: M = 128 output voxels
// (a tile of 8 x 16 x 1 voxels of one sample, row m = 8 y + x), N = output
// channels (16 or 32), K = 16 input channels per instruction, 27 taps.
//
// Per tile the input block with a one-voxel halo, [3 z][18 y][10 x] x 8
// channels, is one TMA box per 8-channel chunk (cp.async.bulk.tensor.5d over
// the tensor (C, x, y, z, sample)); out-of-grid voxels read as zero, which is
// the convolution's zero padding.  In shared memory each chunk is [z][y][x] of
// 16-byte entries: an 8 x 16-byte run of consecutive x is exactly a core
// matrix of the no-swizzle K-major canonical layout, the 16 core matrices of
// the M tile are the 16 y rows (stride 160 bytes), and the next 8 channels are
// the next chunk -- so the A operand of tap (dx, dy, dz) is the same buffer
// with the descriptor's start address moved by dx entries, dy rows and dz
// planes, and no im2col copy exists.  The weights of all taps stay in shared
// memory in the same canonical layout ([tap][chunk][co][8 ci]).
//
// One elected thread issues the tcgen05.mma chain of a tile into a TMEM
// accumulator (128 lanes x N columns FP32) and commits it to an mbarrier; the
// four warps read their 32 lanes back with tcgen05.ld and apply ReLU / the
// ReLU mask of the data gradient, converting to BF16 and / or FP32.  CTAs are
// persistent over the tiles, the halo block is double-buffered so the next
// tile's TMA runs under the current tile's MMAs and epilogue.  Every mbarrier
// wait is bounded: on expiry the kernel records the failure in the status
// word, waits (bounded) for its copies in flight, frees its TMEM and returns.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace fem_umma {

constexpr int kTx = 8, kTy = 16;                 // output tile (x, y), one z plane
constexpr int kHx = kTx + 2, kHy = kTy + 2;      // halo block
constexpr int kChunkBytes = 3 * kHy * kHx * 16;  // one 8-channel chunk of the halo block: 8640
constexpr int kChunkStride = (kChunkBytes + 127) / 128 * 128;  // 8704: TMA destinations 128-byte aligned
constexpr int kThreads = 128;
constexpr unsigned kSpinLimit = 1u << 24;        // bounded mbarrier waits

struct UmmaConvArgs {
    int nb, n;           // samples, grid edge
    int cin, cout;       // channel counts (16 or 32)
    int sign;            // +1 forward, -1 data gradient
    int relu;
    const __nv_bfloat16* w;     // [27][cout][cin] (forward) / [27][cin][cout] (gradient) -- as packed
    const __nv_bfloat16* mask;  // [V][cout] (nullable): out *= mask > 0
    __nv_bfloat16* out_bf;      // [V][cout] (nullable)
    float* out_f;               // [V][cout] (nullable)
    int* status;                // bit 2: a bounded wait expired
};

__host__ __device__ constexpr size_t smem_bytes(int cin, int cout) {
    // weights, two halo buffers, three mbarriers and the TMEM address; 1 KB alignment slack
    return (size_t)27 * (cin / 8) * cout * 16 + 2 * (size_t)(cin / 8) * kChunkStride + 64 + 1024;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// tcgen05 shared-memory matrix descriptor, no swizzle: start, leading-dimension
// (K direction) and stride-dimension (M / N direction) byte offsets between
// core matrices, descriptor version 1
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N and M
__device__ __forceinline__ uint32_t instr_desc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// bounded wait for the phase with the given parity; false on expiry
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (unsigned i = 0; i < kSpinLimit; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_5d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            int c4, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
        "%6}], [%7];" ::"r"(dst),
        "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 32 TMEM lanes (the warp's) x 32 FP32 columns
__device__ __forceinline__ void tmem_load_32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__global__ void __launch_bounds__(kThreads, 1)
    conv_umma_kernel(const __grid_constant__ CUtensorMap in_map, UmmaConvArgs p) {
    extern __shared__ unsigned char smem_raw[];
    // 1 KB aligned base for the TMA destinations and the operand tiles
    unsigned char* smem = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int nchk = p.cin / 8, cout = p.cout;
    const uint32_t wbytes = 27u * nchk * cout * 16;
    unsigned char* wsm = smem;
    unsigned char* halo[2] = {smem + wbytes, smem + wbytes + (uint32_t)nchk * kChunkStride};
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + wbytes + 2u * nchk * kChunkStride);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 3);
    const uint32_t bar_tma[2] = {smem_u32(bars + 0), smem_u32(bars + 1)}, bar_mma = smem_u32(bars + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n = p.n;
    const int tx = (n + kTx - 1) / kTx, ty = (n + kTy - 1) / kTy;
    const int64_t ntiles = (int64_t)p.nb * n * ty * tx;

    // ---- set-up: TMEM, barriers, weights in the canonical layout ---------------
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;" ::"r"(smem_u32(tmem_slot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        mbar_init(bar_tma[0], 1);
        mbar_init(bar_tma[1], 1);
        mbar_init(bar_mma, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // w: [27][cout][cin] -> smem [27][chunk][cout][8]: 16-byte units, coalesced reads
    {
        const uint4* wg = reinterpret_cast<const uint4*>(p.w);
        uint4* ws = reinterpret_cast<uint4*>(wsm);
        const int units = 27 * cout * nchk;
        for (int u = tid; u < units; u += kThreads) {
            const int k = u / (cout * nchk), rem = u - k * cout * nchk, co = rem / nchk, c = rem - co * nchk;
            ws[(k * nchk + c) * cout + co] = wg[u];
        }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const uint32_t idesc = instr_desc(cout);
    const uint32_t wbase = smem_u32(wsm);
    const uint32_t hbase[2] = {smem_u32(halo[0]), smem_u32(halo[1])};
    bool failed = false;

    auto tile_coords = [&](int64_t t, int& x0, int& y0, int& z, int& s) {
        x0 = (int)(t % tx) * kTx;
        t /= tx;
        y0 = (int)(t % ty) * kTy;
        t /= ty;
        z = (int)(t % n);
        s = (int)(t / n);
    };
    // thread 0's bookkeeping of the asynchronous work: loads issued / waited per
    // buffer, MMA chains committed / waited
    uint32_t tma_issued[2] = {0, 0}, tma_waited[2] = {0, 0}, mma_issued = 0;
    auto issue_tma = [&](int64_t t, int b) {
        int x0, y0, z, s;
        tile_coords(t, x0, y0, z, s);
        mbar_expect_tx(bar_tma[b], (uint32_t)nchk * kChunkBytes);
        for (int c = 0; c < nchk; ++c)
            tma_load_5d(hbase[b] + (uint32_t)c * kChunkStride, &in_map, 8 * c, x0 - 1, y0 - 1, z - 1, s, bar_tma[b]);
        ++tma_issued[b];
    };

    int64_t t = blockIdx.x;
    if (tid == 0 && t < ntiles) issue_tma(t, 0);
    for (int i = 0; t < ntiles; ++i, t += gridDim.x) {
        const int b = i & 1;
        if (tid == 0) {
            if (!mbar_wait(bar_tma[b], (uint32_t)(i >> 1) & 1u)) {
                failed = true;
            } else {
                ++tma_waited[b];
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                uint32_t acc = 0;
                for (int k = 0; k < 27; ++k) {
                    const int dx = (k % 3 - 1) * p.sign, dy = ((k / 3) % 3 - 1) * p.sign, dz = (k / 9 - 1) * p.sign;
                    const uint32_t shift = (uint32_t)((((1 + dz) * kHy + (1 + dy)) * kHx + (1 + dx)) * 16);
                    for (int c = 0; c < nchk; c += 2) {
                        const uint64_t ad = smem_desc(hbase[b] + (uint32_t)c * kChunkStride + shift, kChunkStride,
                                                      kHx * 16);
                        const uint64_t bd =
                            smem_desc(wbase + (uint32_t)((k * nchk + c) * cout * 16), (uint32_t)cout * 16, 128);
                        umma_bf16(tmem, ad, bd, idesc, acc);
                        acc = 1;
                    }
                }
                umma_commit(bar_mma);
                ++mma_issued;
                // the next tile's block into the other buffer, whose MMAs (the
                // previous tile's) have completed
                if (t + gridDim.x < ntiles) issue_tma(t + gridDim.x, b ^ 1);
            }
        }
        // all threads: the accumulator of this tile
        if (__syncthreads_or(failed)) {
            failed = true;
            break;
        }
        const bool ok = mbar_wait(bar_mma, (uint32_t)i & 1u);
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        int x0, y0, z, s;
        tile_coords(t, x0, y0, z, s);
        float v[32];
        tmem_load_32(tmem + ((uint32_t)(warp * 32) << 16), v);
        const int m = warp * 32 + lane, x = x0 + (m & 7), y = y0 + (m >> 3);
        if (x < n && y < n) {
            const int64_t vox = (((int64_t)s * n + z) * n + y) * n + x;
            // static indices keep v and the packed words in registers
            if (p.relu) {
#pragma unroll
                for (int c = 0; c < 32; ++c) v[c] = fmaxf(v[c], 0.f);
            }
            if (p.mask) {
                const uint4* mk = reinterpret_cast<const uint4*>(p.mask + vox * cout);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if (q * 8 >= cout) break;
                    const uint4 m4 = mk[q];
                    const uint32_t mw[4] = {m4.x, m4.y, m4.z, m4.w};
#pragma unroll
                    for (int h = 0; h < 8; ++h) {
                        const uint16_t bits = (uint16_t)(mw[h >> 1] >> (16 * (h & 1)));
                        // a BF16 value is > 0 when its sign bit is clear, it is not +0 and not NaN
                        const bool nan = (bits & 0x7F80u) == 0x7F80u && (bits & 0x007Fu);
                        if ((bits & 0x8000u) || bits == 0 || nan) v[q * 8 + h] = 0.f;
                    }
                }
            }
            if (p.out_bf) {
                uint4* o = reinterpret_cast<uint4*>(p.out_bf + vox * cout);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if (q * 8 >= cout) break;
                    uint32_t w4[4];
#pragma unroll
                    for (int h = 0; h < 4; ++h) {
                        __nv_bfloat162 h2 = __floats2bfloat162_rn(v[q * 8 + 2 * h], v[q * 8 + 2 * h + 1]);
                        w4[h] = *reinterpret_cast<uint32_t*>(&h2);
                    }
                    o[q] = make_uint4(w4[0], w4[1], w4[2], w4[3]);
                }
            }
            if (p.out_f) {
                float4* o = reinterpret_cast<float4*>(p.out_f + vox * cout);
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    if (q * 4 >= cout) break;
                    o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();  // TMEM is free for the next tile's chain
    }
    if (failed && tid == 0) {
        atomicOr(p.status, 4);
        // let the copies and the MMA chain in flight finish (bounded) before the
        // shared memory and the TMEM are given up: the last load issued on a
        // buffer completes that buffer's phase (issued - 1), the last chain the
        // MMA barrier's phase (chains - 1)
        for (int b = 0; b < 2; ++b)
            if (tma_issued[b] > tma_waited[b]) mbar_wait(bar_tma[b], (tma_issued[b] - 1) & 1u);
        if (mma_issued) mbar_wait(bar_mma, (mma_issued - 1) & 1u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;" ::"r"(tmem));
}

}  // namespace fem_umma
