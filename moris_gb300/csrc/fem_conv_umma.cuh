// fem_conv_umma.cuh -- 3x3x3 convolution on the 5th-generation tensor cores.
//
// out[v][co] = sum_k sum_ci in[v + s*off_k][ci] * w[k][co][ci]   (s = +1 forward,
// -1 for the data gradient with the transposed weights), channels-last BF16
// activations, FP32 accumulation, as an implicit GEMM with the three x
// offsets of a tap row folded into N:
//
//   D[m][e][co] = sum_(ey, ez) sum_ci in[h(m) + (0, ey, ez)][ci] * W_(e, ey, ez)[co][ci]
//   out[x] = D[x - 1][-1] + D[x][0] + D[x + 1][+1]          (e = x offset)
//
// M = 128 rows m = 16 y + x' of a halo-wide block (16 x' = 14 output x plus
// one halo voxel on each side, 8 y, one z plane), N = 3 x (output channels),
// K = 16 input channels per instruction, 9 (ey, ez) offsets: 9 * cin/16
// instructions per tile instead of 27 * cin/16 with N = cout, so each A
// operand read from shared memory feeds three times the MMA work.  The x
// realignment is a lane shuffle in the epilogue (rows x' +- 1 are the
// neighbouring TMEM lanes of the same warp).
//
// Per tile the input block [3 z][10 y][16 x'] x cin channels is one TMA box
// (cp.async.bulk.tensor.5d over the channels-last tensor (C, x, y, z,
// sample)); out-of-grid voxels read as zero, which is the convolution's zero
// padding.  In shared memory each voxel is one row of cin channels (64 bytes
// for 32 channels, 32 bytes for 16), written by TMA with the 64-byte (32-byte)
// swizzle -- the K-major canonical layout the tensor cores read at full rate:
// 8-row atoms of 512 (256) bytes, the M = 128 rows of a tile's A operand
// consecutive, the second K-step of a 64-byte row 32 bytes further.  The A
// operand of offset (ey, ez) is the same buffer with the descriptor's start
// moved by ey rows of 16 voxels and ez planes -- whole atoms, so no im2col copy
// and no swizzle phase offset.  The weights stay in shared memory as rows
// [(ey, ez)][e][co] of cin channels, stored with the same swizzle, the B
// operand of one (ey, ez) being the N = 3 cout rows of the three e blocks.
//
// Each CTA is a warp-specialised persistent pipeline over its tiles: one lane
// of warp 0 streams the halo blocks through a ring of shared-memory stages
// with TMA, one lane each of warps 1 and 6 issues the tcgen05.mma chains of
// the even and odd tiles (descriptors as compile-time offsets) into four TMEM
// accumulators (all 512 columns: one CTA per SM), and warps 2..5 read their
// lane quadrant back with tcgen05.ld, add the shifted x neighbours, apply
// ReLU / the ReLU mask of the data gradient, convert to BF16 and / or FP32
// and store -- so the copies, the MMAs and the epilogue of consecutive tiles
// overlap.  Every mbarrier wait is bounded: on expiry the
// kernel records the failure in the status word, the other roles stop at
// their next wait, the copies and MMAs in flight are waited for (bounded) and
// the TMEM is freed.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace fem_umma {

constexpr int kHx = 16, kTx = kHx - 2;           // halo block x' extent, output x per tile
constexpr int kTy = 8, kHy = kTy + 2;            // output y per tile, halo block y extent
constexpr int kHaloRows = 3 * kHy * kHx;        // voxels (operand rows) of a halo block: 480
constexpr unsigned kSpinLimit = 1u << 24;        // bounded mbarrier waits
constexpr int kAccCols = 128;                    // TMEM columns per accumulator (3 cout used)

// tiles of nb samples on an n^3 grid: (sample, z, y tile, x tile)
__host__ __device__ constexpr long long num_tiles(int nb, int n) {
    return (long long)nb * n * ((n + kTy - 1) / kTy) * ((n + kTx - 1) / kTx);
}

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

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// tcgen05 shared-memory matrix descriptor of a swizzled K-major operand:
// start address, stride-dimension byte offset between 8-row atoms, descriptor
// version 1 and the layout type (4: 64-byte swizzle, 6: 32-byte swizzle); the
// leading-dimension offset is unused when one instruction's K (32 bytes) lies
// within a row, and set to 16 bytes
template <int ROW_BYTES>
__device__ __forceinline__ uint64_t smem_desc_sw(uint32_t addr) {
    static_assert(ROW_BYTES == 64 || ROW_BYTES == 32, "rows of 32 or 16 BF16 channels");
    constexpr uint64_t layout = ROW_BYTES == 64 ? 4 : 6;
    constexpr uint32_t sbo = 8 * ROW_BYTES;
    return (uint64_t)((addr >> 4) & 0x3FFFu) | (1ull << 16) | ((uint64_t)(sbo >> 4) << 32) | (1ull << 46) |
           (layout << 61);
}

// the swizzle both TMA and the tensor cores apply within an atom: the 16-byte
// chunk of a row is XORed with address bits 7.. (64-byte rows: bits 7-8, i.e.
// row / 2 mod 4; 32-byte rows: bit 7, i.e. row / 4 mod 2)
template <int ROW_BYTES>
__host__ __device__ constexpr int swizzled_chunk(int row, int chunk) {
    return ROW_BYTES == 64 ? chunk ^ ((row >> 1) & 3) : chunk ^ ((row >> 2) & 1);
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

// a bounded wait that also gives up when another role of the CTA has
// already given up (the abort word in shared memory)
__device__ __forceinline__ bool mbar_wait_or_abort(uint32_t bar, uint32_t parity, const volatile int* abort) {
    for (unsigned i = 0; i < kSpinLimit; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
        if ((i & 255u) == 255u && *abort) return false;
    }
    return false;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// issue a load of the 32 TMEM lanes of the warp's quadrant x 32 / 16 FP32
// columns without waiting for it; tmem_wait_ld() waits for all loads issued
// and ties the registers to the wait, so no use of them moves above it
__device__ __forceinline__ void tmem_ld_async(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_async(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
// an empty statement after the wait that the registers pass through
template <int N>
__device__ __forceinline__ void tmem_tie(uint32_t (&r)[N]) {
#pragma unroll
    for (int i = 0; i < N; i += 4) asm volatile("" : "+r"(r[i]), "+r"(r[i + 1]), "+r"(r[i + 2]), "+r"(r[i + 3]));
}

// the 9 (ey, ez) offsets x NCHK/2 K-steps of one tile (groups G .. G_END-1),
// descriptors as compile-time offsets from the stage's and the weights' base
// descriptors (the start address field counts 16-byte units, and every
// operand lies below 256 KB, so adding to the low word never carries out of
// the field)
template <int NCHK, int COUT, int G, int G_END>
__device__ __forceinline__ void tile_mmas(uint32_t d, uint64_t a0, uint64_t b0, uint32_t idesc) {
    if constexpr (G < G_END) {
        constexpr int ey = G % 3 - 1, ez = G / 3 - 1, row_bytes = NCHK * 16;
        constexpr uint32_t shift = (uint32_t)(((1 + ez) * kHy + (1 + ey)) * kHx * row_bytes);
#pragma unroll
        for (int ks = 0; ks < NCHK / 2; ++ks) {
            const uint64_t ad = a0 + ((shift + 32u * ks) >> 4);
            const uint64_t bd = b0 + ((uint32_t)(G * 3 * COUT * row_bytes + 32 * ks) >> 4);
            umma_bf16(d, ad, bd, idesc, (G == 0 && ks == 0) ? 0u : 1u);
        }
        tile_mmas<NCHK, COUT, G + 1, G_END>(d, a0, b0, idesc);
    }
}

constexpr int kStages = 4;  // halo blocks in flight
constexpr int kAcc = 4;     // TMEM accumulators (kAccCols columns each, all 512)
// tile i uses stage and accumulator i % 4, so the commit that completes a
// tile's MMAs also frees its stage: one barrier serves both
static_assert(kStages == kAcc, "a stage is freed by its tile's accumulator commit");
// warp 0 TMA, warp 1 MMA, warps 2..5 epilogue (one per TMEM lane quadrant)
constexpr int kPipeThreads = 224;  // + warp 6: a second MMA lane (odd tiles)

__host__ __device__ constexpr size_t pipe_smem_bytes(int cin, int cout) {
    // weights, the halo ring, kStages + 2 kAcc mbarriers, TMEM address and
    // abort word; 1 KB alignment slack and 2 KB of tail room; at least 120 KB,
    // so that a second CTA never shares the SM (each takes all 512 TMEM
    // columns, and a second allocation would wait for the first CTA to end)
    const size_t need = ((size_t)27 * cin * cout * 2 + 1023) / 1024 * 1024 + (size_t)kStages * kHaloRows * cin * 2 +
                        ((kStages + 2 * kAcc) * 8 + 16) + 1024 + 2048;
    return need > 120 * 1024 ? need : 120 * 1024;
}

// Warp-specialised persistent pipeline.  Warp 0 (one lane) streams the halo
// blocks of the CTA's tiles through a ring of kStages buffers (full barrier
// per stage; a stage is free again when its tile's accumulator is full);
// warp 1 (one lane) issues each tile's 9 * NCHK/2 MMAs into one of kAcc TMEM
// accumulators and commits them to the accumulator's full barrier; warps
// 2..5 read the accumulator of their TMEM lane quadrant, hand it back
// (accumulator empty barrier, one arrival per warp) and store the tile while
// the MMAs of the next tiles run.  With shared memory busy feeding the tensor
// cores every mbarrier operation takes a few hundred cycles, so the MMA lane
// tests the next tile's barriers between groups of the current tile's MMAs,
// while the tensor pipe still has queued work.
template <int NCHK, int COUT>
__global__ void __launch_bounds__(kPipeThreads, 1)
    conv_umma_pipe_kernel(const __grid_constant__ CUtensorMap in_map, UmmaConvArgs p) {
    constexpr int kThreads = kPipeThreads;
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    constexpr int kRow = NCHK * 16;  // bytes of one voxel's (one weight row's) cin channels
    constexpr uint32_t wbytes = (27u * COUT * kRow + 1023) / 1024 * 1024;  // the ring starts on 1 KB
    constexpr uint32_t stage_bytes = (uint32_t)kHaloRows * kRow;      // a multiple of 1 KB
    static_assert(wbytes % 1024 == 0 && stage_bytes % 1024 == 0, "swizzle atoms stay aligned");
    unsigned char* wsm = smem;
    unsigned char* ring = smem + wbytes;
    uint64_t* bars = reinterpret_cast<uint64_t*>(ring + kStages * stage_bytes);
    // bars: full[kStages], acc_full[kAcc], acc_empty[kAcc]
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + kStages + 2 * kAcc);
    volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);
    const uint32_t bar0 = smem_u32(bars);
    auto full = [&](int s) { return bar0 + 8u * (uint32_t)s; };
    auto acc_full = [&](int a) { return bar0 + 8u * (uint32_t)(kStages + a); };
    auto acc_empty = [&](int a) { return bar0 + 8u * (uint32_t)(kStages + kAcc + a); };
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n = p.n;
    const int tx = (n + kTx - 1) / kTx, ty = (n + kTy - 1) / kTy;
    const int64_t ntiles = num_tiles(p.nb, n);
    // tiles of this CTA: blockIdx.x + i * gridDim.x, i < my_tiles
    const int my_tiles = blockIdx.x < ntiles ? (int)((ntiles - 1 - blockIdx.x) / gridDim.x) + 1 : 0;

    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "n"(kAcc * kAccCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(full(s), 1);
        for (int a = 0; a < kAcc; ++a) {
            mbar_init(acc_full(a), 1);
            mbar_init(acc_empty(a), 4);
        }
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    {
        // w: [27 taps][cout][cin] (tap k = 9 kz + 3 ky + kx, offsets sign * (k. - 1))
        // -> smem rows R = ((ey, ez) * 3 + e) * cout + co of cin channels, by the
        // actual offsets (e, ey, ez), 16-byte chunks swizzled like the halo rows
        const uint4* wg = reinterpret_cast<const uint4*>(p.w);
        uint4* ws = reinterpret_cast<uint4*>(wsm);
        constexpr int units = 27 * COUT * NCHK;
        for (int d = tid; d < units; d += kThreads) {
            const int c = d % NCHK, R = d / NCHK;
            const int co = R % COUT, e = (R / COUT) % 3, g = R / (3 * COUT);
            const int kx = p.sign * (e - 1) + 1, ky = p.sign * (g % 3 - 1) + 1, kz = p.sign * (g / 3 - 1) + 1;
            const int k = (kz * 3 + ky) * 3 + kx;
            ws[R * NCHK + swizzled_chunk<kRow>(R, c)] = wg[(k * COUT + co) * NCHK + c];
        }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    // tile counts stay below 2^31 (the host rejects larger launches)
    auto tile_coords = [&](int t, int& x0, int& y0, int& z, int& s) {
        x0 = (int)(t % tx) * kTx;
        t /= tx;
        y0 = (int)(t % ty) * kTy;
        t /= ty;
        z = (int)(t % n);
        s = (int)(t / n);
    };
    auto give_up = [&]() {
        *abort = 1;
        atomicOr(p.status, 4);
    };

    int loads = 0, last_chain = -1;  // the producer's loads, an MMA lane's last committed tile
    if (warp == 0) {
        if (lane == 0) {
            for (int i = 0; i < my_tiles; ++i) {
                const int s = i % kStages;
                // the stage's previous tile (i - kStages) has used it when that
                // tile's accumulator is full
                if (i >= kStages && !mbar_wait_or_abort(acc_full(s), (uint32_t)((i / kStages) - 1) & 1u, abort)) {
                    give_up();
                    break;
                }
                int x0, y0, z, smp;
                tile_coords((int)blockIdx.x + i * (int)gridDim.x, x0, y0, z, smp);
                const uint32_t dst = smem_u32(ring) + (uint32_t)s * stage_bytes;
                mbar_expect_tx(full(s), stage_bytes);
                tma_load_5d(dst, &in_map, 0, x0 - 1, y0 - 1, z - 1, smp, full(s));
                ++loads;
            }
        }
    } else if (warp == 1 || warp == 6) {
        // two MMA lanes, even and odd tiles: a single lane issues one
        // tcgen05.mma per ~80 cycles, slower than the tensor pipe executes
        // these 128 x 3 cout x 16 instructions.  Tiles i and i + kAcc share an
        // accumulator and a stage and have the same parity, so each
        // accumulator's sequence of chains comes from one lane, in order.
        const int first = warp == 1 ? 0 : 1;
        if (lane == 0) {
            const uint32_t idesc = instr_desc(3 * COUT);
            const uint64_t b0 = smem_desc_sw<kRow>(smem_u32(wsm));
            // the barriers tile j needs before its MMAs: its block has landed
            // and its accumulator's previous tile (j - kAcc) has been read
            auto ready = [&](int j) {
                return mbar_wait_or_abort(full(j % kStages), (uint32_t)(j / kStages) & 1u, abort) &&
                       (j < kAcc || mbar_wait_or_abort(acc_empty(j % kAcc), (uint32_t)((j / kAcc) - 1) & 1u, abort));
            };
            bool ok = first >= my_tiles || ready(first);
            for (int i = first; i < my_tiles && ok; i += 2) {
                const int s = i % kStages, a = i % kAcc;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint64_t a0 = smem_desc_sw<kRow>(smem_u32(ring) + (uint32_t)s * stage_bytes);
                const uint32_t d = tmem + (uint32_t)(a * kAccCols);
                tile_mmas<NCHK, COUT, 0, 4>(d, a0, b0, idesc);
                // the next tile's barriers, behind the MMAs still queued
                if (i + 2 < my_tiles) ok = ready(i + 2);
                tile_mmas<NCHK, COUT, 4, 9>(d, a0, b0, idesc);
                umma_commit(acc_full(a));
                last_chain = i;
            }
            if (!ok) give_up();
        }
    } else {
        const int quad = warp & 3;  // the TMEM lanes this warp may access
        const int m = quad * 32 + lane, xh = m & 15;
        const int64_t V = (int64_t)n * n * n;
        // this lane's output voxel of tile i (live: inside the grid and not a
        // halo row) and its ReLU mask, fetched one tile ahead
        auto voxel = [&](int i, bool& live) {
            int x0, y0, z, smp;
            tile_coords((int)blockIdx.x + i * (int)gridDim.x, x0, y0, z, smp);
            const int x = x0 + xh - 1, y = y0 + (m >> 4);
            live = xh >= 1 && xh <= kTx && x < n && y < n;
            return (int64_t)smp * V + ((int64_t)z * n + y) * n + x;
        };
        auto fetch_mask = [&](int64_t vox, bool live, uint4 (&mk)[COUT / 8]) {
#pragma unroll
            for (int q = 0; q < COUT / 8; ++q)
                mk[q] = (p.mask && live) ? reinterpret_cast<const uint4*>(p.mask + vox * COUT)[q] : make_uint4(0, 0, 0, 0);
        };
        bool live_next = false;
        int64_t vox_next = my_tiles > 0 ? voxel(0, live_next) : 0;
        uint4 mk_next[COUT / 8];
        fetch_mask(vox_next, live_next, mk_next);
        for (int i = 0; i < my_tiles; ++i) {
            const int a = i % kAcc;
            const bool live = live_next;
            const int64_t vox = vox_next;
            uint4 mk[COUT / 8];
#pragma unroll
            for (int q = 0; q < COUT / 8; ++q) mk[q] = mk_next[q];
            if (i + 1 < my_tiles) {
                vox_next = voxel(i + 1, live_next);
                fetch_mask(vox_next, live_next, mk_next);
            }
            // lane 0 polls, the warp follows its result (tcgen05.ld needs all lanes)
            int ok = 0;
            if (lane == 0) ok = mbar_wait_or_abort(acc_full(a), (uint32_t)(i / kAcc) & 1u, abort);
            if (!__shfl_sync(0xffffffffu, ok, 0)) {
                if (lane == 0) give_up();
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t acc = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(a * kAccCols);
            // out[x'] = D[x' - 1][e = -1] + D[x'][0] + D[x' + 1][+1]: the x' +- 1
            // rows are lanes +- 1 of this warp (a warp holds two whole x' rows)
            uint32_t rm[COUT], r0[COUT], rp[COUT];
            tmem_ld_async(acc, rm);
            tmem_ld_async(acc + COUT, r0);
            tmem_ld_async(acc + 2 * COUT, rp);
            tmem_wait_ld();
            tmem_tie(rm);
            tmem_tie(r0);
            tmem_tie(rp);
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(acc_empty(a));
            float v[COUT];
#pragma unroll
            for (int c = 0; c < COUT; ++c)
                v[c] = __uint_as_float(r0[c]) + __uint_as_float(__shfl_up_sync(0xffffffffu, rm[c], 1)) +
                       __uint_as_float(__shfl_down_sync(0xffffffffu, rp[c], 1));
            if (live) {
                if (p.relu) {
#pragma unroll
                    for (int c = 0; c < COUT; ++c) v[c] = fmaxf(v[c], 0.f);
                }
                if (p.mask) {
#pragma unroll
                    for (int q = 0; q < COUT / 8; ++q) {
                        const uint32_t mw[4] = {mk[q].x, mk[q].y, mk[q].z, mk[q].w};
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
#pragma unroll
                    for (int q = 0; q < COUT / 8; ++q) {
                        uint32_t w4[4];
#pragma unroll
                        for (int h = 0; h < 4; ++h) {
                            __nv_bfloat162 h2 = __floats2bfloat162_rn(v[q * 8 + 2 * h], v[q * 8 + 2 * h + 1]);
                            w4[h] = *reinterpret_cast<uint32_t*>(&h2);
                        }
                        reinterpret_cast<uint4*>(p.out_bf + vox * COUT)[q] = make_uint4(w4[0], w4[1], w4[2], w4[3]);
                    }
                }
                if (p.out_f) {
                    float4* o = reinterpret_cast<float4*>(p.out_f + vox * COUT);
#pragma unroll
                    for (int q = 0; q < COUT / 4; ++q)
                        o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                }
            }
        }
    }
    __syncthreads();
    if (*abort) {
        // let the copies and MMA chains in flight land (bounded) before the
        // shared memory and the TMEM are given up.  A stage is reloaded only
        // after its previous block was consumed, and an accumulator rewritten
        // only after its previous tile was read, so the last operation on each
        // barrier completes the phase (count - 1) and no earlier one is pending.
        if (warp == 0 && lane == 0) {
            for (int s = 0; s < kStages; ++s) {
                const int issued = loads > s ? (loads - 1 - s) / kStages + 1 : 0;
                if (issued) mbar_wait(full(s), (uint32_t)(issued - 1) & 1u);
            }
        }
        if ((warp == 1 || warp == 6) && lane == 0 && last_chain >= 0)
            mbar_wait(acc_full(last_chain % kAcc), (uint32_t)(last_chain / kAcc) & 1u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(kAcc * kAccCols));
}

}  // namespace fem_umma
