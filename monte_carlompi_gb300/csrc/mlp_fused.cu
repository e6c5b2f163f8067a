// Fused forward (inference) of the surrogate network 4 -> 256 -> 256 -> 256 -> 649
// on the 5th-generation tensor cores.
//
// One CTA (16 warps, one CTA per SM) carries 128 input rows through all four
// layers.  Every layer is a tcgen05.mma (M = 128, N = 256) from shared memory into a
// tensor-memory accumulator:
//  * operands are K-major core matrices (8 rows x 16 bytes; 128 B apart along K,
//    kdim * 16 B apart along M/N), no swizzle;
//  * the input rows (K = 4, zero-padded to 16) are written by the threads; the
//    weights come pre-packed in that layout (mcw_mlp_pack) and arrive by
//    cp.async.bulk, one 128 KB block of 256 output rows at a time, signalled through
//    an mbarrier's transaction count;
//  * the hidden epilogue (bias, SiLU, bf16) writes the next layer's A operand back
//    into the same 64 KB activation tile, so activations never leave shared memory;
//  * the output layer runs as three 256-column blocks ping-ponging between the two
//    halves of a 512-column accumulator, so the MMAs of block j + 1 overlap the
//    epilogue of block j; that epilogue transposes 32 x 16 pieces through a swizzled
//    shared-memory stage so each output row is written as a contiguous run.
// Warp w reads accumulator lanes 32 (w % 4) .. +31 (its rows) and columns
// 64 (w / 4) .. +63 of each 256-column half.  Every wait is bounded by %globaltimer
// (2 s); a timeout sets bit 1 of the error flag read by mcw_mlp_status, waits
// (bounded) for copies and MMAs still in flight, frees the tensor memory and leaves.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/mcw_mlp.h"

namespace mcw {

unsigned int *tc_err_flag();

namespace {

constexpr int FM = 128;                 // rows per CTA
constexpr int FH = MCW_MLP_HIDDEN;      // 256
constexpr int FO = MCW_MLP_OUT;         // 649
constexpr int FIN = MCW_MLP_IN;         // 4
constexpr int FK1 = 16;                 // layer-1 K, zero-padded
constexpr int kThreads = 512;
constexpr int kOutBlocks = (FO + FH - 1) / FH;       // 3 blocks of 256 output rows
constexpr int kBlockBytes = FH * FH * 2;             // 128 KB: 256 rows x 256 k bf16
constexpr int kW1Bytes = FH * FK1 * 2;               // 8 KB
constexpr int kXBytes = FM * FK1 * 2;                // 4 KB
constexpr int kActBytes = FM * FH * 2;               // 64 KB
constexpr int kStageBytes = 16 * 32 * 16 * 4;        // 32 KB: per warp 32 rows x 16 floats
constexpr size_t kSmemBytes = (size_t)kActBytes + kBlockBytes + kStageBytes;
constexpr size_t kW1Offset = (size_t)(2 + kOutBlocks) * kBlockBytes;   // W1 tile after the five blocks
constexpr uint32_t kTmemCols = 512;
constexpr unsigned long long kWaitNs = 2000000000ull;
// F32 += BF16 x BF16, both K-major, N = 256 (bits 17-22: N >> 3), M = 128 (bits 24-28: M >> 4)
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(FH >> 3) << 17) |
                            ((uint32_t)(FM >> 4) << 24);

static_assert(kW1Offset + kW1Bytes == MCW_MLP_PACK_BYTES, "packed blob layout");
static_assert(kXBytes + kW1Bytes <= kStageBytes, "layer-1 operands live in the stage region");

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Shared-memory matrix descriptor, no swizzle: start >> 4 (bits 0-13), leading byte
// offset >> 4 (bits 16-29, K-adjacent core matrices), stride byte offset >> 4
// (bits 32-45, M/N-adjacent core matrices), descriptor version 1 (bit 46).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ float silu(float z) { return __fdividef(z, 1.f + __expf(-z)); }

// Byte offset of element (row, k) in a K-major core-matrix tile whose rows are kdim long.
__host__ __device__ __forceinline__ uint32_t core_off(int row, int k, int kdim) {
    return (uint32_t)((row >> 3) * (kdim / 8) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ bool try_wait(uint64_t *bar, uint32_t phase) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done) : "r"(smem_u32(bar)), "r"(phase));
    return done != 0;
}

// Bounded wait on an mbarrier phase; false on timeout.
__device__ __forceinline__ bool wait_phase(uint64_t *bar, uint32_t phase) {
    const unsigned long long t0 = now_ns();
    while (!try_wait(bar, phase))
        if (now_ns() - t0 > kWaitNs) return false;
    return true;
}

__device__ __forceinline__ void expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" :: "r"(smem_u32(bar)), "r"(bytes));
}

__device__ __forceinline__ void bulk_copy(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n"
                 :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// acc (+)= A [128 x 16 ksteps] * B [256 x 16 ksteps]^T, K-major core matrices with rows of kdim.
__device__ __forceinline__ void issue_mma(uint32_t tmem, const unsigned char *a, const unsigned char *b, int kdim,
                                          uint64_t *bar) {
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t a0 = smem_u32(a), b0 = smem_u32(b);
    const uint32_t sbo = (uint32_t)(kdim / 8) * 128;
#pragma unroll 1
    for (int s = 0; s < kdim / 16; ++s) {
        const uint64_t da = smem_desc(a0 + s * 256, 128, sbo);
        const uint64_t db = smem_desc(b0 + s * 256, 128, sbo);
        const uint32_t accumulate = s > 0 ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
            :: "r"(tmem), "l"(da), "l"(db), "r"(kIdesc), "r"(accumulate));
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n"
                 :: "r"(smem_u32(bar)));
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
          "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
          "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n");
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

// Hidden epilogue: this warp's 32 rows x 64 columns of the accumulator half at tcol
// -> SiLU(z + b) as bf16 into the activation tile.
__device__ __forceinline__ void epilogue_hidden(uint32_t tmem, uint32_t tcol, const float *bias,
                                                unsigned char *act, int quarter, int group, int lane) {
    const int row = quarter * 32 + lane;
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
        const int c0 = group * 64 + h * 32;
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + tcol + (uint32_t)c0, v);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float4 ba = __ldg(reinterpret_cast<const float4 *>(bias + c0 + q * 8));
            const float4 bb = __ldg(reinterpret_cast<const float4 *>(bias + c0 + q * 8 + 4));
            const float bv[8] = {ba.x, ba.y, ba.z, ba.w, bb.x, bb.y, bb.z, bb.w};
            uint32_t packed[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const __nv_bfloat162 two = __floats2bfloat162_rn(silu(v[q * 8 + 2 * e] + bv[2 * e]),
                                                                 silu(v[q * 8 + 2 * e + 1] + bv[2 * e + 1]));
                packed[e] = *reinterpret_cast<const uint32_t *>(&two);
            }
            *reinterpret_cast<uint4 *>(act + core_off(row, c0 + q * 8, FH)) =
                make_uint4(packed[0], packed[1], packed[2], packed[3]);
        }
    }
}

// Output epilogue of block `blk` (output columns 256 blk ..): z + b4 through the
// warp's 32 x 16 stage (element (r, c) at r * 16 + (c ^ ((r >> 1) & 15)), free of bank
// conflicts both ways) into rows of y, 16 consecutive columns per half-warp.
__device__ __forceinline__ void epilogue_out(uint32_t tmem, uint32_t tcol, int blk, const float *b4, float *stage,
                                             float *y, int ldy, int row0, int rows, int quarter, int group,
                                             int lane) {
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
        const int c0 = group * 64 + h * 32;
        const int nb = blk * FH + c0;
        if (nb >= FO) break;
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + tcol + (uint32_t)c0, v);
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int ch = nb + half * 16;
            if (ch >= FO) break;
            const int sw = (lane >> 1) & 15;
            if (ch + 16 <= FO) {
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float4 b = __ldg(reinterpret_cast<const float4 *>(b4 + ch + q * 4));
                    stage[lane * 16 + ((q * 4 + 0) ^ sw)] = v[half * 16 + q * 4 + 0] + b.x;
                    stage[lane * 16 + ((q * 4 + 1) ^ sw)] = v[half * 16 + q * 4 + 1] + b.y;
                    stage[lane * 16 + ((q * 4 + 2) ^ sw)] = v[half * 16 + q * 4 + 2] + b.z;
                    stage[lane * 16 + ((q * 4 + 3) ^ sw)] = v[half * 16 + q * 4 + 3] + b.w;
                }
            } else {
#pragma unroll
                for (int c = 0; c < 16; ++c)
                    stage[lane * 16 + (c ^ sw)] = v[half * 16 + c] + (ch + c < FO ? __ldg(b4 + ch + c) : 0.f);
            }
            __syncwarp();
            const int c = lane & 15;
            if (ch + c < FO) {
#pragma unroll 4
                for (int i = 0; i < 16; ++i) {
                    const int r = 2 * i + (lane >> 4);
                    if (r < rows) y[(size_t)(row0 + r) * ldy + ch + c] = stage[r * 16 + (c ^ (i & 15))];
                }
            }
            __syncwarp();
        }
    }
}

__global__ void __launch_bounds__(kThreads, 1) mlp_fused_kernel(const float *x, int m, const float *b1,
                                                                const float *b2, const float *b3, const float *b4,
                                                                const unsigned char *blob, float *y, int ldy,
                                                                unsigned int *err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *act = smem;                                   // 64 KB activation tile
    unsigned char *wbuf = smem + kActBytes;                      // 128 KB weight block
    unsigned char *stage_all = smem + kActBytes + kBlockBytes;   // 32 KB: output stage
    unsigned char *xt = stage_all;                               // layer 1: 4 KB input tile ...
    unsigned char *w1t = stage_all + kXBytes;                    // ... and 8 KB W1 tile
    __shared__ __align__(8) uint64_t wbar, mbar;
    __shared__ uint32_t tmem_slot;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int quarter = warp & 3, group = warp >> 2;
    const int m0 = blockIdx.x * FM;
    const int row0 = m0 + quarter * 32;
    const int rows = min(32, max(0, m - row0));
    float *stage = reinterpret_cast<float *>(stage_all) + warp * 32 * 16;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
                     :: "r"(smem_u32(&tmem_slot)), "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(&wbar)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(&mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem = tmem_slot;
    uint32_t wphase = 0, mphase = 0;
    bool w_pending = false, m_pending = false, ok = true;
    const bool leader = threadIdx.x == 0;

    // W1 and W2 start arriving while the input tile is written
    if (leader) {
        expect_tx(&wbar, kW1Bytes + kBlockBytes);
        bulk_copy(w1t, blob + kW1Offset, kW1Bytes, &wbar);
        bulk_copy(wbuf, blob, kBlockBytes, &wbar);
    }
    w_pending = true;
    if (threadIdx.x < FM) {
        const int r = threadIdx.x, gm = m0 + r;
        float xin[FIN];
#pragma unroll
        for (int k = 0; k < FIN; ++k) xin[k] = gm < m ? x[(size_t)gm * FIN + k] : 0.f;
        const __nv_bfloat162 p0 = __floats2bfloat162_rn(xin[0], xin[1]);
        const __nv_bfloat162 p1 = __floats2bfloat162_rn(xin[2], xin[3]);
        *reinterpret_cast<uint4 *>(xt + core_off(r, 0, FK1)) =
            make_uint4(*reinterpret_cast<const uint32_t *>(&p0), *reinterpret_cast<const uint32_t *>(&p1), 0u, 0u);
        *reinterpret_cast<uint4 *>(xt + core_off(r, 8, FK1)) = make_uint4(0u, 0u, 0u, 0u);
    }
    asm volatile("fence.proxy.async.shared::cta;\n");

    // Waits below are made uniform across the CTA; a timeout ends the sequence.
#define MCW_WAIT(bar, phase, pending)                                  \
    do {                                                               \
        ok = __syncthreads_and(wait_phase(&(bar), (phase))) != 0;      \
        if (!ok) goto done;                                            \
        (phase) ^= 1u;                                                 \
        (pending) = false;                                             \
    } while (0)

    MCW_WAIT(wbar, wphase, w_pending);                       // W1, W2 landed; input tile written
    if (leader) issue_mma(tmem, xt, w1t, FK1, &mbar);        // layer 1
    m_pending = true;
    MCW_WAIT(mbar, mphase, m_pending);
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    epilogue_hidden(tmem, 0, b1, act, quarter, group, lane);
    asm volatile("fence.proxy.async.shared::cta;\n");
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();

    // layers 2 and 3: the weights of the next block arrive during the epilogue
    for (int layer = 0; layer < 2; ++layer) {
        if (layer > 0) MCW_WAIT(wbar, wphase, w_pending);
        if (leader) issue_mma(tmem, act, wbuf, FH, &mbar);
        m_pending = true;
        MCW_WAIT(mbar, mphase, m_pending);
        asm volatile("tcgen05.fence::after_thread_sync;\n");
        if (leader) {
            expect_tx(&wbar, kBlockBytes);
            bulk_copy(wbuf, blob + (size_t)(layer + 1) * kBlockBytes, kBlockBytes, &wbar);
        }
        w_pending = true;
        epilogue_hidden(tmem, 0, layer == 0 ? b2 : b3, act, quarter, group, lane);
        asm volatile("fence.proxy.async.shared::cta;\n");
        asm volatile("tcgen05.fence::before_thread_sync;\n");
        __syncthreads();
    }

    // output layer: block 0 -> columns 0-255 of tensor memory, block 1 -> 256-511, block 2 -> 0-255
    MCW_WAIT(wbar, wphase, w_pending);
    if (leader) issue_mma(tmem, act, wbuf, FH, &mbar);
    m_pending = true;
    MCW_WAIT(mbar, mphase, m_pending);
    if (leader) {
        expect_tx(&wbar, kBlockBytes);
        bulk_copy(wbuf, blob + 3 * (size_t)kBlockBytes, kBlockBytes, &wbar);
    }
    w_pending = true;
    MCW_WAIT(wbar, wphase, w_pending);
    if (leader) issue_mma(tmem + FH, act, wbuf, FH, &mbar);      // block 1 runs during block 0's epilogue
    m_pending = true;
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    epilogue_out(tmem, 0, 0, b4, stage, y, ldy, row0, rows, quarter, group, lane);
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    MCW_WAIT(mbar, mphase, m_pending);                       // block 1 done: wbuf free, columns 0-255 read
    if (leader) {
        expect_tx(&wbar, kBlockBytes);
        bulk_copy(wbuf, blob + 4 * (size_t)kBlockBytes, kBlockBytes, &wbar);
    }
    w_pending = true;
    MCW_WAIT(wbar, wphase, w_pending);
    if (leader) issue_mma(tmem, act, wbuf, FH, &mbar);           // block 2 runs during block 1's epilogue
    m_pending = true;
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    epilogue_out(tmem, FH, 1, b4, stage, y, ldy, row0, rows, quarter, group, lane);
    MCW_WAIT(mbar, mphase, m_pending);
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    epilogue_out(tmem, 0, 2, b4, stage, y, ldy, row0, rows, quarter, group, lane);
#undef MCW_WAIT

done:
    if (!ok) {
        if (leader) atomicOr(err, 2u);
        // copies and MMAs still in flight finish (bounded) before the CTA leaves
        if (w_pending) wait_phase(&wbar, wphase);
        if (m_pending) wait_phase(&mbar, mphase);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" :: "r"(tmem), "r"(kTmemCols));
    }
}

// Repack rows [row0, row0 + rows_out) of W [n, k] (row-major bf16) into a K-major
// core-matrix tile with rows of kdim; rows >= n and k >= k_in are zero.
__global__ void pack_kernel(const __nv_bfloat16 *w, int n, int k_in, int row0, int rows_out, int kdim,
                            unsigned char *tile) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;   // one 16-byte chunk: row, k8
    const int per_row = kdim / 8;
    if (c >= rows_out * per_row) return;
    const int r = c / per_row, k8 = c % per_row;
    __align__(16) __nv_bfloat16 h[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const int gr = row0 + r, gk = k8 * 8 + e;
        h[e] = (gr < n && gk < k_in) ? w[(size_t)gr * k_in + gk] : __float2bfloat16(0.f);
    }
    *reinterpret_cast<uint4 *>(tile + core_off(r, k8 * 8, kdim)) = *reinterpret_cast<const uint4 *>(h);
}

}  // namespace

}  // namespace mcw

using namespace mcw;

extern "C" {

int mcw_mlp_pack(const void *w1, const void *w2, const void *w3, const void *w4, void *blob, void *stream) {
    if (!w1 || !w2 || !w3 || !w4 || !blob) return MCW_MLP_ERR_ARG;
    if (((uintptr_t)blob & 15) != 0) return MCW_MLP_ERR_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned char *b = static_cast<unsigned char *>(blob);
    const int threads = 256;
    const int grid = (FH * (FH / 8) + threads - 1) / threads;
    const __nv_bfloat16 *w[3] = {static_cast<const __nv_bfloat16 *>(w2), static_cast<const __nv_bfloat16 *>(w3),
                                 static_cast<const __nv_bfloat16 *>(w4)};
    pack_kernel<<<grid, threads, 0, s>>>(w[0], FH, FH, 0, FH, FH, b);
    pack_kernel<<<grid, threads, 0, s>>>(w[1], FH, FH, 0, FH, FH, b + kBlockBytes);
    for (int j = 0; j < kOutBlocks; ++j)
        pack_kernel<<<grid, threads, 0, s>>>(w[2], FO, FH, j * FH, FH, FH, b + (size_t)(2 + j) * kBlockBytes);
    pack_kernel<<<(FH * (FK1 / 8) + threads - 1) / threads, threads, 0, s>>>(
        static_cast<const __nv_bfloat16 *>(w1), FH, FIN, 0, FH, FK1, b + kW1Offset);
    return cudaGetLastError() == cudaSuccess ? 0 : MCW_MLP_ERR_CUDA;
}

int mcw_mlp_forward(const float *x, int32_t m, const float *b1, const float *b2, const float *b3, const float *b4,
                    const void *blob, float *y, int32_t ldy, void *stream) {
    if (!x || !b1 || !b2 || !b3 || !b4 || !blob || !y || m < 0 || ldy < FO) return MCW_MLP_ERR_ARG;
    if ((((uintptr_t)blob | (uintptr_t)b1 | (uintptr_t)b2 | (uintptr_t)b3 | (uintptr_t)b4) & 15) != 0)
        return MCW_MLP_ERR_ARG;
    if (m == 0) return 0;
    unsigned int *err = tc_err_flag();
    if (!err) return MCW_MLP_ERR_CUDA;
    cudaError_t e = cudaFuncSetAttribute(mlp_fused_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kSmemBytes);
    if (e != cudaSuccess) return MCW_MLP_ERR_CUDA;
    mlp_fused_kernel<<<(m + FM - 1) / FM, kThreads, kSmemBytes, static_cast<cudaStream_t>(stream)>>>(
        x, m, b1, b2, b3, b4, static_cast<const unsigned char *>(blob), y, ldy, err);
    return cudaGetLastError() == cudaSuccess ? 0 : MCW_MLP_ERR_CUDA;
}

}  // extern "C"
