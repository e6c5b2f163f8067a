// Fused forward (inference) of the surrogate network 4 -> 256 -> 256 -> 256 -> 649
// on the 5th-generation tensor cores.
//
// One CTA carries 128 input rows through all four layers; two CTAs share an SM
// (112 KB of shared memory and 256 tensor-memory columns each), so one CTA's
// epilogue runs while the other's MMAs occupy the tensor core.  Warps are
// specialised:
//  * warp 8 (producer) streams the pre-packed weights (mcw_mlp_pack) as 41 chunks of
//    at most 16 KB through a two-slot shared-memory ring with cp.async.bulk, each
//    chunk signalled through its slot's mbarrier transaction count;
//  * warp 9 (MMA) owns the tensor memory and issues tcgen05.mma (M = 128, K-major
//    core-matrix operands, no swizzle) from shared memory into it: layer 1 (K = 4
//    zero-padded to 16) and layers 2 and 3 with N = 256, the output layer as six
//    N = 128 blocks ping-ponging between the two halves of the accumulator;
//  * warps 0-7 write the input tile and run the epilogues: hidden layers (bias,
//    SiLU, bf16) write the next layer's A operand back into the 64 KB activation
//    tile, so activations never leave shared memory; output blocks are transposed
//    8 rows at a time through a small per-warp stage so that every output row is
//    written as whole 128-byte runs (a warp's 16-byte stores cover 4 rows x 128 B).
//    Epilogue warp w reads accumulator lanes 32 (w % 4) .. +31 (its rows).
// Hand-offs are mbarriers: ring full/empty, accumulator full (tcgen05.commit) and
// empty, activation tile ready.  Every wait is bounded by %globaltimer (2 s) and
// checks a CTA-wide abort flag; a timeout sets bit 1 of the error flag read by
// mcw_mlp_status, lets copies and MMAs in flight finish (bounded), frees the tensor
// memory and leaves.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/mcw_mlp.h"

namespace mcw {

unsigned int *tc_err_flag();

namespace {

constexpr int FM = 128;                 // rows per CTA
constexpr int FH = MCW_MLP_HIDDEN;      // 256
constexpr int FO = MCW_MLP_OUT;         // 649
constexpr int FIN = MCW_MLP_IN;         // 4
constexpr int FK1 = 16;                 // layer-1 K, zero-padded
#ifndef MCW_FUSED_SLOTS
#define MCW_FUSED_SLOTS 2
#endif
#ifndef MCW_FUSED_EPI_WARPS
#define MCW_FUSED_EPI_WARPS 8
#endif
#ifndef MCW_FUSED_TILES
#define MCW_FUSED_TILES 1
#endif
#ifndef MCW_FUSED_CTAS_PER_SM
#define MCW_FUSED_CTAS_PER_SM (MCW_FUSED_TILES == 1 ? 2 : 1)
#endif
constexpr int kSlots = MCW_FUSED_SLOTS;              // weight ring depth
constexpr int kEpiWarps = MCW_FUSED_EPI_WARPS;       // 8 or 16
constexpr int kCtasPerSm = MCW_FUSED_CTAS_PER_SM;
// 128-row tiles a CTA carries at once, each with its own accumulator and activation
// tile: the MMAs of one tile's next layer run while the other tile's epilogue does
constexpr int kTiles = MCW_FUSED_TILES;
static_assert(kTiles == 1 || kTiles == 2, "one or two tiles per CTA");
constexpr int kGroups = kEpiWarps / 4;               // column groups per accumulator lane quarter
constexpr int kProducerWarp = kEpiWarps, kMmaWarp = kEpiWarps + 1;
constexpr int kThreads = 32 * (kEpiWarps + 2);
constexpr int kEpiThreads = 32 * kEpiWarps;
constexpr int kOutN = 128;                            // output block width
constexpr int kOutBlocks = (FO + kOutN - 1) / kOutN;  // 6
// weight chunks, in the order the MMA warp consumes them
constexpr int kHidK = 32;                             // k per hidden-layer chunk (256 rows)
constexpr int kOutK = 64;                             // k per output chunk (128 rows)
constexpr int kHidChunks = FH / kHidK;                // 8 per hidden layer
constexpr int kOutChunks = FH / kOutK;                // 4 per output block
constexpr int kChunkBytes = 16384;
constexpr int kW1Bytes = FH * FK1 * 2;                // 8 KB, chunk 0
constexpr int kNumChunks = 1 + 2 * kHidChunks + kOutBlocks * kOutChunks;   // 41
constexpr int kXBytes = FM * FK1 * 2;                 // 4 KB
constexpr int kActBytes = FM * FH * 2;                // 64 KB
constexpr int kRingBytes = kSlots * kChunkBytes;
constexpr int kStagePitch = 36 * 4;                   // stage row: 32 floats + 16 B pad (no bank conflicts)
constexpr int kStageWarp = 8 * kStagePitch;           // 8 rows per warp
constexpr int kStageBytes = kEpiWarps * kStageWarp < 4096 ? 4096 : kEpiWarps * kStageWarp;
#ifndef MCW_FUSED_TMA_OUT
#define MCW_FUSED_TMA_OUT 1
#endif
// fp16 output through tensor stores: a warp's stage is 1 KB (8 rows x 128 bytes in the
// tensor map's 128-byte swizzle), 1024-byte aligned; columns [0, kTmaCols) go through the
// tensor map, the ragged rest (640 .. 648) through plain stores
constexpr int kStageTma = 1024;
constexpr int kTmaCols = (FO / 64) * 64;
// biases in shared memory: b1, b2, b3 (256 each), b4 zero-padded to the six 128-column blocks
constexpr int kB4Pad = 6 * 128;
constexpr int kBiasFloats = 3 * 256 + kB4Pad;
constexpr int kBiasBytes = kBiasFloats * 4;
constexpr int kHidCols = FH / kGroups;                // hidden columns per epilogue warp
constexpr int kOutCols = kOutN / kGroups;             // output-block columns per epilogue warp
static_assert(kEpiWarps % 4 == 0 && kHidCols % 32 == 0 && kOutCols % 32 == 0, "epilogue split");
static_assert(kTiles * kActBytes + kRingBytes + kStageBytes + kBiasBytes <= 227 * 1024, "shared memory");
constexpr size_t kSmemBytes = (size_t)kTiles * kActBytes + kRingBytes + kStageBytes + kBiasBytes;
constexpr uint32_t kTmemCols = 256 * kTiles;
constexpr int kSeqChunks = kTiles * kNumChunks;       // weight chunks a CTA consumes
constexpr unsigned long long kWaitNs = 2000000000ull;
constexpr uint32_t kSuspendNs = 1000000;              // a waiting thread sleeps until the phase completes or 1 ms
// F32 += BF16 x BF16, both K-major; N >> 3 in bits 17-22, M >> 4 in bits 24-28
__host__ __device__ constexpr uint32_t idesc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(FM >> 4) << 24);
}

static_assert(kHidK * FH * 2 == kChunkBytes && kOutK * kOutN * 2 == kChunkBytes, "chunk sizes");
static_assert(kW1Bytes + (kNumChunks - 1) * kChunkBytes == MCW_MLP_PACK_BYTES, "packed blob layout");
static_assert(kTiles * kXBytes <= kStageBytes, "the input tiles live in the stage region");
static_assert(kEpiWarps * kStageTma <= kStageBytes && (kTiles * kActBytes + kRingBytes) % 1024 == 0,
              "tensor-store stages: 1 KB per epilogue warp, 1024-byte aligned");

// The i-th weight chunk a CTA consumes: per layer the chunks of tile 0, then those of
// tile 1 (the order in which the MMA warp issues the layers of its tiles).
__host__ __device__ constexpr int chunk_at(int i) {
    return i < kTiles ? 0
         : i < kTiles * (1 + kHidChunks) ? 1 + (i - kTiles) % kHidChunks
         : i < kTiles * (1 + 2 * kHidChunks) ? 1 + kHidChunks + (i - kTiles * (1 + kHidChunks)) % kHidChunks
         : 1 + 2 * kHidChunks + (i - kTiles * (1 + 2 * kHidChunks)) % (kOutBlocks * kOutChunks);
}

__host__ __device__ constexpr size_t chunk_offset(int i) { return i == 0 ? 0 : kW1Bytes + (size_t)(i - 1) * kChunkBytes; }
__host__ __device__ constexpr uint32_t chunk_bytes(int i) { return i == 0 ? kW1Bytes : kChunkBytes; }

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

#ifndef MCW_FUSED_SILU_TANH
#define MCW_FUSED_SILU_TANH 1
#endif
__device__ __forceinline__ float silu(float z) { return __fdividef(z, 1.f + __expf(-z)); }

__device__ __forceinline__ float tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// SiLU of a pair of pre-activations.  With MCW_FUSED_SILU_TANH (the default):
// z sigmoid(z) = h + h tanh(h), h = z / 2, one hardware tanh per value (relative
// error about 2^-11, below the bf16 rounding of the stored activation) and packed
// FP32 pair operations; otherwise z / (1 + exp(-z)) per value.
__device__ __forceinline__ float2 silu2(const float2 z) {
#if MCW_FUSED_SILU_TANH
    const float2 h = __fmul2_rn(z, make_float2(0.5f, 0.5f));
    return __ffma2_rn(h, make_float2(tanh_approx(h.x), tanh_approx(h.y)), h);
#else
    return make_float2(silu(z.x), silu(z.y));
#endif
}

// Byte offset of element (row, k) in a K-major core-matrix tile whose rows are kdim long.
__host__ __device__ __forceinline__ uint32_t core_off(int row, int k, int kdim) {
    return (uint32_t)((row >> 3) * (kdim / 8) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ bool try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done) : "r"(smem_u32(bar)), "r"(parity), "r"(kSuspendNs));
    return done != 0;
}

// Bounded wait on the phase of the given parity.  With an abort flag the wait also
// gives up as soon as another role has given up, and a timeout raises the flag.
__device__ __forceinline__ bool wait_bar(uint64_t *bar, uint32_t parity, volatile int *abort) {
    const unsigned long long t0 = now_ns();
    while (!try_wait(bar, parity)) {
        if (abort && *abort) return false;
        if (now_ns() - t0 > kWaitNs) {
            if (abort) *abort = 1;
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ void arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" :: "r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void bar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" :: "r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void load_chunk(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" :: "r"(smem_u32(bar)), "r"(bytes));
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n"
                 :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n"
                 :: "r"(smem_u32(bar)));
}

// `steps` MMAs of K = 16: A k-steps a_step0 .. from a tile with rows of a_kdim,
// B k-steps 0 .. from a tile with rows of b_kdim.
__device__ __forceinline__ void mma_steps(uint32_t tmem, uint32_t a_base, int a_kdim, int a_step0, uint32_t b_base,
                                          int b_kdim, int steps, uint32_t id, bool accumulate_first) {
#pragma unroll 1
    for (int t = 0; t < steps; ++t) {
        const uint64_t da = smem_desc(a_base + (uint32_t)(a_step0 + t) * 256, 128, (uint32_t)(a_kdim / 8) * 128);
        const uint64_t db = smem_desc(b_base + (uint32_t)t * 256, 128, (uint32_t)(b_kdim / 8) * 128);
        const uint32_t acc = (accumulate_first || t > 0) ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
            :: "r"(tmem), "l"(da), "l"(db), "r"(id), "r"(acc));
    }
}

// 32 consecutive accumulator columns of this warp's 32 lanes: issue, then wait.  The
// wait names the destination registers so no use of them is scheduled before it.
__device__ __forceinline__ void tmem_ld32_issue(uint32_t taddr, uint32_t (&r)[32]) {
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
}

__device__ __forceinline__ void tmem_ld_wait(uint32_t (&r)[32]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;\n"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]),
                   "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]),
                   "+r"(r[14]), "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]),
                   "+r"(r[21]), "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]),
                   "+r"(r[28]), "+r"(r[29]), "+r"(r[30]), "+r"(r[31]));
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    tmem_ld32_issue(taddr, r);
    tmem_ld_wait(r);
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

// SiLU(z + b) of 32 accumulator columns -> bf16 at (row, c0 ..) of the activation tile.
__device__ __forceinline__ void silu_store32(const uint32_t (&r)[32], const float *bias, unsigned char *act, int row,
                                             int c0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float4 ba = *reinterpret_cast<const float4 *>(bias + c0 + q * 8);       // shared memory
        const float4 bb = *reinterpret_cast<const float4 *>(bias + c0 + q * 8 + 4);
        const float bv[8] = {ba.x, ba.y, ba.z, ba.w, bb.x, bb.y, bb.z, bb.w};
        uint32_t packed[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float2 a = silu2(__fadd2_rn(
                make_float2(__uint_as_float(r[q * 8 + 2 * e]), __uint_as_float(r[q * 8 + 2 * e + 1])),
                make_float2(bv[2 * e], bv[2 * e + 1])));
            const __nv_bfloat162 two = __floats2bfloat162_rn(a.x, a.y);
            packed[e] = *reinterpret_cast<const uint32_t *>(&two);
        }
        *reinterpret_cast<uint4 *>(act + core_off(row, c0 + q * 8, FH)) =
            make_uint4(packed[0], packed[1], packed[2], packed[3]);
    }
}

// Hidden epilogue: this warp's 32 rows x kHidCols columns of the 256-column
// accumulator -> SiLU(z + b) as bf16 into the activation tile.  The load of the next
// 32 columns is in flight while the current ones are computed.
__device__ __forceinline__ void epilogue_hidden(uint32_t tlane, const float *bias, unsigned char *act, int quarter,
                                                int group, int lane) {
    const int row = quarter * 32 + lane;
    const int cbase = group * kHidCols;
    uint32_t ra[32], rb[32];
    tmem_ld32_issue(tlane + (uint32_t)cbase, ra);
    tmem_ld_wait(ra);
#pragma unroll
    for (int h = 0; h < kHidCols / 32; h += 2) {
        if (h + 1 < kHidCols / 32) tmem_ld32_issue(tlane + (uint32_t)(cbase + (h + 1) * 32), rb);
        silu_store32(ra, bias, act, row, cbase + h * 32);
        if (h + 1 < kHidCols / 32) {
            tmem_ld_wait(rb);
            if (h + 2 < kHidCols / 32) tmem_ld32_issue(tlane + (uint32_t)(cbase + (h + 2) * 32), ra);
            silu_store32(rb, bias, act, row, cbase + (h + 1) * 32);
            if (h + 2 < kHidCols / 32) tmem_ld_wait(ra);
        }
    }
}

// Output epilogue of block blk (output columns 128 blk ..): this warp's 32 rows x
// kOutCols columns, z + b4.  Per 32 columns the warp's rows go through its stage 8 at
// a time (lanes 8p .. 8p + 7 write their rows, then every lane reads 16 bytes), and
// each 16-byte store instruction writes 4 rows x 128 contiguous bytes of y.  The
// ragged last 32 columns (640 .. 648 valid) are written one float per lane.
__device__ __forceinline__ void epilogue_out(uint32_t tlane, int blk, const float *b4, unsigned char *stage, float *y,
                                             int ldy, int m, int row0, int group, int lane) {
#pragma unroll 1
    for (int h = 0; h < kOutCols / 32; ++h) {
        const int c0 = group * kOutCols + h * 32;
        const int nb = blk * kOutN + c0;
        if (nb >= FO) break;
        const bool full = nb + 32 <= FO;
        float z[32];
#pragma unroll
        for (int q = 0; q < 8; ++q) {      // b4 in shared memory, zero past column 648
            const float4 b = *reinterpret_cast<const float4 *>(b4 + nb + 4 * q);
            z[4 * q] = b.x, z[4 * q + 1] = b.y, z[4 * q + 2] = b.z, z[4 * q + 3] = b.w;
        }
        {
            float v[32];
            tmem_ld32(tlane + (uint32_t)c0, v);
#pragma unroll
            for (int c = 0; c < 32; ++c) z[c] += v[c];
        }
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            __syncwarp();
            if ((lane >> 3) == p) {
                float4 *dst = reinterpret_cast<float4 *>(stage + (lane & 7) * kStagePitch);
#pragma unroll
                for (int q = 0; q < 8; ++q) dst[q] = make_float4(z[4 * q], z[4 * q + 1], z[4 * q + 2], z[4 * q + 3]);
            }
            __syncwarp();
            const int rbase = row0 + 8 * p;      // first of the 8 rows in the stage
            if (full) {
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    const int r = (lane >> 3) + 4 * k;
                    const float4 val = *reinterpret_cast<const float4 *>(stage + r * kStagePitch + (lane & 7) * 16);
                    if (rbase + r < m)
                        *reinterpret_cast<float4 *>(y + (size_t)(rbase + r) * ldy + nb + (lane & 7) * 4) = val;
                }
            } else if (nb + lane < FO) {
#pragma unroll
                for (int r = 0; r < 8; ++r)
                    if (rbase + r < m)
                        y[(size_t)(rbase + r) * ldy + nb + lane] =
                            *reinterpret_cast<const float *>(stage + r * kStagePitch + lane * 4);
            }
        }
        __syncwarp();
    }
}

// The same in fp16: this warp's kOutCols (64 or 32) columns are packed into half2
// first, so a stage row holds 128 (64) bytes and each output row leaves as runs of
// that length.  Row pitch ldy (halves) is a multiple of 8.
__device__ __forceinline__ void epilogue_out_half(uint32_t tlane, int blk, const float *b4, unsigned char *stage,
                                                  __half *y, int ldy, int m, int row0, int group, int lane) {
    static_assert(kOutCols == 64 || kOutCols == 32, "fp16 output: 32 or 64 columns per warp");
    constexpr int kHalves = kOutCols / 32;                // 32-column halves of the warp's share
    constexpr int kLanesPerRow = kOutCols * 2 / 16;       // 16-byte pieces of a row: 8 or 4
    constexpr int kRowsPerStore = 32 / kLanesPerRow;      // rows one store instruction covers: 4 or 8
    const int c0 = group * kOutCols;
    const int nb = blk * kOutN + c0;
    if (nb >= FO) return;
    uint32_t hp[16 * kHalves];
#pragma unroll
    for (int h = 0; h < kHalves; ++h) {
        float v[32];
        tmem_ld32(tlane + (uint32_t)(c0 + 32 * h), v);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const float4 b = *reinterpret_cast<const float4 *>(b4 + nb + 32 * h + 4 * q);
            const float2 zl = __fadd2_rn(make_float2(v[4 * q], v[4 * q + 1]), make_float2(b.x, b.y));
            const float2 zh = __fadd2_rn(make_float2(v[4 * q + 2], v[4 * q + 3]), make_float2(b.z, b.w));
            const __half2 lo = __floats2half2_rn(zl.x, zl.y);
            const __half2 hi = __floats2half2_rn(zh.x, zh.y);
            hp[16 * h + 2 * q] = *reinterpret_cast<const uint32_t *>(&lo);
            hp[16 * h + 2 * q + 1] = *reinterpret_cast<const uint32_t *>(&hi);
        }
    }
    const bool full = nb + kOutCols <= FO;
#pragma unroll
    for (int p = 0; p < 4; ++p) {
        __syncwarp();
        if ((lane >> 3) == p) {
            uint4 *dst = reinterpret_cast<uint4 *>(stage + (lane & 7) * kStagePitch);
#pragma unroll
            for (int q = 0; q < 4 * kHalves; ++q)
                dst[q] = make_uint4(hp[4 * q], hp[4 * q + 1], hp[4 * q + 2], hp[4 * q + 3]);
        }
        __syncwarp();
        const int rbase = row0 + 8 * p;
        if (full) {
#pragma unroll
            for (int k = 0; k < 8 / kRowsPerStore; ++k) {
                const int r = lane / kLanesPerRow + kRowsPerStore * k;
                const int piece = lane % kLanesPerRow;
                const uint4 val = *reinterpret_cast<const uint4 *>(stage + r * kStagePitch + piece * 16);
                if (rbase + r < m)
                    *reinterpret_cast<uint4 *>(y + (size_t)(rbase + r) * ldy + nb + piece * 8) = val;
            }
        } else if (nb + lane < FO) {       // the ragged block: columns 640 .. 648
#pragma unroll
            for (int r = 0; r < 8; ++r)
                if (rbase + r < m)
                    y[(size_t)(rbase + r) * ldy + nb + lane] =
                        *reinterpret_cast<const __half *>(stage + r * kStagePitch + lane * 2);
        }
    }
    __syncwarp();
}

__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, uint32_t src, int x, int y) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];\n"
                 :: "l"(reinterpret_cast<uint64_t>(map)), "r"(src), "r"(x), "r"(y) : "memory");
}
// A tensor store of the ensemble's output map {columns, rows, member}: box {64, 8, 1}.
__device__ __forceinline__ void tma_store_3d(const CUtensorMap *map, uint32_t src, int x, int y, int z) {
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%2, %3, %4}], [%1];\n"
                 :: "l"(reinterpret_cast<uint64_t>(map)), "r"(src), "r"(x), "r"(y), "r"(z) : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }
// the thread's tensor stores have read their shared-memory sources
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory"); }
// the thread's tensor stores are complete
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }

// fp16 output through tensor stores: this warp's 64 columns, 8 rows at a time through its
// 1 KB stage (16-byte chunk c of row r at r * 128 + (c ^ r) * 16, the map's 128-byte
// swizzle, so the stage writes are free of bank conflicts), one tensor store per 8 rows
// issued by lane 0; the warp goes on while the store drains.  The ragged block
// (columns 640 .. 648) is written with plain stores from the same stage.
template <bool kEnsemble>
__device__ __forceinline__ void epilogue_out_half_tma(uint32_t tlane, int blk, const float *b4, unsigned char *stage,
                                                      const CUtensorMap *ymap, __half *y, int ldy, int m, int row0,
                                                      int member, int group, int lane) {
    static_assert(kOutCols == 64, "tensor stores: 64 columns (128 bytes) per warp");
    const int c0 = group * kOutCols;
    const int nb = blk * kOutN + c0;
    if (nb >= FO) return;
    uint32_t hp[32];
    // both 32-column loads in flight before the one wait
    uint32_t ra[2][32];
    tmem_ld32_issue(tlane + (uint32_t)c0, ra[0]);
    tmem_ld32_issue(tlane + (uint32_t)(c0 + 32), ra[1]);
    tmem_ld_wait(ra[0]);
    tmem_ld_wait(ra[1]);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const uint32_t (&v)[32] = ra[h];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const float4 b = *reinterpret_cast<const float4 *>(b4 + nb + 32 * h + 4 * q);
            const float2 zl = __fadd2_rn(make_float2(__uint_as_float(v[4 * q]), __uint_as_float(v[4 * q + 1])),
                                         make_float2(b.x, b.y));
            const float2 zh = __fadd2_rn(make_float2(__uint_as_float(v[4 * q + 2]), __uint_as_float(v[4 * q + 3])),
                                         make_float2(b.z, b.w));
            const __half2 lo = __floats2half2_rn(zl.x, zl.y);
            const __half2 hi = __floats2half2_rn(zh.x, zh.y);
            hp[16 * h + 2 * q] = *reinterpret_cast<const uint32_t *>(&lo);
            hp[16 * h + 2 * q + 1] = *reinterpret_cast<const uint32_t *>(&hi);
        }
    }
    const bool full = nb + kOutCols <= kTmaCols;
    const int r = lane & 7;
#pragma unroll
    for (int p = 0; p < 4; ++p) {
        if (lane == 0) bulk_wait_read();          // the stage's last tensor store has read it
        __syncwarp();
        if ((lane >> 3) == p) {
#pragma unroll
            for (int q = 0; q < 8; ++q)
                *reinterpret_cast<uint4 *>(stage + r * 128 + ((q ^ r) << 4)) =
                    make_uint4(hp[4 * q], hp[4 * q + 1], hp[4 * q + 2], hp[4 * q + 3]);
        }
        const int rbase = row0 + 8 * p;
        if (full) {
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) {
                if (kEnsemble)
                    tma_store_3d(ymap, smem_u32(stage), nb, rbase, member);
                else
                    tma_store_2d(ymap, smem_u32(stage), nb, rbase);
                bulk_commit();
            }
        } else {
            __syncwarp();
            if (nb + lane < FO) {
#pragma unroll
                for (int rr = 0; rr < 8; ++rr)
                    if (rbase + rr < m)
                        y[(size_t)(rbase + rr) * ldy + nb + lane] = *reinterpret_cast<const __half *>(
                            stage + rr * 128 + (((lane >> 3) ^ rr) << 4) + (lane & 7) * 2);
            }
        }
    }
    __syncwarp();
}

struct Bars {
    uint64_t full[kSlots], empty[kSlots];   // weight ring
    uint64_t accf[kTiles][2], acce[kTiles][2];  // accumulator halves per tile: full (MMA -> epilogue), empty
    uint64_t act[kTiles];         // input / activation tile written (epilogue -> MMA)
    uint64_t fin;                 // every MMA of the CTA complete
};

// kEnsemble: the instance that carries several networks (tiles per member, member
// strides); the one-network instance has none of that arithmetic.
template <bool kHalf, bool kEnsemble>
__device__ __forceinline__ void mlp_fused_body(const float *x, int m, const float *b1, const float *b2,
                                               const float *b3, const float *b4, const unsigned char *blob, void *y,
                                               int ldy, unsigned int *err, const CUtensorMap *ymap, int use_tma,
                                               int tiles, int bias_stride, long long blob_stride) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *act0 = smem;                                  // 64 KB activation tile per tile
    unsigned char *ring = smem + kTiles * kActBytes;             // 2 x 16 KB weight chunks
    unsigned char *stage_all = ring + kRingBytes;                // 16 KB output stage ...
    unsigned char *xt0 = stage_all;                              // ... and, for layer 1, the input tiles
    float *sbias = reinterpret_cast<float *>(stage_all + kStageBytes);   // b1 | b2 | b3 | b4 (padded)
    __shared__ __align__(8) Bars bars;
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;
    volatile int *abort = &abort_flag;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // networks of an ensemble: CTA blockIdx.x carries tile (blockIdx.x % tiles) of member
    // (blockIdx.x / tiles), whose biases lie bias_stride floats and whose packed weights
    // blob_stride bytes after the previous member's, its output rows m * ldy after them
    // (member is recomputed where it is used, so it holds no register through the kernel)
    const int m0 = (kEnsemble ? (int)blockIdx.x % tiles : (int)blockIdx.x) * FM * kTiles;

    if (warp == kMmaWarp) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
                     :: "r"(smem_u32(&tmem_slot)), "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (threadIdx.x == 0) {
        abort_flag = 0;
        for (int i = 0; i < kSlots; ++i) {
            bar_init(&bars.full[i], 1);
            bar_init(&bars.empty[i], 1);
        }
        for (int t = 0; t < kTiles; ++t) {
            for (int i = 0; i < 2; ++i) {
                bar_init(&bars.accf[t][i], 1);
                bar_init(&bars.acce[t][i], kEpiThreads);
            }
            bar_init(&bars.act[t], kEpiThreads);
        }
        bar_init(&bars.fin, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem = tmem_slot;

    if (warp == kProducerWarp) {
        if (lane == 0) {
            int issued = 0;
            for (int i = 0; i < kSeqChunks; ++i) {
                const int slot = i % kSlots;
                if (i >= kSlots && !wait_bar(&bars.empty[slot], (uint32_t)(i / kSlots - 1) & 1u, abort)) break;
                const int c = chunk_at(i);
                load_chunk(ring + slot * kChunkBytes,
                           blob + (kEnsemble ? (size_t)((int)blockIdx.x / tiles) * (size_t)blob_stride : 0) +
                               chunk_offset(c),
                           chunk_bytes(c), &bars.full[slot]);
                issued = i + 1;
            }
            // the last copy into each slot has landed before the CTA can leave
            for (int i = issued - kSlots < 0 ? 0 : issued - kSlots; i < issued; ++i)
                wait_bar(&bars.full[i % kSlots], (uint32_t)(i / kSlots) & 1u, nullptr);
        }
    } else if (warp == kMmaWarp) {
        if (lane == 0) {
            const uint32_t ring_a = smem_u32(ring);
            int chunk = 0;
            uint32_t act_phase[kTiles];
            for (int t = 0; t < kTiles; ++t) act_phase[t] = 0u;
            bool ok = true;
            auto take = [&](void) -> uint32_t {      // wait for the next chunk; its shared address
                const int slot = chunk % kSlots;
                ok = ok && wait_bar(&bars.full[slot], (uint32_t)(chunk / kSlots) & 1u, abort);
                asm volatile("tcgen05.fence::after_thread_sync;\n");
                return ring_a + (uint32_t)slot * kChunkBytes;
            };
            auto release = [&](void) {               // chunk's MMAs issued: free its slot when they finish
                commit(&bars.empty[chunk % kSlots]);
                ++chunk;
            };
            auto wait_act = [&](int t) {             // tile t's input / activations written
                ok = ok && wait_bar(&bars.act[t], act_phase[t], abort);
                act_phase[t] ^= 1u;
                asm volatile("tcgen05.fence::after_thread_sync;\n");
            };
            // layer 1 of each tile: input tile x W1
            for (int t = 0; t < kTiles && ok; ++t) {
                wait_act(t);
                if (!ok) break;
                const uint32_t w = take();
                if (!ok) break;
                mma_steps(tmem + (uint32_t)(t * 256), smem_u32(xt0 + t * kXBytes), FK1, 0, w, FK1, 1, idesc(FH), false);
                release();
                commit(&bars.accf[t][0]);
            }
            // layers 2 and 3: eight chunks of 32 k each, tile by tile (one tile's MMAs run
            // while the other's epilogue writes its activations)
            for (int layer = 0; layer < 2 && ok; ++layer) {
                for (int t = 0; t < kTiles && ok; ++t) {
                    wait_act(t);
                    const uint32_t act_a = smem_u32(act0 + t * kActBytes);
                    for (int c = 0; c < kHidChunks && ok; ++c) {
                        const uint32_t w = take();
                        if (!ok) break;
                        mma_steps(tmem + (uint32_t)(t * 256), act_a, FH, c * (kHidK / 16), w, kHidK, kHidK / 16,
                                  idesc(FH), c > 0);
                        release();
                    }
                    if (ok) commit(&bars.accf[t][0]);
                }
            }
            // output layer: six 128-column blocks per tile alternating between the halves
            // of the tile's accumulator
            for (int t = 0; t < kTiles && ok; ++t) {
                wait_act(t);
                const uint32_t act_a = smem_u32(act0 + t * kActBytes);
                for (int j = 0; j < kOutBlocks && ok; ++j) {
                    const int h = j & 1;
                    if (j >= 2) {
                        ok = wait_bar(&bars.acce[t][h], (uint32_t)((j >> 1) - 1) & 1u, abort);
                        asm volatile("tcgen05.fence::after_thread_sync;\n");
                        if (!ok) break;
                    }
                    for (int c = 0; c < kOutChunks && ok; ++c) {
                        const uint32_t w = take();
                        if (!ok) break;
                        mma_steps(tmem + (uint32_t)(t * 256 + h * kOutN), act_a, FH, c * (kOutK / 16), w, kOutK,
                                  kOutK / 16, idesc(kOutN), c > 0);
                        release();
                    }
                    if (ok) commit(&bars.accf[t][h]);
                }
            }
            // every MMA issued by this thread has completed before the memory is freed
            commit(&bars.fin);
            wait_bar(&bars.fin, 0, nullptr);
        }
    } else {
        // epilogue warps
        const int quarter = warp & 3, group = warp >> 2;   // lane quarter, column group
        unsigned char *stage = stage_all + warp * kStageWarp;
        uint32_t accf_phase[kTiles][2];
        for (int t = 0; t < kTiles; ++t) accf_phase[t][0] = accf_phase[t][1] = 0u;
        // biases into shared memory (b4 zero past column 648), then the epilogue warps meet
        {
            const size_t bo = kEnsemble ? (size_t)((int)blockIdx.x / tiles) * (size_t)bias_stride : 0;
            for (int i = threadIdx.x; i < kBiasFloats; i += kEpiThreads) {
                float v;
                if (i < 256) v = b1[bo + i];
                else if (i < 512) v = b2[bo + i - 256];
                else if (i < 768) v = b3[bo + i - 512];
                else v = i - 768 < FO ? b4[bo + i - 768] : 0.f;
                sbias[i] = v;
            }
        }
        asm volatile("bar.sync 1, %0;\n" :: "n"(kEpiThreads) : "memory");
        for (int t = 0; t < kTiles; ++t) {
            if (threadIdx.x < FM) {
                const int r = threadIdx.x, gm = m0 + t * FM + r;
                float xin[FIN];
#pragma unroll
                for (int k = 0; k < FIN; ++k) xin[k] = gm < m ? x[(size_t)gm * FIN + k] : 0.f;
                const __nv_bfloat162 p0 = __floats2bfloat162_rn(xin[0], xin[1]);
                const __nv_bfloat162 p1 = __floats2bfloat162_rn(xin[2], xin[3]);
                unsigned char *xt = xt0 + t * kXBytes;
                *reinterpret_cast<uint4 *>(xt + core_off(r, 0, FK1)) = make_uint4(
                    *reinterpret_cast<const uint32_t *>(&p0), *reinterpret_cast<const uint32_t *>(&p1), 0u, 0u);
                *reinterpret_cast<uint4 *>(xt + core_off(r, 8, FK1)) = make_uint4(0u, 0u, 0u, 0u);
            }
            asm volatile("fence.proxy.async.shared::cta;\n");
            arrive(&bars.act[t]);
        }
        const float *hb[3] = {sbias, sbias + 256, sbias + 512};
        bool ok = true;
        for (int layer = 0; layer < 3 && ok; ++layer) {
            for (int t = 0; t < kTiles && ok; ++t) {
                ok = wait_bar(&bars.accf[t][0], accf_phase[t][0], abort);
                accf_phase[t][0] ^= 1u;
                if (!ok) break;
                asm volatile("tcgen05.fence::after_thread_sync;\n");
                const uint32_t tlane = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(t * 256);
                epilogue_hidden(tlane, hb[layer], act0 + t * kActBytes, quarter, group, lane);
                asm volatile("fence.proxy.async.shared::cta;\n");
                asm volatile("tcgen05.fence::before_thread_sync;\n");
                arrive(&bars.act[t]);
            }
        }
        for (int t = 0; t < kTiles && ok; ++t) {
            const uint32_t tlane = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(t * 256);
            const int row0 = m0 + t * FM + quarter * 32;
            for (int j = 0; j < kOutBlocks && ok; ++j) {
                const int h = j & 1;
                ok = wait_bar(&bars.accf[t][h], accf_phase[t][h], abort);
                accf_phase[t][h] ^= 1u;
                if (!ok) break;
                asm volatile("tcgen05.fence::after_thread_sync;\n");
                // this member's output rows (plain stores; the tensor map takes the member as a coordinate)
                const int member = kEnsemble ? (int)blockIdx.x / tiles : 0;
                const size_t yoff = kEnsemble ? (size_t)member * (size_t)m * (size_t)ldy : 0;
                if (kHalf && use_tma)
                    epilogue_out_half_tma<kEnsemble>(tlane + (uint32_t)(h * kOutN), j, sbias + 768,
                                                     stage_all + warp * kStageTma,
                                          ymap, static_cast<__half *>(y) + yoff, ldy, m, row0, member, group, lane);
                else if (kHalf)
                    epilogue_out_half(tlane + (uint32_t)(h * kOutN), j, sbias + 768, stage,
                                      static_cast<__half *>(y) + yoff, ldy, m, row0, group, lane);
                else
                    epilogue_out(tlane + (uint32_t)(h * kOutN), j, sbias + 768, stage, static_cast<float *>(y) + yoff,
                                 ldy, m, row0, group, lane);
                asm volatile("tcgen05.fence::before_thread_sync;\n");
                arrive(&bars.acce[t][h]);
            }
        }
        if (kHalf && use_tma && lane == 0) bulk_wait_all();   // this warp's tensor stores are done
    }

    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    if (threadIdx.x == 0 && abort_flag) atomicOr(err, 2u);
    if (warp == kMmaWarp) {
        __syncwarp();
        asm volatile("tcgen05.fence::after_thread_sync;\n");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" :: "r"(tmem), "r"(kTmemCols));
    }
}

// One network: CTA blockIdx.x carries rows 128 blockIdx.x ...
template <bool kHalf>
__global__ void __launch_bounds__(kThreads, kCtasPerSm) mlp_fused_kernel(const float *x, int m, const float *b1,
                                                                const float *b2, const float *b3, const float *b4,
                                                                const unsigned char *blob, void *y, int ldy,
                                                                unsigned int *err,
                                                                const __grid_constant__ CUtensorMap ymap,
                                                                int use_tma) {
    mlp_fused_body<kHalf, false>(x, m, b1, b2, b3, b4, blob, y, ldy, err, &ymap, use_tma, (int)gridDim.x, 0, 0);
}

// An ensemble: fp16 outputs, tiles CTAs per member (mlp_fused_body).
__global__ void __launch_bounds__(kThreads, kCtasPerSm) mlp_fused_ensemble_kernel(
        const float *x, int m, const float *b1, const float *b2, const float *b3, const float *b4,
        const unsigned char *blob, void *y, int ldy, unsigned int *err, const __grid_constant__ CUtensorMap ymap,
        int use_tma, int tiles, int bias_stride, long long blob_stride) {
    mlp_fused_body<true, true>(x, m, b1, b2, b3, b4, blob, y, ldy, err, &ymap, use_tma, tiles, bias_stride,
                               blob_stride);
}

// Rows [row0, row0 + rows_out) and k [k0, k0 + kdim) of W [n, k_in] (row-major bf16) as a
// K-major core-matrix tile with rows of kdim; entries outside W are zero.
__global__ void pack_kernel(const __nv_bfloat16 *w, int n, int k_in, int row0, int rows_out, int k0, int kdim,
                            unsigned char *tile) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;   // one 16-byte chunk: row, k8
    const int per_row = kdim / 8;
    if (c >= rows_out * per_row) return;
    const int r = c / per_row, k8 = c % per_row;
    __align__(16) __nv_bfloat16 h[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const int gr = row0 + r, gk = k0 + k8 * 8 + e;
        h[e] = (gr < n && gk < k_in) ? w[(size_t)gr * k_in + gk] : __float2bfloat16(0.f);
    }
    *reinterpret_cast<uint4 *>(tile + core_off(r, k8 * 8, kdim)) = *reinterpret_cast<const uint4 *>(h);
}

}  // namespace

}  // namespace mcw

using namespace mcw;

namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

// fp16 output [m, kTmaCols] at row pitch ldy halves, box 64 x 8, and for an ensemble
// [members, m, kTmaCols] (members m * ldy halves apart), box 64 x 8 x 1, so that a box
// passing row m - 1 of a member is clipped there; 128-byte swizzle.  False when the
// driver entry point is missing or the layout breaks a tensor-map rule.
bool make_out_map(CUtensorMap *map, void *y, int m, int ldy, int members) {
    EncodeTiledFn fn = encode_fn();
    if (!fn || (reinterpret_cast<uintptr_t>(y) & 15) || (ldy & 7) || ldy < kTmaCols || members < 1) return false;
    const cuuint32_t rank = members > 1 ? 3 : 2;
    const cuuint64_t dims[3] = {(cuuint64_t)kTmaCols, (cuuint64_t)m, (cuuint64_t)members};
    const cuuint64_t strides[2] = {(cuuint64_t)ldy * 2, (cuuint64_t)m * (cuuint64_t)ldy * 2};
    const cuuint32_t box[3] = {64, 8, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, rank, y, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_NONE,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// members networks (1 for one network) on the same inputs: member e's biases bias_stride
// floats and its packed weights blob_stride bytes after member e - 1's, its outputs at
// y + e * m * ldy.
int forward(const float *x, int32_t m, const float *b1, const float *b2, const float *b3, const float *b4,
            const void *blob, void *y, int32_t ldy, bool half, void *stream, int members = 1, int bias_stride = 0,
            long long blob_stride = 0) {
    const int align = half ? 8 : 4;   // 16-byte row starts
    if (!x || !b1 || !b2 || !b3 || !b4 || !blob || !y || m < 0 || ldy < FO || (ldy % align) != 0)
        return MCW_MLP_ERR_ARG;
    if ((((uintptr_t)blob | (uintptr_t)y) & 15) != 0) return MCW_MLP_ERR_ARG;
    if (members < 1 || (members > 1 && (bias_stride < 0 || blob_stride <= 0 || (blob_stride & 15) != 0)))
        return MCW_MLP_ERR_ARG;
    if (m == 0) return 0;
    unsigned int *err = tc_err_flag();
    if (!err) return MCW_MLP_ERR_CUDA;
    const void *fn = half ? (members > 1 ? reinterpret_cast<const void *>(mlp_fused_ensemble_kernel)
                                         : reinterpret_cast<const void *>(mlp_fused_kernel<true>))
                          : reinterpret_cast<const void *>(mlp_fused_kernel<false>);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes);
    if (e != cudaSuccess) return MCW_MLP_ERR_CUDA;
    const int tiles = (m + FM * kTiles - 1) / (FM * kTiles);
    if ((long long)tiles * members > 0x7fffffffLL) return MCW_MLP_ERR_ARG;
    const unsigned grid = (unsigned)(tiles * members);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const unsigned char *wb = static_cast<const unsigned char *>(blob);
    CUtensorMap ymap;
    memset(&ymap, 0, sizeof(ymap));
    const int use_tma = (half && MCW_FUSED_TMA_OUT && make_out_map(&ymap, y, m, ldy, members)) ? 1 : 0;
    if (half && members > 1)
        mlp_fused_ensemble_kernel<<<grid, kThreads, kSmemBytes, s>>>(x, m, b1, b2, b3, b4, wb, y, ldy, err, ymap,
                                                                     use_tma, tiles, bias_stride, blob_stride);
    else if (half)
        mlp_fused_kernel<true><<<grid, kThreads, kSmemBytes, s>>>(x, m, b1, b2, b3, b4, wb, y, ldy, err, ymap, use_tma);
    else
        mlp_fused_kernel<false><<<grid, kThreads, kSmemBytes, s>>>(x, m, b1, b2, b3, b4, wb, y, ldy, err, ymap, 0);
    return cudaGetLastError() == cudaSuccess ? 0 : MCW_MLP_ERR_CUDA;
}

}  // namespace

extern "C" {

int mcw_mlp_pack(const void *w1, const void *w2, const void *w3, const void *w4, void *blob, void *stream) {
    if (!w1 || !w2 || !w3 || !w4 || !blob) return MCW_MLP_ERR_ARG;
    if (((uintptr_t)blob & 15) != 0) return MCW_MLP_ERR_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned char *b = static_cast<unsigned char *>(blob);
    const int threads = 256;
    auto pack = [&](const void *w, int n, int k_in, int row0, int rows_out, int k0, int kdim, int chunk) {
        const int units = rows_out * (kdim / 8);
        pack_kernel<<<(units + threads - 1) / threads, threads, 0, s>>>(
            static_cast<const __nv_bfloat16 *>(w), n, k_in, row0, rows_out, k0, kdim, b + chunk_offset(chunk));
    };
    int chunk = 0;
    pack(w1, FH, FIN, 0, FH, 0, FK1, chunk++);
    for (const void *w : {w2, w3})
        for (int c = 0; c < kHidChunks; ++c) pack(w, FH, FH, 0, FH, c * kHidK, kHidK, chunk++);
    for (int j = 0; j < kOutBlocks; ++j)
        for (int c = 0; c < kOutChunks; ++c) pack(w4, FO, FH, j * kOutN, kOutN, c * kOutK, kOutK, chunk++);
    return cudaGetLastError() == cudaSuccess ? 0 : MCW_MLP_ERR_CUDA;
}

int mcw_mlp_forward(const float *x, int32_t m, const float *b1, const float *b2, const float *b3, const float *b4,
                    const void *blob, float *y, int32_t ldy, void *stream) {
    return forward(x, m, b1, b2, b3, b4, blob, y, ldy, false, stream);
}

int mcw_mlp_forward_f16(const float *x, int32_t m, const float *b1, const float *b2, const float *b3,
                        const float *b4, const void *blob, void *y, int32_t ldy, void *stream) {
    return forward(x, m, b1, b2, b3, b4, blob, y, ldy, true, stream);
}

int mcw_mlp_forward_ensemble_f16(const float *x, int32_t m, int32_t members, const float *bias, const void *blob,
                                 void *y, int32_t ldy, void *stream) {
    if (!bias || members < 1) return MCW_MLP_ERR_ARG;
    return forward(x, m, bias, bias + 256, bias + 512, bias + 768, blob, y, ldy, true, stream, members,
                   MCW_MLP_BIAS_FLOATS, (long long)MCW_MLP_PACK_BYTES);
}

}  // extern "C"
