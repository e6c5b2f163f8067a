// Training engine of the surrogate network: every kernel of one Adam step of a
// whole ensemble (all members at once), so a step is a short, fixed sequence of
// launches that a CUDA graph replays.
//
//  * gemm_tma_kernel: C = A B^T for `groups` independent products (ensemble
//    members) in one launch, bf16 operands stored K-major, FP32 accumulation in
//    tensor memory.  Operand tiles reach shared memory by TMA
//    (cp.async.bulk.tensor.3d from a {K, rows, group} tensor map, 16-byte boxes of
//    128 rows, so each lands as a column of 8 x 16-byte core matrices) through a
//    3-stage ring with mbarrier transaction counts; one thread issues the copies,
//    one the tcgen05.mma (128 x 128 x 16, four per 64-wide K chunk), each stage
//    handed back to the copier by tcgen05.commit.  Split-K (grid.z = groups x
//    splits) writes FP32 partial products that mlp_reduce_splits adds.  Epilogues
//    (four warps, tcgen05.ld): FP32 store; bias; bias + SiLU keeping the FP32
//    pre-activation and a transposed bf16 copy of the activation; the SiLU'
//    product of the backward pass with the same copies.  The transposed copies
//    are the K-major operands of the weight-gradient products, so every operand
//    of every product of a step is K-major.
//  * loss_grouped_kernel, colsum_grouped_kernel, adam_grouped_kernel,
//    gather_kernel, advance_kernel: the rest of the step, each one launch for all
//    members; the learning rate and step count are read from device memory so a
//    captured step can be replayed unchanged.
//
// Every mbarrier wait is bounded (2 s of %globaltimer); a wait that runs out raises
// bit 2 of mcw_mlp_status, the CTA waits (bounded) for its copies and MMAs in
// flight, frees its tensor memory and leaves.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/mcw_mlp.h"

namespace mcw {

namespace {

constexpr int TM = 128, TN = 128, TK = 64;
constexpr int kStages = 3;
constexpr int kOpBytes = TM * TK * 2;             // one operand's 128 x 64 bf16 chunk: 16 KB
constexpr int kStageBytes = 2 * kOpBytes;         // A and B
constexpr int kBoxBytes = 128 * 16;               // one TMA box: 128 rows x 8 bf16
constexpr uint32_t kTmemCols = 128;
constexpr unsigned long long kWaitNs = 2000000000ull;
constexpr size_t kSmemBytes = (size_t)kStages * kStageBytes + 1024;  // + alignment slack

// Instruction descriptor of tcgen05.mma kind::f16: F32 accumulate, BF16 A and B,
// both K-major, N = 128 (bits 17-22: N >> 3), M = 128 (bits 24-28: M >> 4).
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) |
                            ((uint32_t)(TM >> 4) << 24);

// Shared-memory matrix descriptor, no swizzle: start >> 4 (bits 0-13), leading byte
// offset >> 4 (bits 16-29: K-adjacent core matrices), stride byte offset >> 4 (bits
// 32-45: M/N-adjacent core matrices), descriptor version 1 (bit 46).  A stage holds
// an operand as eight TMA boxes, box j (k = 8j .. 8j + 7) at j * 2048 with row r at
// (r / 8) * 128 + (r % 8) * 16: K-adjacent core matrices 2048 bytes apart, row-group
// adjacent ones 128 bytes apart.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((2048u >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((128u >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ float silu(float z) { return __fdividef(z, 1.f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
    const float s = 1.f / (1.f + __expf(-z));
    return s * (1.f + z * (1.f - s));
}

__device__ __forceinline__ bool try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return done != 0;
}

// Bounded wait; gives up when another role of the CTA has given up, and raises the
// CTA's abort flag when its own time runs out.
__device__ __forceinline__ bool wait_bar(uint64_t *bar, uint32_t parity, volatile int *abort) {
    const unsigned long long t0 = now_ns();
    while (!try_wait(bar, parity)) {
        if (*abort) return false;
        if (now_ns() - t0 > kWaitNs) {
            *abort = 1;
            return false;
        }
    }
    return true;
}

// Bounded wait that ignores the abort flag (draining copies and MMAs in flight).
__device__ __forceinline__ void drain_bar(uint64_t *bar, uint32_t parity) {
    const unsigned long long t0 = now_ns();
    while (!try_wait(bar, parity) && now_ns() - t0 <= kWaitNs) {
    }
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int x, int y, int z,
                                            uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];\n"
        :: "r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
        : "memory");
}

__device__ __forceinline__ void commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n"
                 :: "r"(smem_u32(bar)) : "memory");
}

struct TmaGemmArgs {
    CUtensorMap ta;          // A: {k, m, groups}, box {8, 128, 1}
    CUtensorMap tb;          // B: {k, n, groups}
    int32_t m, n, k;
    int32_t splits, kps;     // K per split (multiple of TK)
    int32_t pad;
    const float *bias;
    long long s_bias;
    const float *aux;
    long long ld_aux, s_aux;
    void *c;
    long long ldc, s_c, s_split;
    void *c2;
    long long ldc2, s_c2;
    void *ct;
    long long ldct, s_ct;
    unsigned int *err;
};

template <int kEpi>
__global__ void __launch_bounds__(128) gemm_tma_kernel(const __grid_constant__ TmaGemmArgs p) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full_bar[kStages], empty_bar[kStages], acc_bar;
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * TM, n0 = blockIdx.y * TN;
    const int g = blockIdx.z / p.splits, sp = blockIdx.z % p.splits;
    const int kbeg = sp * p.kps;
    const int kend = min(p.k, kbeg + p.kps);
    const int nch = kend > kbeg ? (kend - kbeg + TK - 1) / TK : 0;
    volatile int *abort = &abort_flag;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
                     :: "r"(smem_u32(&tmem_slot)), "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (threadIdx.x == 32) {
        for (int s = 0; s < kStages; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(&full_bar[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(&empty_bar[s])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(&acc_bar)));
        asm volatile("fence.mbarrier_init.release.cluster;\n");
        abort_flag = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem = tmem_slot;

    int issued = 0;      // chunks whose copies were issued (producer)
    int consumed = 0;    // chunks whose MMAs were issued (MMA thread)
    if (warp == 0 && lane == 0) {
        // producer: TMA copies of each chunk into its stage, once the stage is free
        for (int kc = 0; kc < nch; ++kc) {
            const int s = kc % kStages, use = kc / kStages;
            if (use > 0 && !wait_bar(&empty_bar[s], (uint32_t)((use - 1) & 1), abort)) break;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n"
                         :: "r"(smem_u32(&full_bar[s])), "r"((uint32_t)kStageBytes) : "memory");
            const uint32_t sa = smem_u32(smem + (size_t)s * kStageBytes), sb = sa + kOpBytes;
            const int k0 = kbeg + kc * TK;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                tma_load_3d(sa + j * kBoxBytes, &p.ta, k0 + 8 * j, m0, g, &full_bar[s]);
                tma_load_3d(sb + j * kBoxBytes, &p.tb, k0 + 8 * j, n0, g, &full_bar[s]);
            }
            issued = kc + 1;
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer: four K = 16 steps per chunk; the stage goes back to the producer
        // when they complete
        for (int kc = 0; kc < nch; ++kc) {
            const int s = kc % kStages, use = kc / kStages;
            if (!wait_bar(&full_bar[s], (uint32_t)(use & 1), abort)) break;
            asm volatile("tcgen05.fence::after_thread_sync;\n");
            const uint32_t a0 = smem_u32(smem + (size_t)s * kStageBytes), b0 = a0 + kOpBytes;
#pragma unroll
            for (int t = 0; t < TK / 16; ++t) {
                const uint64_t da = smem_desc(a0 + t * 2 * kBoxBytes);
                const uint64_t db = smem_desc(b0 + t * 2 * kBoxBytes);
                const uint32_t accumulate = (kc > 0 || t > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
                    :: "r"(tmem), "l"(da), "l"(db), "r"(kIdesc), "r"(accumulate));
            }
            commit(&empty_bar[s]);
            consumed = kc + 1;
        }
        // the accumulator is complete when every MMA issued above is (no MMA: arrives now)
        if (consumed > 0) commit(&acc_bar);
        else asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" :: "r"(smem_u32(&acc_bar)) : "memory");
    }
    __syncwarp();
    const bool ok = wait_bar(&acc_bar, 0u, abort) && !*abort;
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;\n");

    if (ok) {
        // epilogue: lane l of warp w holds row m0 + 32w + l of each 32-column block;
        // the pipeline's shared memory (free now) gives every warp a 32 x 33 staging
        // tile, so row-major loads and stores go one row (128 bytes) per instruction
        float *tile = reinterpret_cast<float *>(smem + (size_t)warp * (32 * 33 * 4));
        const int rbase = m0 + warp * 32;
        const int m = rbase + lane;
        const bool row_ok = m < p.m;
        const bool have_acc = nch > 0;
#pragma unroll 1
        for (int c0 = 0; c0 < TN; c0 += 32) {
            uint32_t v[32];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                  "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                  "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]),
                  "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]),
                  "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            const int nb = n0 + c0;
            if (nb >= p.n) break;                                   // warp-uniform
            const int cnt = min(32, p.n - nb);
            float z[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) z[j] = have_acc ? __uint_as_float(v[j]) : 0.f;
            if (kEpi == MCW_EPI_BIAS_F32 || kEpi == MCW_EPI_BIAS_SILU) {
                const float *b = p.bias + (size_t)g * p.s_bias + nb;
#pragma unroll
                for (int j = 0; j < 32; ++j)
                    if (j < cnt) z[j] += __ldg(b + j);
            }
            if (kEpi == MCW_EPI_DSILU) {
                // the pre-activations, row by row into the tile, then column j of lane's row
                const float *ax = p.aux + (size_t)g * p.s_aux + nb + lane;
                float av[32];   // all 32 loads in flight before the first store
#pragma unroll
                for (int r = 0; r < 32; ++r) {
                    const int row = rbase + r;
                    av[r] = (row < p.m && lane < cnt) ? __ldg(ax + (size_t)row * p.ld_aux) : 0.f;
                }
#pragma unroll
                for (int r = 0; r < 32; ++r) tile[r * 33 + lane] = av[r];
                __syncwarp();
#pragma unroll
                for (int j = 0; j < 32; ++j) z[j] *= dsilu(tile[lane * 33 + j]);
                __syncwarp();
            }
            // f32 output: the product (F32, BIAS_F32, split partials) or the kept
            // pre-activation / gradient (c2 of BIAS_SILU and DSILU)
            float *c32 = nullptr;
            long long ld32 = 0;
            if (kEpi == MCW_EPI_F32) {
                c32 = static_cast<float *>(p.c) + (size_t)sp * p.s_split + (size_t)g * p.s_c;
                ld32 = p.ldc;
            } else if (kEpi == MCW_EPI_BIAS_F32) {
                c32 = static_cast<float *>(p.c) + (size_t)g * p.s_c;
                ld32 = p.ldc;
            } else if (p.c2) {
                c32 = static_cast<float *>(p.c2) + (size_t)g * p.s_c2;
                ld32 = p.ldc2;
            }
            if (c32) {
#pragma unroll
                for (int j = 0; j < 32; ++j) tile[lane * 33 + j] = z[j];
                __syncwarp();
                float *dst = c32 + nb + lane;
#pragma unroll 4
                for (int r = 0; r < 32; ++r) {
                    const int row = rbase + r;
                    if (row < p.m && lane < cnt) dst[(size_t)row * ld32] = tile[r * 33 + lane];
                }
                __syncwarp();
            }
            if (kEpi == MCW_EPI_BIAS_SILU || kEpi == MCW_EPI_DSILU) {
                float h[32];
#pragma unroll
                for (int j = 0; j < 32; ++j) h[j] = kEpi == MCW_EPI_BIAS_SILU ? silu(z[j]) : z[j];
                if (p.ct && row_ok) {
                    // transposed copy [n, m]: for each column the warp's lanes write 32
                    // consecutive rows
                    __nv_bfloat16 *t16 = static_cast<__nv_bfloat16 *>(p.ct) + (size_t)g * p.s_ct + m;
#pragma unroll
                    for (int j = 0; j < 32; ++j)
                        if (j < cnt) t16[(size_t)(nb + j) * p.ldct] = __float2bfloat16(h[j]);
                }
#pragma unroll
                for (int j = 0; j < 32; ++j) tile[lane * 33 + j] = h[j];
                __syncwarp();
                __nv_bfloat16 *dst = static_cast<__nv_bfloat16 *>(p.c) + (size_t)g * p.s_c + nb + lane;
#pragma unroll 4
                for (int r = 0; r < 32; ++r) {
                    const int row = rbase + r;
                    if (row < p.m && lane < cnt) dst[(size_t)row * p.ldc] = __float2bfloat16(tile[r * 33 + lane]);
                }
                __syncwarp();
            }
        }
    } else if (threadIdx.x == 0) {
        atomicOr(p.err, 4u);
    }
    if (!ok) {
        // copies and MMAs still in flight complete (bounded) before the memory is freed:
        // the producer waits for its last stages' copies, the MMA thread for the
        // accumulator barrier its final commit tracks every issued MMA with
        if (warp == 0 && lane == 0)
            for (int kc = max(0, issued - kStages); kc < issued; ++kc)
                drain_bar(&full_bar[kc % kStages], (uint32_t)((kc / kStages) & 1));
        if (warp == 1 && lane == 0 && consumed > 0) drain_bar(&acc_bar, 0u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" :: "r"(tmem), "r"(kTmemCols));
    }
}

// ---------------------------------------------------------------- the other kernels

// Sum of `splits` partial products: dst[g][i][j] = sum_s src[s][g][i][j] (fixed order).
__global__ void reduce_splits_kernel(const float *src, long long s_split, long long s_src_g, long long ld_src,
                                     float *dst, long long s_dst_g, long long ld_dst, int splits, int m, int n) {
    const int g = blockIdx.z;
    const long long total = (long long)m * n;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long i = e / n, j = e % n;
        const float *s = src + (size_t)g * s_src_g + (size_t)i * ld_src + j;
        float acc = 0.f;
        for (int q = 0; q < splits; ++q) acc += s[(size_t)q * s_split];
        dst[(size_t)g * s_dst_g + (size_t)i * ld_dst + j] = acc;
    }
}

// Weighted squared error of `groups` outputs: each block takes a strip of 32 columns x
// kLossRows rows in 32 x 32 tiles; loss[g] += sum w_j d^2 / (m n) (one atomic per block);
// the gradient 2 w_j d / (m n) as f32 and bf16 [m, n] and bf16 transposed [n, m]
// (through a shared-memory tile, so both stores are coalesced).
constexpr int kLossRows = 256;

__global__ void loss_grouped_kernel(const float *y, long long ldy, long long s_y, const float *t, long long ldt,
                                    long long s_t, const float *w, int m, int n, float *g32, long long ldg,
                                    long long s_g32, __nv_bfloat16 *g16, long long s_g16, __nv_bfloat16 *g16t,
                                    long long ldgt, long long s_g16t, float *loss) {
    __shared__ __nv_bfloat16 tile[32][33];
    __shared__ float wsum[8];
    const int g = blockIdx.z;
    const int c0 = blockIdx.x * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8 threads
    const float scale = 1.f / ((float)m * (float)n);
    const int c = c0 + tx;
    const float wc = (c < n) ? (w ? w[c] : 1.f) : 0.f;
    float l = 0.f;
    for (int r0 = blockIdx.y * kLossRows; r0 < min(m, (blockIdx.y + 1) * kLossRows); r0 += 32) {
        for (int rr = ty; rr < 32; rr += 8) {
            const int r = r0 + rr;
            __nv_bfloat16 h = __float2bfloat16(0.f);
            if (r < m && c < n) {
                const float d = y[(size_t)g * s_y + (size_t)r * ldy + c] - t[(size_t)g * s_t + (size_t)r * ldt + c];
                l += wc * d * d * scale;
                const float gv = 2.f * wc * d * scale;
                g32[(size_t)g * s_g32 + (size_t)r * ldg + c] = gv;
                h = __float2bfloat16(gv);
                g16[(size_t)g * s_g16 + (size_t)r * ldg + c] = h;
            }
            tile[rr][tx] = h;
        }
        __syncthreads();
        for (int cc = ty; cc < 32; cc += 8) {
            const int cw = c0 + cc, r = r0 + tx;
            if (cw < n && r < m) g16t[(size_t)g * s_g16t + (size_t)cw * ldgt + r] = tile[tx][cc];
        }
        __syncthreads();
    }
    for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if (tx == 0) wsum[ty] = l;
    __syncthreads();
    if (threadIdx.x == 0) {
        float b = 0.f;
#pragma unroll
        for (int q = 0; q < 8; ++q) b += wsum[q];
        if (b != 0.f) atomicAdd(loss + g, b);
    }
}

// Bias gradients: out[g * s_out + off_l + j] = sum_i G_l[g][i][j] for the layers of
// the table (fixed summation order: 8 row lanes per column, then the 8 partials).
struct ColsumLayer {
    const float *src;
    long long ld, s_g;
    long long off;     // column 0's offset in out
    int n;
    int pad;
};
struct ColsumTable {
    ColsumLayer l[4];
    int n_layers;
};

// One pass over rows [row0, row1) of every (layer, group): 8 row lanes per column,
// their partial sums combined in a fixed order.  blockIdx.y is the row chunk; the
// result goes to out (one chunk) or to partial[((z * chunks + chunk) * ldp) + col].
__global__ void colsum_grouped_kernel(const ColsumTable tab, int groups, int m, int rows_per_chunk, float *out,
                                      long long s_out, float *partial, int ldp) {
    const int layer = blockIdx.z / groups, g = blockIdx.z % groups;
    const ColsumLayer L = tab.l[layer];
    const int col = blockIdx.x * 32 + (threadIdx.x & 31);
    const int row_lane = threadIdx.x >> 5;
    const int r0 = blockIdx.y * rows_per_chunk, r1 = min(m, r0 + rows_per_chunk);
    __shared__ float part[8][32];
    float acc = 0.f;
    if (col < L.n) {
        const float *s = L.src + (size_t)g * L.s_g + col;
        for (int r = r0 + row_lane; r < r1; r += 8) acc += s[(size_t)r * L.ld];
    }
    part[row_lane][threadIdx.x & 31] = acc;
    __syncthreads();
    if (row_lane == 0 && col < L.n) {
        float t = 0.f;
#pragma unroll
        for (int q = 0; q < 8; ++q) t += part[q][threadIdx.x];
        if (partial) partial[((size_t)blockIdx.z * gridDim.y + blockIdx.y) * ldp + col] = t;
        else out[(size_t)g * s_out + L.off + col] = t;
    }
}

// Second pass: the chunks' partial sums added in order.
__global__ void colsum_finish_kernel(const ColsumTable tab, int groups, int chunks, const float *partial, int ldp,
                                     float *out, long long s_out) {
    const int layer = blockIdx.z / groups, g = blockIdx.z % groups;
    const ColsumLayer L = tab.l[layer];
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= L.n) return;
    const float *p = partial + (size_t)blockIdx.z * chunks * ldp + col;
    float t = 0.f;
    for (int c = 0; c < chunks; ++c) t += p[(size_t)c * ldp];
    out[(size_t)g * s_out + L.off + col] = t;
}

// Transposed bf16 copies of weight blocks written by Adam (the B operands of the
// backward products): wt[g * s_t + off_t + c * ld_t + o] = w[o, c] for the block's
// rows o < rows and columns c < cols, which start at offset off in the flat layout.
struct TransposeBlock {
    long long off, off_t, ld_t;
    int rows, cols;
};
struct TransposeTable {
    TransposeBlock b[4];
    int n_blocks;
    int pad;
};

// Adam over the flat parameters of every member (the same update as mcw_mlp_adam),
// lr and the 1-based step count read from device memory; writes the bf16 copy of every
// parameter (w16, the same layout) and the transposed copies of the table's blocks.
__global__ void adam_grouped_kernel(float *w, const float *gr, float *mo, float *ve, __nv_bfloat16 *w16,
                                    long long n, const float *lr_dev, const int *step_dev, float b1, float b2,
                                    float eps, __nv_bfloat16 *wt, long long s_t, const TransposeTable tt) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int g = blockIdx.y;
    if (i >= n) return;
    const int step = *step_dev;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    const float lr = *lr_dev;
    const size_t e = (size_t)g * n + i;
    const float gi = gr[e];
    const float m = b1 * mo[e] + (1.f - b1) * gi;
    const float v = b2 * ve[e] + (1.f - b2) * gi * gi;
    mo[e] = m;
    ve[e] = v;
    const float wn = w[e] - lr * (m / c1) / (sqrtf(v / c2) + eps);
    w[e] = wn;
    const __nv_bfloat16 h = __float2bfloat16(wn);
    w16[e] = h;
    if (wt) {
        for (int q = 0; q < tt.n_blocks; ++q) {
            const TransposeBlock &B = tt.b[q];
            const long long k = i - B.off;
            if (k >= 0 && k < (long long)B.rows * B.cols) {
                const long long o = k / B.cols, c = k % B.cols;
                wt[(size_t)g * s_t + B.off_t + (size_t)c * B.ld_t + o] = h;
            }
        }
    }
}

// Batch of the step: rows perm[g][b * batch + i] of the encoded inputs (bf16, row
// pitch 16, as x [batch, 16] and transposed [16, batch]) and of the targets, b the
// step's batch counter (device memory).
__global__ void gather_kernel(const __nv_bfloat16 *x_all, const float *t_all, long long ldt_all, int n_out,
                              const int *perm, long long n_rows, const int *counter, int batch,
                              __nv_bfloat16 *x, long long s_x, __nv_bfloat16 *xt, long long s_xt, float *t,
                              long long ldt, long long s_t) {
    const int g = blockIdx.y;
    const int i = blockIdx.x;             // row of the batch
    const long long idx = (long long)(*counter) * batch + i;
    if (idx >= n_rows) return;            // more steps than the epoch's batches: nothing to gather
    const long long src = perm[(size_t)g * n_rows + (size_t)idx];
    for (int j = threadIdx.x; j < n_out; j += blockDim.x)
        t[(size_t)g * s_t + (size_t)i * ldt + j] = t_all[(size_t)src * ldt_all + j];
    if (threadIdx.x < 16) {
        const __nv_bfloat16 v = x_all[(size_t)src * 16 + threadIdx.x];
        x[(size_t)g * s_x + (size_t)i * 16 + threadIdx.x] = v;
        xt[(size_t)g * s_xt + (size_t)threadIdx.x * batch + i] = v;
    }
}

__global__ void advance_kernel(int *counter, int *step) {
    if (threadIdx.x == 0) {
        *counter += 1;
        *step += 1;
    }
}

// ---------------------------------------------------------------- host side

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

// {k, rows, groups} bf16 tensor map, box {8, 128, 1}; false if the operand breaks a
// TMA rule (16-byte base, strides multiples of 16 bytes).
bool make_map(CUtensorMap *map, const void *base, int k, int rows, int groups, long long ld, long long stride) {
    EncodeTiledFn fn = encode_fn();
    if (!fn || !base || (reinterpret_cast<uintptr_t>(base) & 15) || (ld & 7) || ld < k) return false;
    if (groups > 1 && ((stride & 7) || stride < ld * rows)) return false;
    const long long gstride = groups > 1 ? stride : ld * rows;
    const cuuint64_t dims[3] = {(cuuint64_t)k, (cuuint64_t)rows, (cuuint64_t)groups};
    const cuuint64_t strides[2] = {(cuuint64_t)ld * 2, (cuuint64_t)gstride * 2};
    const cuuint32_t box[3] = {8, 128, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void *>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int kEpi>
cudaError_t launch_tma(const TmaGemmArgs &a, dim3 grid, cudaStream_t s) {
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] {
        attr = cudaFuncSetAttribute(gemm_tma_kernel<kEpi>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes);
    });
    if (attr != cudaSuccess) return attr;
    gemm_tma_kernel<kEpi><<<grid, 128, kSmemBytes, s>>>(a);
    return cudaGetLastError();
}

}  // namespace

unsigned int *tc_err_flag();

}  // namespace mcw

using namespace mcw;

extern "C" {

int mcw_mlp_gemm_grouped(const McwGemmGrouped *q, void *stream) {
    if (!q || q->m < 0 || q->n < 0 || q->k <= 0 || q->groups < 1 || q->splits < 1 || !q->a || !q->b || !q->c)
        return MCW_MLP_ERR_ARG;
    if (q->m == 0 || q->n == 0) return 0;
    if (q->splits > 1 && q->epilogue != MCW_EPI_F32) return MCW_MLP_ERR_ARG;
    if ((q->epilogue == MCW_EPI_BIAS_SILU) && !q->bias) return MCW_MLP_ERR_ARG;
    if (q->epilogue == MCW_EPI_DSILU && !q->aux) return MCW_MLP_ERR_ARG;
    if (q->epilogue < MCW_EPI_F32 || q->epilogue > MCW_EPI_DSILU) return MCW_MLP_ERR_ARG;
    if ((long long)q->groups * q->splits > 65535) return MCW_MLP_ERR_ARG;
    TmaGemmArgs a;
    memset(&a, 0, sizeof(a));
    if (!make_map(&a.ta, q->a, q->k, q->m, q->groups, q->lda, q->stride_a)) return MCW_MLP_ERR_ARG;
    if (!make_map(&a.tb, q->b, q->k, q->n, q->groups, q->ldb, q->stride_b)) return MCW_MLP_ERR_ARG;
    // K per split: whole chunks, and no split without a chunk
    const int chunks = (q->k + TK - 1) / TK;
    const int splits = q->splits < chunks ? q->splits : chunks;
    const int per = (chunks + splits - 1) / splits;
    a.m = q->m;
    a.n = q->n;
    a.k = q->k;
    a.kps = per * TK;
    a.splits = (chunks + per - 1) / per;
    if (a.splits != q->splits && q->splits > 1) return MCW_MLP_ERR_ARG;   // the caller's partial layout
    a.bias = q->bias;
    a.s_bias = q->stride_bias;
    a.aux = q->aux;
    a.ld_aux = q->ldaux;
    a.s_aux = q->stride_aux;
    a.c = q->c;
    a.ldc = q->ldc;
    a.s_c = q->stride_c;
    a.s_split = q->stride_split;
    a.c2 = q->c2;
    a.ldc2 = q->ldc2;
    a.s_c2 = q->stride_c2;
    a.ct = q->ct;
    a.ldct = q->ldct;
    a.s_ct = q->stride_ct;
    a.err = tc_err_flag();
    if (!a.err) return MCW_MLP_ERR_CUDA;
    const dim3 grid((q->m + TM - 1) / TM, (q->n + TN - 1) / TN, q->groups * a.splits);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    switch (q->epilogue) {
        case MCW_EPI_F32: e = launch_tma<MCW_EPI_F32>(a, grid, s); break;
        case MCW_EPI_BIAS_F32: e = launch_tma<MCW_EPI_BIAS_F32>(a, grid, s); break;
        case MCW_EPI_BIAS_SILU: e = launch_tma<MCW_EPI_BIAS_SILU>(a, grid, s); break;
        default: e = launch_tma<MCW_EPI_DSILU>(a, grid, s); break;
    }
    return e == cudaSuccess ? 0 : MCW_MLP_ERR_CUDA;
}

int mcw_mlp_reduce_splits(const float *src, int64_t stride_split, int64_t stride_src, int64_t ld_src, float *dst,
                          int64_t stride_dst, int64_t ld_dst, int32_t splits, int32_t groups, int32_t m, int32_t n,
                          void *stream) {
    if (!src || !dst || splits < 1 || groups < 1 || m < 0 || n < 0) return MCW_MLP_ERR_ARG;
    if (m == 0 || n == 0) return 0;
    const long long total = (long long)m * n;
    const int blocks = (int)((total + 255) / 256 < 1024 ? (total + 255) / 256 : 1024);
    reduce_splits_kernel<<<dim3(blocks, 1, groups), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        src, stride_split, stride_src, ld_src, dst, stride_dst, ld_dst, splits, m, n);
    return cudaGetLastError() == cudaSuccess ? 0 : MCW_MLP_ERR_CUDA;
}

int mcw_mlp_loss_grouped(const float *y, int64_t ldy, int64_t stride_y, const float *t, int64_t ldt,
                         int64_t stride_t, const float *w, int32_t groups, int32_t m, int32_t n, float *g32,
                         int64_t ldg, int64_t stride_g32, void *g16, int64_t stride_g16, void *g16t, int64_t ldgt,
                         int64_t stride_g16t, float *loss, void *stream) {
    if (!y || !t || !g32 || !g16 || !g16t || !loss || groups < 1 || m < 0 || n < 0) return MCW_MLP_ERR_ARG;
    if (m == 0 || n == 0) return 0;
    const dim3 grid((n + 31) / 32, (m + kLossRows - 1) / kLossRows, groups);
    loss_grouped_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        y, ldy, stride_y, t, ldt, stride_t, w, m, n, g32, ldg, stride_g32, static_cast<__nv_bfloat16 *>(g16),
        stride_g16, static_cast<__nv_bfloat16 *>(g16t), ldgt, stride_g16t, loss);
    return cudaGetLastError() == cudaSuccess ? 0 : MCW_MLP_ERR_CUDA;
}

int mcw_mlp_colsum_grouped(const McwColsumLayer *layers, int32_t n_layers, int32_t groups, int32_t m, float *out,
                           int64_t stride_out, float *partial, int32_t rows_per_chunk, void *stream) {
    if (!layers || n_layers < 1 || n_layers > 4 || groups < 1 || m < 0 || !out) return MCW_MLP_ERR_ARG;
    ColsumTable tab;
    memset(&tab, 0, sizeof(tab));
    int nmax = 0;
    for (int q = 0; q < n_layers; ++q) {
        if (!layers[q].g || layers[q].n < 0) return MCW_MLP_ERR_ARG;
        tab.l[q].src = layers[q].g;
        tab.l[q].ld = layers[q].ld;
        tab.l[q].s_g = layers[q].stride;
        tab.l[q].off = layers[q].out_offset;
        tab.l[q].n = layers[q].n;
        nmax = layers[q].n > nmax ? layers[q].n : nmax;
    }
    tab.n_layers = n_layers;
    if (nmax == 0) return 0;
    const bool split = partial && rows_per_chunk > 0 && rows_per_chunk < m;
    const int rpc = split ? rows_per_chunk : (m > 0 ? m : 1);
    const int chunks = (m + rpc - 1) / rpc > 0 ? (m + rpc - 1) / rpc : 1;
    if (chunks > 65535 || (long long)n_layers * groups > 65535) return MCW_MLP_ERR_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    colsum_grouped_kernel<<<dim3((nmax + 31) / 32, chunks, n_layers * groups), 256, 0, s>>>(
        tab, groups, m, rpc, out, stride_out, split ? partial : nullptr, nmax);
    if (split)
        colsum_finish_kernel<<<dim3((nmax + 127) / 128, 1, n_layers * groups), 128, 0, s>>>(
            tab, groups, chunks, partial, nmax, out, stride_out);
    return cudaGetLastError() == cudaSuccess ? 0 : MCW_MLP_ERR_CUDA;
}

int mcw_mlp_adam_grouped(float *w, const float *g, float *m, float *v, void *w16, int64_t n, int32_t groups,
                         const float *lr_dev, const int32_t *step_dev, float beta1, float beta2, float eps,
                         void *wt, int64_t stride_t, const McwTransposeBlock *blocks, int32_t n_blocks,
                         void *stream) {
    if (!w || !g || !m || !v || !w16 || !lr_dev || !step_dev || n < 0 || groups < 1 || n_blocks < 0 ||
        n_blocks > 4 || (n_blocks > 0 && (!blocks || !wt)))
        return MCW_MLP_ERR_ARG;
    if (n == 0) return 0;
    TransposeTable tt;
    memset(&tt, 0, sizeof(tt));
    for (int q = 0; q < n_blocks; ++q) {
        if (blocks[q].offset < 0 || blocks[q].rows < 0 || blocks[q].cols < 0 ||
            blocks[q].offset + (int64_t)blocks[q].rows * blocks[q].cols > n || blocks[q].ld_t < blocks[q].rows)
            return MCW_MLP_ERR_ARG;
        tt.b[q].off = blocks[q].offset;
        tt.b[q].off_t = blocks[q].offset_t;
        tt.b[q].ld_t = blocks[q].ld_t;
        tt.b[q].rows = blocks[q].rows;
        tt.b[q].cols = blocks[q].cols;
    }
    tt.n_blocks = n_blocks;
    const dim3 grid((unsigned)((n + 255) / 256), groups);
    adam_grouped_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        w, g, m, v, static_cast<__nv_bfloat16 *>(w16), n, lr_dev, step_dev, beta1, beta2, eps,
        static_cast<__nv_bfloat16 *>(wt), stride_t, tt);
    return cudaGetLastError() == cudaSuccess ? 0 : MCW_MLP_ERR_CUDA;
}

int mcw_mlp_gather(const void *x_all, const float *t_all, int64_t ldt_all, int32_t n_out, const int32_t *perm,
                   int64_t n_rows, const int32_t *counter_dev, int32_t batch, int32_t groups, void *x,
                   int64_t stride_x, void *xt, int64_t stride_xt, float *t, int64_t ldt, int64_t stride_t,
                   void *stream) {
    if (!x_all || !t_all || !perm || !counter_dev || !x || !xt || !t || batch < 1 || groups < 1 || n_out < 0 ||
        n_rows < batch)
        return MCW_MLP_ERR_ARG;
    gather_kernel<<<dim3(batch, groups), 128, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const __nv_bfloat16 *>(x_all), t_all, ldt_all, n_out, perm, n_rows, counter_dev, batch,
        static_cast<__nv_bfloat16 *>(x), stride_x, static_cast<__nv_bfloat16 *>(xt), stride_xt, t, ldt, stride_t);
    return cudaGetLastError() == cudaSuccess ? 0 : MCW_MLP_ERR_CUDA;
}

int mcw_mlp_advance(int32_t *counter_dev, int32_t *step_dev, void *stream) {
    if (!counter_dev || !step_dev) return MCW_MLP_ERR_ARG;
    advance_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(counter_dev, step_dev);
    return cudaGetLastError() == cudaSuccess ? 0 : MCW_MLP_ERR_CUDA;
}

}  // extern "C"
