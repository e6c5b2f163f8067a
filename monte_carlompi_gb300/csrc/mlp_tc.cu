// GEMM of the surrogate network on the 5th-generation tensor cores:
// C[m, n] = sum_k A(m, k) B(n, k), bf16 operands stored K-major ([m, k], [n, k]) or
// transposed ([k, m], [k, n]), FP32 accumulation in tensor memory, fused epilogues
// (bias, bias + SiLU, SiLU' product of the backward pass).  Used for the forward and
// the backward GEMMs of training.
//
// One CTA of four warps computes a 128 x 128 tile.  K is walked in chunks of 64
// through two shared-memory buffers: all threads stage chunk k + 1 as 8 x 16-byte
// core matrices (no swizzle; 128 B apart along K, 1024 B apart along M / N) while
// the tensor core runs chunk k's four tcgen05.mma (K = 16 each), issued by one
// thread into a 128-column TMEM accumulator and committed to the buffer's mbarrier;
// a buffer is restaged only after that barrier reports its MMAs complete (bounded
// wait).  Transposed operands are staged with rows fastest across the threads, so a
// warp's loads of one k cover 32 consecutive rows.  The epilogue reads the
// accumulator with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31, i.e. tile rows).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <mutex>

#include "../../include/mcw_mlp.h"

namespace mcw {

namespace {

constexpr int TM = 128, TN = 128, TK = 64;
constexpr int kChunkBytes = TM * TK * 2;          // 16 KB per operand chunk
constexpr int kBufBytes = 2 * kChunkBytes;        // A and B chunks of one buffer
constexpr uint32_t kTmemCols = 128;
constexpr unsigned long long kWaitNs = 2000000000ull;  // bounded wait on an MMA barrier (2 s)

// Instruction descriptor of tcgen05.mma kind::f16: F32 accumulate, BF16 A and B,
// both K-major, N = 128 (bits 17-22: N >> 3), M = 128 (bits 24-28: M >> 4).
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) |
                            ((uint32_t)(TM >> 4) << 24);

// Shared-memory matrix descriptor, no swizzle: start >> 4 (bits 0-13), leading
// byte offset >> 4 (bits 16-29, K-adjacent core matrices), stride byte offset
// >> 4 (bits 32-45, M/N-adjacent core matrices), descriptor version 1 (bit 46).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
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

// Stage a 128-row x 64-k chunk into the core-matrix layout; rows >= rows_valid and
// k >= K read as zero.  Stored K-major (g[row * ld + k]): 16-byte loads along k.  All
// eight loads of a thread are issued before any store, so their latencies overlap.
__device__ __forceinline__ void stage_chunk(unsigned char *dst, const __nv_bfloat16 *g, int ld, int row0,
                                            int rows_valid, int k0, int K, bool vec) {
    const bool full = vec && row0 + 128 <= rows_valid && k0 + 64 <= K;
    uint4 v[8];
    if (full) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int c = threadIdx.x + 128 * q;  // 1024 chunks of 16 B
            const int r = c >> 3, k8 = c & 7;
            v[q] = __ldg(reinterpret_cast<const uint4 *>(g + (size_t)(row0 + r) * ld + k0 + k8 * 8));
        }
    } else {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int c = threadIdx.x + 128 * q;
            const int r = c >> 3, k8 = c & 7;
            const int gr = row0 + r, gk = k0 + k8 * 8;
            __align__(16) __nv_bfloat16 tmp[8];
#pragma unroll
            for (int e = 0; e < 8; ++e)
                tmp[e] = (gr < rows_valid && gk + e < K) ? g[(size_t)gr * ld + gk + e] : __float2bfloat16(0.f);
            v[q] = *reinterpret_cast<const uint4 *>(tmp);
        }
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int c = threadIdx.x + 128 * q;
        const int r = c >> 3, k8 = c & 7;
        *reinterpret_cast<uint4 *>(dst + (r >> 3) * 1024 + k8 * 128 + (r & 7) * 16) = v[q];
    }
}

// The same from a transposed operand (g[k * ld + row]): thread c takes row c % 128,
// so for each k a warp reads 32 consecutive rows; four 16-byte chunks' loads at a time.
__device__ __forceinline__ void stage_chunk_t(unsigned char *dst, const __nv_bfloat16 *g, int ld, int row0,
                                              int rows_valid, int k0, int K) {
    const bool full = row0 + 128 <= rows_valid && k0 + 64 <= K;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        __nv_bfloat16 tv[4][8];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int c = threadIdx.x + 128 * (4 * half + q);
            const int r = c & 127, k8 = c >> 7;
            const int gr = row0 + r, gk = k0 + k8 * 8;
#pragma unroll
            for (int e = 0; e < 8; ++e)
                tv[q][e] = (full || (gr < rows_valid && gk + e < K)) ? g[(size_t)(gk + e) * ld + gr]
                                                                     : __float2bfloat16(0.f);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int c = threadIdx.x + 128 * (4 * half + q);
            const int r = c & 127, k8 = c >> 7;
            __align__(16) __nv_bfloat16 tmp[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) tmp[e] = tv[q][e];
            *reinterpret_cast<uint4 *>(dst + (r >> 3) * 1024 + k8 * 128 + (r & 7) * 16) =
                *reinterpret_cast<const uint4 *>(tmp);
        }
    }
}

__device__ __forceinline__ bool bar_wait(uint64_t *bar, uint32_t parity) {
    const unsigned long long t0 = now_ns();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done) : "r"(smem_u32(bar)), "r"(parity));
        if (done) return true;
        if (now_ns() - t0 > kWaitNs) return false;
    }
}

template <int kEpi>
__global__ void __launch_bounds__(128) gemm_tc_kernel(const McwGemm p, unsigned int *err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_base_slot;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * TM, n0 = blockIdx.y * TN;
    const __nv_bfloat16 *A = static_cast<const __nv_bfloat16 *>(p.a);
    const __nv_bfloat16 *W = static_cast<const __nv_bfloat16 *>(p.b);
    const bool vec_a = ((reinterpret_cast<uintptr_t>(A) & 15) == 0) && ((p.lda & 7) == 0);
    const bool vec_b = ((reinterpret_cast<uintptr_t>(W) & 15) == 0) && ((p.ldb & 7) == 0);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
                     :: "r"(smem_u32(&tmem_base_slot)), "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(&mbar[0])));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(smem_u32(&mbar[1])));
        asm volatile("fence.mbarrier_init.release.cluster;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem = tmem_base_slot;

    bool ok = true;
    uint32_t phase[2] = {0u, 0u};
    bool pending[2] = {false, false};
    const int n_chunks = (p.k + TK - 1) / TK;
    for (int kc = 0; kc < n_chunks && ok; ++kc) {
        const int b = kc & 1;
        unsigned char *sa = smem + b * kBufBytes;
        unsigned char *sb = sa + kChunkBytes;
        // the buffer's previous MMAs (chunk kc - 2) must be done before it is restaged
        if (pending[b]) {
            ok = __syncthreads_and(bar_wait(&mbar[b], phase[b])) != 0;
            if (!ok) break;
            phase[b] ^= 1u;
            pending[b] = false;
        }
        const int k0 = kc * TK;
        if (p.trans_a) stage_chunk_t(sa, A, p.lda, m0, p.m, k0, p.k);
        else stage_chunk(sa, A, p.lda, m0, p.m, k0, p.k, vec_a);
        if (p.trans_b) stage_chunk_t(sb, W, p.ldb, n0, p.n, k0, p.k);
        else stage_chunk(sb, W, p.ldb, n0, p.n, k0, p.k, vec_b);
        // make the generic-proxy stores visible to the tensor core (async proxy)
        asm volatile("fence.proxy.async.shared::cta;\n");
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n");
            const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
#pragma unroll
            for (int s = 0; s < TK / 16; ++s) {
                const uint64_t da = smem_desc(a0 + s * 256, 128, 1024);
                const uint64_t db = smem_desc(b0 + s * 256, 128, 1024);
                const uint32_t accumulate = (kc > 0 || s > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
                    :: "r"(tmem), "l"(da), "l"(db), "r"(kIdesc), "r"(accumulate));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n"
                         :: "r"(smem_u32(&mbar[b])));
        }
        pending[b] = true;
    }
    // the last MMAs (and with them all earlier ones) complete before the epilogue
    for (int b = 0; b < 2 && ok; ++b) {
        if (pending[b]) {
            ok = __syncthreads_and(bar_wait(&mbar[b], phase[b])) != 0;
            if (ok) pending[b] = false;
        }
    }
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    if (!ok) {
        if (threadIdx.x == 0) atomicOr(err, 1u);
        // MMAs still in flight finish (bounded) before the memory is freed
        for (int b = 0; b < 2; ++b)
            if (pending[b]) bar_wait(&mbar[b], phase[b]);
    }

    if (ok) {
        // epilogue: warp w holds rows m0 + 32w + lane, 32 columns per load
        const int m = m0 + warp * 32 + lane;
#pragma unroll
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
            asm volatile("tcgen05.wait::ld.sync.aligned;\n");
            const int nb = n0 + c0;
            if (m < p.m && nb < p.n) {
                const int cnt = min(32, p.n - nb);
                // the inputs of the 32 columns first (their loads overlap), then the stores
                float add[32];
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    add[j] = 0.f;
                    if (j < cnt) {
                        if (kEpi == MCW_EPI_DSILU) add[j] = __ldg(p.aux + (size_t)m * p.ldaux + nb + j);
                        else if (kEpi != MCW_EPI_F32 && p.bias) add[j] = __ldg(p.bias + nb + j);
                    }
                }
                float z[32];
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    z[j] = __uint_as_float(v[j]);
                    if (kEpi == MCW_EPI_DSILU) z[j] *= dsilu(add[j]);
                    else z[j] += add[j];
                }
                float *c32 = nullptr;
                if (kEpi == MCW_EPI_F32 || kEpi == MCW_EPI_BIAS_F32) c32 = static_cast<float *>(p.c) + (size_t)m * p.ldc + nb;
                else if (p.c2) c32 = static_cast<float *>(p.c2) + (size_t)m * p.ldc2 + nb;
                __nv_bfloat16 *c16 = nullptr;
                if (kEpi == MCW_EPI_BIAS_SILU || kEpi == MCW_EPI_DSILU)
                    c16 = static_cast<__nv_bfloat16 *>(p.c) + (size_t)m * p.ldc + nb;
                if (c32) {
                    if (cnt == 32 && (reinterpret_cast<uintptr_t>(c32) & 15) == 0) {
#pragma unroll
                        for (int q = 0; q < 8; ++q)
                            reinterpret_cast<float4 *>(c32)[q] =
                                make_float4(z[4 * q], z[4 * q + 1], z[4 * q + 2], z[4 * q + 3]);
                    } else {
#pragma unroll
                        for (int j = 0; j < 32; ++j)
                            if (j < cnt) c32[j] = z[j];
                    }
                }
                if (c16) {
                    __align__(16) __nv_bfloat16 h[32];
#pragma unroll
                    for (int j = 0; j < 32; ++j)
                        h[j] = __float2bfloat16(kEpi == MCW_EPI_BIAS_SILU ? silu(z[j]) : z[j]);
                    if (cnt == 32 && (reinterpret_cast<uintptr_t>(c16) & 15) == 0) {
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            reinterpret_cast<uint4 *>(c16)[q] = reinterpret_cast<const uint4 *>(h)[q];
                    } else {
#pragma unroll
                        for (int j = 0; j < 32; ++j)
                            if (j < cnt) c16[j] = h[j];
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" :: "r"(tmem), "r"(kTmemCols));
    }
}

}  // namespace

// Error flags of the tensor-core GEMM (bit 0: an MMA barrier wait timed out), one
// word per device, read and cleared by mcw_mlp_status.
static __device__ unsigned int g_tc_err;

unsigned int *tc_err_flag() {
    // looked up once per device (no runtime call while a stream is being captured)
    static std::mutex mu;
    static std::map<int, unsigned int *> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(mu);
    const auto it = cache.find(dev);
    if (it != cache.end()) return it->second;
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_tc_err) != cudaSuccess) return nullptr;
    cache[dev] = static_cast<unsigned int *>(p);
    return static_cast<unsigned int *>(p);
}

// Dynamic shared memory: two buffers of two 16 KB chunks (at most three CTAs per SM,
// 3 x 128 TMEM columns of the SM's 512).
constexpr size_t kTcSmem = 2 * kBufBytes;

cudaError_t launch_gemm_tc(const McwGemm &p, unsigned int *err, cudaStream_t s) {
    dim3 grid((p.m + TM - 1) / TM, (p.n + TN - 1) / TN);
    cudaError_t e;
    switch (p.epilogue) {
        case MCW_EPI_BIAS_SILU:
            e = cudaFuncSetAttribute(gemm_tc_kernel<MCW_EPI_BIAS_SILU>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
            if (e != cudaSuccess) return e;
            gemm_tc_kernel<MCW_EPI_BIAS_SILU><<<grid, 128, kTcSmem, s>>>(p, err);
            break;
        case MCW_EPI_BIAS_F32:
            e = cudaFuncSetAttribute(gemm_tc_kernel<MCW_EPI_BIAS_F32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
            if (e != cudaSuccess) return e;
            gemm_tc_kernel<MCW_EPI_BIAS_F32><<<grid, 128, kTcSmem, s>>>(p, err);
            break;
        case MCW_EPI_F32:
            e = cudaFuncSetAttribute(gemm_tc_kernel<MCW_EPI_F32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
            if (e != cudaSuccess) return e;
            gemm_tc_kernel<MCW_EPI_F32><<<grid, 128, kTcSmem, s>>>(p, err);
            break;
        case MCW_EPI_DSILU:
            e = cudaFuncSetAttribute(gemm_tc_kernel<MCW_EPI_DSILU>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
            if (e != cudaSuccess) return e;
            gemm_tc_kernel<MCW_EPI_DSILU><<<grid, 128, kTcSmem, s>>>(p, err);
            break;
        default:
            return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace mcw
