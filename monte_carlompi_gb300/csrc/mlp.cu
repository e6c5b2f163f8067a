// Kernels of the BRF surrogate MLP (4 -> 256 -> 256 -> 256 -> 649, SiLU):
// BF16 tensor-core GEMMs with FP32 accumulation and fused epilogues, bias
// gradients, the loss and its gradient, Adam on FP32 master weights, and the
// FP32 -> BF16 weight copy.
//
// GEMM: C[M,N] = sum_k A(m,k) B(n,k), tiles of 64 x 64 x 32 per block of four
// warps, each warp 32 x 32 as 2 x 4 mma.sync.m16n8k16 (bf16 in, f32 out).
// A is stored [M,K] (trans_a = 0) or [K,M] (trans_a = 1); B is stored [N,K]
// (trans_b = 0) or [K,N] (trans_b = 1).  Tiles are staged in shared memory with
// K contiguous (transposed on the way in when needed), rows padded to 40
// elements so ldmatrix reads are conflict-free.  Out-of-range rows and columns
// read as zero and are not stored.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/mcw_mlp.h"

namespace mcw {

namespace {

constexpr int BM = 64, BN = 64, BK = 32, LDS = BK + 8;

__device__ __forceinline__ float silu(float z) { return __fdividef(z, 1.f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
    const float s = 1.f / (1.f + __expf(-z));
    return s * (1.f + z * (1.f - s));
}

// Load a 64 x 32 tile of a bf16 operand into shared memory [64][LDS] with K
// contiguous.  Stored [rows, K] row-major (ld = leading dimension) when
// !trans, or [K, rows] row-major when trans.
template <bool kTrans>
__device__ __forceinline__ void load_tile(__nv_bfloat16 (*s)[LDS], const __nv_bfloat16 *g, int ld, int row0,
                                          int rows, int k0, int K) {
    const int t = threadIdx.x;
    const bool vec = ((reinterpret_cast<uintptr_t>(g) & 15) == 0) && ((ld & 7) == 0);
    if (!kTrans) {
        // 64 rows x 32 k = 256 chunks of 8 elements (16 B); 2 per thread
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int c = t + q * 128;
            const int r = c >> 2, kk = (c & 3) * 8;
            const int gr = row0 + r, gk = k0 + kk;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (vec && gr < rows && gk + 8 <= K) {
                v = *reinterpret_cast<const uint4 *>(g + (size_t)gr * ld + gk);
            } else if (gr < rows) {
                __align__(16) __nv_bfloat16 tmp[8];
#pragma unroll
                for (int e = 0; e < 8; ++e)
                    tmp[e] = (gk + e < K) ? g[(size_t)gr * ld + gk + e] : __float2bfloat16(0.f);
                v = *reinterpret_cast<uint4 *>(tmp);
            }
            *reinterpret_cast<uint4 *>(&s[r][kk]) = v;
        }
    } else {
        // element (row r, k kk) lives at g[(k0 + kk) * ld + row0 + r]; 2048 elements, 16 per thread
#pragma unroll 4
        for (int q = 0; q < 16; ++q) {
            const int e = t + q * 128;
            const int kk = e >> 6, r = e & 63;
            const int gr = row0 + r, gk = k0 + kk;
            s[r][kk] = (gr < rows && gk < K) ? g[(size_t)gk * ld + gr] : __float2bfloat16(0.f);
        }
    }
}

__device__ __forceinline__ void ldmatrix_x4(uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3, const void *p) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(a));
}

__device__ __forceinline__ void ldmatrix_x2(uint32_t &r0, uint32_t &r1, const void *p) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(a));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <bool kTA, bool kTB, int kEpi>
__global__ void __launch_bounds__(128) gemm_kernel(const McwGemm p) {
    __shared__ __align__(16) __nv_bfloat16 sA[BM][LDS];
    __shared__ __align__(16) __nv_bfloat16 sB[BN][LDS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const __nv_bfloat16 *A = static_cast<const __nv_bfloat16 *>(p.a);
    const __nv_bfloat16 *B = static_cast<const __nv_bfloat16 *>(p.b);
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;

    for (int k0 = 0; k0 < p.k; k0 += BK) {
        load_tile<kTA>(sA, A, p.lda, m0, p.m, k0, p.k);
        load_tile<kTB>(sB, B, p.ldb, n0, p.n, k0, p.k);
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            uint32_t af[2][4], bfr[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = wm + i * 16 + (lane & 15);
                const int c = kk + (lane >> 4) * 8;
                ldmatrix_x4(af[i][0], af[i][1], af[i][2], af[i][3], &sA[r][c]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int r = wn + j * 8 + (lane & 7);
                const int c = kk + ((lane >> 3) & 1) * 8;
                ldmatrix_x2(bfr[j][0], bfr[j][1], &sB[r][c]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bfr[j]);
        }
        __syncthreads();
    }

    // epilogue: fragment element e of tile (i, j) is row wm+16i+lane/4 (+8 for e >= 2),
    // column wn+8j+2(lane%4) (+1 for odd e)
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int m = m0 + wm + i * 16 + (lane >> 2) + ((e >> 1) << 3);
                const int n = n0 + wn + j * 8 + (lane & 3) * 2 + (e & 1);
                if (m >= p.m || n >= p.n) continue;
                float v = acc[i][j][e];
                if (kEpi == MCW_EPI_BIAS_SILU) {
                    v += p.bias[n];
                    if (p.c2) static_cast<float *>(p.c2)[(size_t)m * p.ldc2 + n] = v;  // pre-activation
                    static_cast<__nv_bfloat16 *>(p.c)[(size_t)m * p.ldc + n] = __float2bfloat16(silu(v));
                } else if (kEpi == MCW_EPI_BIAS_F32) {
                    if (p.bias) v += p.bias[n];
                    static_cast<float *>(p.c)[(size_t)m * p.ldc + n] = v;
                } else if (kEpi == MCW_EPI_DSILU) {
                    v *= dsilu(p.aux[(size_t)m * p.ldaux + n]);
                    static_cast<__nv_bfloat16 *>(p.c)[(size_t)m * p.ldc + n] = __float2bfloat16(v);
                    if (p.c2) static_cast<float *>(p.c2)[(size_t)m * p.ldc2 + n] = v;
                } else {  // MCW_EPI_F32
                    static_cast<float *>(p.c)[(size_t)m * p.ldc + n] = v;
                }
            }
}

template <bool kTA, bool kTB>
cudaError_t launch_gemm(const McwGemm &p, cudaStream_t s) {
    dim3 grid((p.m + BM - 1) / BM, (p.n + BN - 1) / BN);
    switch (p.epilogue) {
        case MCW_EPI_F32: gemm_kernel<kTA, kTB, MCW_EPI_F32><<<grid, 128, 0, s>>>(p); break;
        case MCW_EPI_BIAS_F32: gemm_kernel<kTA, kTB, MCW_EPI_BIAS_F32><<<grid, 128, 0, s>>>(p); break;
        case MCW_EPI_BIAS_SILU: gemm_kernel<kTA, kTB, MCW_EPI_BIAS_SILU><<<grid, 128, 0, s>>>(p); break;
        case MCW_EPI_DSILU: gemm_kernel<kTA, kTB, MCW_EPI_DSILU><<<grid, 128, 0, s>>>(p); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// db[n] = sum_m G[m, n] (fp32 G, ld = ldg), one warp per column block of 32.
__global__ void colsum_kernel(const float *g, int m, int n, int ldg, float *out) {
    const int col = blockIdx.x * 32 + (threadIdx.x & 31);
    const int row0 = threadIdx.x >> 5;
    __shared__ float part[8][32];
    float acc = 0.f;
    if (col < n)
        for (int r = row0; r < m; r += 8) acc += g[(size_t)r * ldg + col];
    part[row0][threadIdx.x & 31] = acc;
    __syncthreads();
    if (row0 == 0 && col < n) {
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < 8; ++q) s += part[q][threadIdx.x];
        out[col] = s;
    }
}

// Weighted squared error: loss += sum w_n (y - t)^2 / (m * n_out); grad = d loss / d y.
__global__ void loss_kernel(const float *y, int ldy, const float *t, int ldt, const float *w, int m, int n,
                            float *grad, int ldg, __nv_bfloat16 *grad16, int ldg16, float *loss) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (idx < m * n) {
        const int r = idx / n, c = idx % n;
        const float d = y[(size_t)r * ldy + c] - t[(size_t)r * ldt + c];
        const float wc = w ? w[c] : 1.f;
        const float scale = 1.f / ((float)m * (float)n);
        l = wc * d * d * scale;
        const float gv = 2.f * wc * d * scale;
        grad[(size_t)r * ldg + c] = gv;
        grad16[(size_t)r * ldg16 + c] = __float2bfloat16(gv);
    }
    for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0 && l != 0.f) atomicAdd(loss, l);
}

// Adam on FP32 master weights; writes the BF16 copy used by the GEMMs.
__global__ void adam_kernel(float *w, const float *g, float *mo, float *ve, __nv_bfloat16 *w16, int n, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float m = b1 * mo[i] + (1.f - b1) * gi;
    const float v = b2 * ve[i] + (1.f - b2) * gi * gi;
    mo[i] = m;
    ve[i] = v;
    const float wn = w[i] - lr * (m / c1) / (sqrtf(v / c2) + eps);
    w[i] = wn;
    if (w16) w16[i] = __float2bfloat16(wn);
}

__global__ void cast_kernel(const float *x, __nv_bfloat16 *y, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __float2bfloat16(x[i]);
}

}  // namespace

cudaError_t launch_gemm_tc(const McwGemm &p, unsigned int *err, cudaStream_t s);
unsigned int *tc_err_flag();

}  // namespace mcw

using namespace mcw;

extern "C" {

int mcw_mlp_gemm(const McwGemm *p, void *stream) {
    if (!p || p->m < 0 || p->n < 0 || p->k < 0 || !p->a || !p->b || !p->c) return MCW_MLP_ERR_ARG;
    if (p->epilogue == MCW_EPI_BIAS_SILU && !p->bias) return MCW_MLP_ERR_ARG;
    if (p->epilogue == MCW_EPI_DSILU && !p->aux) return MCW_MLP_ERR_ARG;
    if (p->engine < MCW_ENGINE_MMA_SYNC || p->engine > MCW_ENGINE_TCGEN05) return MCW_MLP_ERR_ARG;
    if (p->m == 0 || p->n == 0) return 0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    if (p->engine == MCW_ENGINE_TCGEN05) {
        unsigned int *err = tc_err_flag();
        if (!err) return MCW_MLP_ERR_CUDA;
        e = launch_gemm_tc(*p, err, s);
        return e == cudaSuccess ? 0 : MCW_MLP_ERR_CUDA;
    }
    if (!p->trans_a && !p->trans_b) e = launch_gemm<false, false>(*p, s);
    else if (!p->trans_a && p->trans_b) e = launch_gemm<false, true>(*p, s);
    else if (p->trans_a && !p->trans_b) e = launch_gemm<true, false>(*p, s);
    else e = launch_gemm<true, true>(*p, s);
    return e == cudaSuccess ? 0 : MCW_MLP_ERR_CUDA;
}

int mcw_mlp_colsum(const float *g, int32_t m, int32_t n, int32_t ldg, float *out, void *stream) {
    if (!g || !out || m < 0 || n < 0) return MCW_MLP_ERR_ARG;
    if (n == 0) return 0;
    colsum_kernel<<<(n + 31) / 32, 256, 0, static_cast<cudaStream_t>(stream)>>>(g, m, n, ldg, out);
    return cudaGetLastError() == cudaSuccess ? 0 : MCW_MLP_ERR_CUDA;
}

int mcw_mlp_loss(const float *y, int32_t ldy, const float *t, int32_t ldt, const float *w, int32_t m, int32_t n,
                 float *grad, int32_t ldg, void *grad16, int32_t ldg16, float *loss, void *stream) {
    if (!y || !t || !grad || !grad16 || !loss || m < 0 || n < 0) return MCW_MLP_ERR_ARG;
    const int total = m * n;
    if (total == 0) return 0;
    loss_kernel<<<(total + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        y, ldy, t, ldt, w, m, n, grad, ldg, static_cast<__nv_bfloat16 *>(grad16), ldg16, loss);
    return cudaGetLastError() == cudaSuccess ? 0 : MCW_MLP_ERR_CUDA;
}

int mcw_mlp_adam(float *w, const float *g, float *m, float *v, void *w16, int64_t n, float lr, float beta1,
                 float beta2, float eps, int64_t step, void *stream) {
    if (!w || !g || !m || !v || n < 0 || step < 1) return MCW_MLP_ERR_ARG;
    if (n == 0) return 0;
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    adam_kernel<<<(int)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        w, g, m, v, static_cast<__nv_bfloat16 *>(w16), (int)n, lr, beta1, beta2, eps, c1, c2);
    return cudaGetLastError() == cudaSuccess ? 0 : MCW_MLP_ERR_CUDA;
}

int mcw_mlp_status(int32_t clear, uint32_t *flags) {
    if (!flags) return MCW_MLP_ERR_ARG;
    unsigned int *err = tc_err_flag();
    if (!err) return MCW_MLP_ERR_CUDA;
    unsigned int h = 0;
    if (cudaMemcpy(&h, err, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return MCW_MLP_ERR_CUDA;
    *flags = h;
    if (clear && h) {
        h = 0;
        if (cudaMemcpy(err, &h, sizeof(h), cudaMemcpyHostToDevice) != cudaSuccess) return MCW_MLP_ERR_CUDA;
    }
    return 0;
}

int mcw_mlp_cast_bf16(const float *x, void *y, int64_t n, void *stream) {
    if (!x || !y || n < 0) return MCW_MLP_ERR_ARG;
    if (n == 0) return 0;
    cast_kernel<<<(int)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        x, static_cast<__nv_bfloat16 *>(y), (int)n);
    return cudaGetLastError() == cudaSuccess ? 0 : MCW_MLP_ERR_CUDA;
}

}  // extern "C"
