/*
 * mcw_mlp.h - kernels of the BRF surrogate network (libmcwalk.so).
 *
 * The surrogate maps (r_eff, lambda, cos theta0, depth) to the 648-bin BRF and
 * the albedo that the walk (mcwalk.h) would produce; it has no counterpart in
 * the reference, whose only route to a BRF is the Monte Carlo walk plus
 * post_processing.py:46-100.  All pointers are device pointers; all calls are
 * asynchronous on the given cudaStream_t (NULL = default stream) and return 0
 * or a negative MCW_MLP_ERR_*.
 */
#ifndef MCW_MLP_H
#define MCW_MLP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCW_MLP_ERR_ARG (-1)
#define MCW_MLP_ERR_CUDA (-2)

/* GEMM engines */
#define MCW_ENGINE_MMA_SYNC 0  /* mma.sync m16n8k16 */
#define MCW_ENGINE_TCGEN05 1   /* tcgen05.mma into tensor memory, double-buffered K chunks */
/* Both engines take any operand layout and every epilogue. */

/* GEMM epilogues */
#define MCW_EPI_F32 0        /* c (f32) = acc */
#define MCW_EPI_BIAS_F32 1   /* c (f32) = acc + bias (bias may be NULL) */
#define MCW_EPI_BIAS_SILU 2  /* c2 (f32, optional) = z = acc + bias; c (bf16) = silu(z) */
#define MCW_EPI_DSILU 3      /* g = acc * silu'(aux); c (bf16) = g; c2 (f32, optional) = g */

/* C[m, n] = sum_k A(m, k) B(n, k) on BF16 tensor cores with FP32 accumulation.
 * A is bf16 stored [m, k] (trans_a = 0) or [k, m] (trans_a = 1), leading
 * dimension lda; B is bf16 stored [n, k] (trans_b = 0) or [k, n] (trans_b = 1). */
typedef struct {
    int32_t m, n, k;
    int32_t trans_a, trans_b;
    int32_t epilogue;
    const void *a;
    int32_t lda;
    int32_t ldb;
    const void *b;
    const float *bias;   /* n */
    const float *aux;    /* [m, n] pre-activation for MCW_EPI_DSILU */
    int32_t ldaux;
    int32_t ldc;
    void *c;
    void *c2;
    int32_t ldc2;
    int32_t engine;      /* MCW_ENGINE_* */
} McwGemm;

int mcw_mlp_gemm(const McwGemm *p, void *stream);

/* out[j] = sum_i g[i * ldg + j] for j < n (bias gradients). */
int mcw_mlp_colsum(const float *g, int32_t m, int32_t n, int32_t ldg, float *out, void *stream);

/* Weighted mean squared error of y [m, n] against t: *loss += sum_ij w_j (y-t)^2 / (m n);
 * grad (f32) and grad16 (bf16) receive its gradient with respect to y.  w may be NULL. */
int mcw_mlp_loss(const float *y, int32_t ldy, const float *t, int32_t ldt, const float *w, int32_t m,
                 int32_t n, float *grad, int32_t ldg, void *grad16, int32_t ldg16, float *loss,
                 void *stream);

/* Adam step `step` (1-based) on n FP32 master weights; w16 (bf16, optional) receives the
 * updated weights for the GEMMs. */
int mcw_mlp_adam(float *w, const float *g, float *m, float *v, void *w16, int64_t n, float lr,
                 float beta1, float beta2, float eps, int64_t step, void *stream);

/* Error flags of the tensor-core path on the current device (bit 0: an MMA completion
 * wait of the tcgen05 GEMM ran out of time and the kernel left early; bit 1: the same in
 * mcw_mlp_forward); clear != 0 resets them. */
int mcw_mlp_status(int32_t clear, uint32_t *flags);

/* y (bf16) = x (f32), n elements. */
int mcw_mlp_cast_bf16(const float *x, void *y, int64_t n, void *stream);

/* Fused inference of the whole network MCW_MLP_IN -> 3 x MCW_MLP_HIDDEN (SiLU) -> MCW_MLP_OUT. */
#define MCW_MLP_IN 4
#define MCW_MLP_HIDDEN 256
#define MCW_MLP_OUT 649
/* five 256 x 256 bf16 blocks (W2, W3, three 256-row blocks of W4) and the 256 x 16 W1 tile */
#define MCW_MLP_PACK_BYTES (5 * MCW_MLP_HIDDEN * MCW_MLP_HIDDEN * 2 + MCW_MLP_HIDDEN * 16 * 2)

/* Repack the bf16 weights w1 [256, 4], w2, w3 [256, 256] and w4 [649, 256] (row-major
 * [out, in]) into blob (MCW_MLP_PACK_BYTES, 16-byte aligned), the tensor-core operand
 * layout read by mcw_mlp_forward.  Call again whenever the weights change. */
int mcw_mlp_pack(const void *w1, const void *w2, const void *w3, const void *w4, void *blob, void *stream);

/* y [m, 649] (f32; y 16-byte aligned, leading dimension ldy >= 652 and a multiple of 4;
 * columns 649 .. ldy - 1 are left untouched) = network(x [m, 4] f32) from the packed
 * weights and the f32 biases: one kernel, the hidden activations never leave shared
 * memory.  Inputs and activations are rounded to bf16 as the layer-by-layer
 * mcw_mlp_gemm path rounds them.  A wait that runs out sets bit 1 of mcw_mlp_status. */
int mcw_mlp_forward(const float *x, int32_t m, const float *b1, const float *b2, const float *b3,
                    const float *b4, const void *blob, float *y, int32_t ldy, void *stream);

/* The same with y rounded to fp16 (11-bit significand, below the bf16 rounding of the
 * activations): y 16-byte aligned, ldy >= 656 halves and a multiple of 8.  Half the
 * bytes of the output stream. */
int mcw_mlp_forward_f16(const float *x, int32_t m, const float *b1, const float *b2, const float *b3,
                        const float *b4, const void *blob, void *y, int32_t ldy, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* MCW_MLP_H */
