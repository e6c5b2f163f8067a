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
 * mcw_mlp_forward; bit 2: the same in mcw_mlp_gemm_grouped); clear != 0 resets them. */
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

/* The biases of one network, b1 | b2 | b3 | b4, as one f32 row. */
#define MCW_MLP_BIAS_FLOATS (3 * MCW_MLP_HIDDEN + MCW_MLP_OUT)

/* mcw_mlp_forward_f16 of `members` networks (an ensemble) on the same inputs, in one
 * launch: member e's biases at bias + e * MCW_MLP_BIAS_FLOATS, its packed weights at
 * blob + e * MCW_MLP_PACK_BYTES, its outputs at y + e * m * ldy halves (ldy as
 * mcw_mlp_forward_f16).  Each member's outputs equal those of mcw_mlp_forward_f16 bit
 * for bit.  No reference counterpart (the ensemble's spread judges the surrogate). */
int mcw_mlp_forward_ensemble_f16(const float *x, int32_t m, int32_t members, const float *bias, const void *blob,
                                 void *y, int32_t ldy, void *stream);

/* ---- training engine: one Adam step of an ensemble in a fixed sequence of launches.
 * "groups" are independent problems of the same shape (ensemble members) whose
 * operands lie stride_* elements apart; strides and leading dimensions count
 * elements. */

/* C[g] = A[g] B[g]^T for g < groups on the tcgen05 tensor cores, A bf16 [m, k] and B
 * bf16 [n, k] both K-major (rows lda / ldb apart), operand tiles staged by TMA.
 * Rules of the copies: a and b 16-byte aligned, lda, ldb, stride_a and stride_b
 * multiples of 8 with stride >= ld * rows; rows past m / n and columns past k read as
 * zero.  Epilogues as mcw_mlp_gemm (bias and aux per group: bias + g * stride_bias,
 * aux + g * stride_aux + i * ldaux), and for MCW_EPI_BIAS_SILU / MCW_EPI_DSILU an
 * optional bf16 transposed copy of the bf16 output, ct [n, m] with leading dimension
 * ldct.  splits > 1 (MCW_EPI_F32 only): K is cut into `splits` whole-64 ranges and
 * range s writes its partial product at c + s * stride_split (mcw_mlp_reduce_splits
 * adds them); splits must equal ceil(c / ceil(c / splits)) for c = ceil(k / 64). */
typedef struct {
    int32_t m, n, k;
    int32_t groups;
    int32_t splits;
    int32_t epilogue;
    const void *a;
    int64_t lda, stride_a;
    const void *b;
    int64_t ldb, stride_b;
    const float *bias;
    int64_t stride_bias;
    const float *aux;
    int64_t ldaux, stride_aux;
    void *c;
    int64_t ldc, stride_c, stride_split;
    void *c2;
    int64_t ldc2, stride_c2;
    void *ct;
    int64_t ldct, stride_ct;
} McwGemmGrouped;

int mcw_mlp_gemm_grouped(const McwGemmGrouped *p, void *stream);

/* dst[g][i][j] = sum over s < splits of src[s * stride_split + g * stride_src + i * ld_src + j]. */
int mcw_mlp_reduce_splits(const float *src, int64_t stride_split, int64_t stride_src, int64_t ld_src, float *dst,
                          int64_t stride_dst, int64_t ld_dst, int32_t splits, int32_t groups, int32_t m, int32_t n,
                          void *stream);

/* mcw_mlp_loss for `groups` outputs y[g] against t[g] (loss[g] += ...), the gradient as
 * f32 g32 and bf16 g16 [m, n] (leading dimension ldg) and bf16 transposed g16t [n, m]
 * (leading dimension ldgt). */
int mcw_mlp_loss_grouped(const float *y, int64_t ldy, int64_t stride_y, const float *t, int64_t ldt,
                         int64_t stride_t, const float *w, int32_t groups, int32_t m, int32_t n, float *g32,
                         int64_t ldg, int64_t stride_g32, void *g16, int64_t stride_g16, void *g16t, int64_t ldgt,
                         int64_t stride_g16t, float *loss, void *stream);

/* Column sums of up to four gradient matrices (bias gradients):
 * out[g * stride_out + out_offset + j] = sum over i < m of g[g * stride + i * ld + j], j < n.
 * With partial (n_layers * groups * ceil(m / rows_per_chunk) * max n floats) and
 * 0 < rows_per_chunk < m, the rows are summed in chunks in parallel and the chunks'
 * sums added in order (the result does not depend on the launch either way). */
typedef struct {
    const float *g;
    int64_t ld, stride;
    int64_t out_offset;
    int32_t n;
    int32_t pad;
} McwColsumLayer;

int mcw_mlp_colsum_grouped(const McwColsumLayer *layers, int32_t n_layers, int32_t groups, int32_t m, float *out,
                           int64_t stride_out, float *partial, int32_t rows_per_chunk, void *stream);

/* A block of the flat parameters whose bf16 copy is also kept transposed:
 * wt[offset_t + c * ld_t + o] = w[offset + o * cols + c] for o < rows, c < cols. */
typedef struct {
    int64_t offset, offset_t, ld_t;
    int32_t rows, cols;
} McwTransposeBlock;

/* mcw_mlp_adam over `groups` flat parameter vectors of n elements (w, g, m, v and the
 * bf16 copy w16 each g * n apart), the learning rate and the 1-based step read from
 * device memory (lr_dev, step_dev); wt (stride_t per group) receives the transposed
 * bf16 copies of up to four blocks. */
int mcw_mlp_adam_grouped(float *w, const float *g, float *m, float *v, void *w16, int64_t n, int32_t groups,
                         const float *lr_dev, const int32_t *step_dev, float beta1, float beta2, float eps,
                         void *wt, int64_t stride_t, const McwTransposeBlock *blocks, int32_t n_blocks,
                         void *stream);

/* The batch of a step: for g < groups and i < batch, row r = perm[g * n_rows + c * batch + i]
 * (c = *counter_dev) of x_all (bf16 [n_rows, 16]) and t_all (f32, leading dimension
 * ldt_all, n_out columns) into x (bf16 [batch, 16]), xt (bf16 [16, batch]) and t
 * (leading dimension ldt).  Rows past n_rows are skipped. */
int mcw_mlp_gather(const void *x_all, const float *t_all, int64_t ldt_all, int32_t n_out, const int32_t *perm,
                   int64_t n_rows, const int32_t *counter_dev, int32_t batch, int32_t groups, void *x,
                   int64_t stride_x, void *xt, int64_t stride_xt, float *t, int64_t ldt, int64_t stride_t,
                   void *stream);

/* *counter_dev += 1 and *step_dev += 1 (the end of a captured step). */
int mcw_mlp_advance(int32_t *counter_dev, int32_t *step_dev, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* MCW_MLP_H */
