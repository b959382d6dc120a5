/*
 * c2a_mlp.h -- the learned seeding's network kernels (C ABI, device pointers).
 *
 * The network proposes leaf-cluster pairs whose exact distances tighten the
 * first upper bound of the CANONICAL closest-pair search: it changes how
 * much the search prunes, never a result.  It is a BF16 multilayer
 * perceptron with FP32 accumulation,
 *
 *     x (50: relative pose 12, relative velocity 6, two 16-float mesh
 *        embeddings) -> 256 -> 256 -> 256 -> 4096 logits (64 x 64 cluster pairs),
 *
 * GELU after each hidden layer, trained with softmax cross-entropy and Adam.
 * The same network, trained on 64 log-cost buckets, orders REFERENCE batches
 * so that the costliest queries start first (c2a_solve_batch_ordered).
 * These entry points are the building blocks (tensor-core GEMM with fused
 * epilogues, the loss, the optimizer step, top-k); c2a_gb300/learned.py
 * composes them into training and inference.
 *
 * Conventions: bf16 arrays are uint16_t (IEEE bfloat16 bits); matrices are
 * row-major; every call is asynchronous on `stream` (a cudaStream_t, NULL:
 * the default stream) and returns C2A_ERR_INVALID_ARGUMENT for shapes the
 * kernels do not take.
 */
#ifndef C2A_MLP_H
#define C2A_MLP_H

#include <stdint.h>

#include "c2a_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* GEMM epilogue flags */
#define C2A_MLP_BIAS 1 /* add bias[n] */
#define C2A_MLP_GELU 2 /* out_bf16 = GELU(acc (+ bias)); out_f32 keeps the pre-activation */

/* out[m][n] = sum_k A[m][k] * B[n][k] (+ bias[n]), A: M x K, B: N x K (both
 * bf16, K contiguous), FP32 accumulation on the tensor cores.  out_f32 (M x N
 * floats) and out_bf16 (M x N bf16, GELU applied when flagged) may each be
 * NULL.  M, N multiples of 128, K a multiple of 32. */
c2a_status c2a_mlp_gemm(const uint16_t *A, const uint16_t *B, const float *bias, int32_t M, int32_t N, int32_t K,
                        int32_t flags, float *out_f32, uint16_t *out_bf16, void *stream);

/* Synchronises the stream and reports whether any GEMM since the last check
 * ran out of a bounded wait (C2A_ERR_CUDA; its output is then undefined);
 * clears the record. */
c2a_status c2a_mlp_check(void *stream);

/* out (cols x rows) = in (rows x cols) transposed, bf16; rows, cols multiples of 32 */
c2a_status c2a_mlp_transpose(const uint16_t *in, int32_t rows, int32_t cols, uint16_t *out, void *stream);

/* d_pre (bf16, M x N) = d_act (FP32, M x N) * GELU'(pre) (FP32, M x N) */
c2a_status c2a_mlp_gelu_backward(const float *d_act, const float *pre, int64_t count, uint16_t *d_pre,
                                 void *stream);

/* softmax cross-entropy over N logits per row: loss[m] (FP32) and
 * d_logits = (softmax - onehot(label)) * scale as bf16; labels < 0 are
 * ignored rows (zero loss and gradient) */
c2a_status c2a_mlp_softmax_xent(const float *logits, const int32_t *labels, int32_t M, int32_t N, float scale,
                                float *loss, uint16_t *d_logits, void *stream);

/* out[m] = sum_n softmax(logits[m])[n] * n: the expected class index of each row */
c2a_status c2a_mlp_expect(const float *logits, int32_t M, int32_t N, float *out, void *stream);

/* out[n] = sum_m in[m][n] (FP32; in is bf16, M x N) */
c2a_status c2a_mlp_colsum(const uint16_t *in, int32_t M, int32_t N, float *out, void *stream);

/* Adam on count FP32 parameters (step t >= 1): updates w, m, v from the
 * gradient g; writes the bf16 copy (w_bf16, may be NULL) and, for a rows x
 * cols matrix, its transposed bf16 copy (w_bf16_t, may be NULL) */
c2a_status c2a_mlp_adam(float *w, float *m, float *v, const float *g, int64_t count, float lr, float beta1,
                        float beta2, float eps, int32_t t, uint16_t *w_bf16, uint16_t *w_bf16_t, int32_t rows,
                        int32_t cols, void *stream);

/* the input rows: x[m] = [feat[m] (18 floats), emb[ia[m]] (16), emb[ib[m]] (16), 0 ...] as bf16, width K
 * (>= 50, a multiple of 32); rows m >= n_valid are zero */
c2a_status c2a_mlp_assemble(const float *feat, const int32_t *ia, const int32_t *ib, const float *emb,
                            int32_t n_valid, int32_t M, int32_t K, uint16_t *x, void *stream);

/* the embedding gradient: g_emb[ia[m]] += dx[m][18:34], g_emb[ib[m]] += dx[m][34:50] (dx FP32, width K) */
c2a_status c2a_mlp_embed_backward(const float *dx, const int32_t *ia, const int32_t *ib, int32_t n_valid,
                                  int32_t K, float *g_emb, void *stream);

/* the k (<= 16) largest of N logits per row, in decreasing order (ties: lower index first) */
c2a_status c2a_mlp_topk(const float *logits, int32_t M, int32_t N, int32_t k, int32_t *index, void *stream);

/* The schedule from expected costs: order[0..n) = the indices 0..n-1 by
 * decreasing key, key in [0, key_max] quantised to C2A_ORDER_BINS levels,
 * ties (same level) in increasing index (a stable, deterministic counting
 * sort: histogram per 1024-key chunk, one scan, a ranked scatter).  scratch:
 * C2A_ORDER_SCRATCH(n) int32 of device memory. */
#define C2A_ORDER_BINS 1024
#define C2A_ORDER_SCRATCH(n) ((int64_t)(((n) + 1023) / 1024) * C2A_ORDER_BINS)
c2a_status c2a_mlp_order_desc(const float *key, int32_t n, float key_max, int32_t *order, int32_t *scratch,
                              void *stream);

#ifdef __cplusplus
}
#endif

#endif
