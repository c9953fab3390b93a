/*
 * libglgpu, learned CG warm start: the kernels of a small convolutional
 * encoder-decoder that predicts a near-minimum (psi, A) from (material mask, H,
 * 1/kappa, initial psi), used as a starting point for the CG.  No counterpart in
 * the reference, whose only minimiser is the CG of svirl/solvers/cg.py.
 *
 * Conventions
 *  - Activations and their gradients: NHWC, bfloat16 (uint16 storage), channel
 *    counts multiples of 8.  Weights of a 3x3 convolution: float32 master copy
 *    W[cout][3][3][cin]; the kernels read bfloat16 copies made by
 *    glnn_prep_weights (Wb: same layout, Wt: [3][3][cin][cout]).  Weight and
 *    bias gradients, optimiser state: float32.  Products are accumulated in
 *    float32 on the tensor cores (tcgen05; the weight gradient of shapes the
 *    tcgen05 kernel does not take runs on mma).
 *  - "Same" padding (zeros), stride 1.  A convolution may read the channel
 *    concatenation [x1 | x2] of two tensors (x2 may be NULL with c2 = 0), so the
 *    decoder's skip connections need no copy; the data gradient is written split
 *    the same way.
 *  - relu = 1: y = max(0, conv + b); the backward kernels then take y and apply
 *    the ReLU derivative (y > 0) to dy on the fly.
 *  - Every call enqueues work on `stream` (a cudaStream_t, NULL = default
 *    stream) and returns GLGPU_OK (0), GLGPU_E_ARG or GLGPU_E_CUDA (glgpu.h).
 */
#ifndef GLGPU_NN_H
#define GLGPU_NN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* y = conv3x3([x1|x2], Wb) + b (+ ReLU).  y: n*h*w*cout.  Runs on the
 * 5th-generation tensor cores (tcgen05.mma, FP32 accumulator in tensor memory,
 * 128 x 64 output tile per CTA).  *err (a device int) is set to 1 if a CTA's
 * bounded wait for its MMAs ran out (that CTA's outputs are then not written). */
int glnn_conv3x3_fwd(const void* x1, int32_t c1, const void* x2, int32_t c2, const void* wb, const float* bias,
                     void* y, int32_t n, int32_t h, int32_t w, int32_t cout, int32_t relu, int32_t* err, void* stream);

/* Operand loads of glnn_conv3x3_fwd (and of glnn_conv3x3_bwd_data with relu = 0):
 * 2 (default) = by TMA (cp.async.bulk.tensor from 4-D / 2-D / 3-D tensor maps) in a
 * persistent kernel (CTAs loop over output tiles, two tensor-memory accumulators,
 * the epilogue of one tile under the MMAs of the next); 1 = by TMA, one output tile
 * per CTA; both for the shapes they take (c1, c2, cout multiples of 64; w a multiple
 * of 128 or a divisor of 128; h*w a multiple of 128), the thread gather otherwise;
 * 0 = always the thread gather.  Every setting computes the same values bitwise.
 * Nonzero also selects the tcgen05 weight gradient (0: the mma.sync one).
 * Process-wide. */
int glnn_set_conv_tma(int32_t enable);
/* [dx1|dx2] = conv3x3^T(dy * relu'(y), Wt), on tcgen05 like the forward.  y may be
 * NULL when relu = 0.  With relu = 0 and the shapes of the TMA forward (roles of
 * input and output channels exchanged) the operands are loaded by TMA (dy as the
 * 4-D activation tensor, Wt as the 3-D tensor [9][cin][cout]); else the threads
 * gather them (and apply the ReLU derivative).  Callers that have both gradients
 * to compute mask dy once with glnn_relu_mask and pass relu = 0. */
int glnn_relu_mask(const void* dy, const void* y, void* out, int64_t count, void* stream); /* out = dy * (y > 0), bf16, count % 8 == 0 */
int glnn_conv3x3_bwd_data(const void* dy, const void* y, int32_t relu, const void* wt, void* dx1, int32_t c1,
                          void* dx2, int32_t c2, int32_t n, int32_t h, int32_t w, int32_t cout, int32_t* err,
                          void* stream);

/* dW[cout][9*cin] and db[cout] (float32, overwritten) from dy * relu'(y) and
 * the input [x1|x2].  work: float32 scratch of glnn_conv3x3_bwd_weight_work()
 * floats, 16-byte aligned (split-K partial sums, reduced in a fixed order:
 * deterministic).  With glnn_set_conv_tma(1) and c1, c2, cout multiples of 64,
 * w a multiple or a divisor of 64 and h*w a multiple of 64, it runs on tcgen05
 * (M = two taps x 64 input channels, N = 64 output channels, K = pixels, both
 * operands MN-major boxes loaded by TMA, FP32 accumulator in tensor memory); else
 * on mma.sync.  *err (a device int) is set to 1 if a CTA's bounded wait ran out
 * (its partial sums are then NaN). */
int64_t glnn_conv3x3_bwd_weight_work(int32_t n, int32_t h, int32_t w, int32_t cin, int32_t cout);
int glnn_conv3x3_bwd_weight(const void* dy, const void* y, int32_t relu, const void* x1, int32_t c1, const void* x2,
                            int32_t c2, float* dw, float* db, float* work, int64_t work_floats, int32_t n, int32_t h,
                            int32_t w, int32_t cout, int32_t* err, void* stream);

/* bfloat16 copies of a float32 weight W[cout][9][cin]: wb (same layout) and
 * wt[9][cin][cout] (for the data gradient); either may be NULL. */
int glnn_prep_weights(const float* w, void* wb, void* wt, int32_t cout, int32_t cin, void* stream);

/* 2x2 average pooling (h, w even) and nearest 2x upsampling, with their
 * gradients; h, w are the dimensions of the larger tensor. */
int glnn_pool2_fwd(const void* x, void* y, int32_t n, int32_t h, int32_t w, int32_t c, void* stream);
int glnn_pool2_bwd(const void* dy, void* dx, int32_t n, int32_t h, int32_t w, int32_t c, void* stream);
int glnn_up2_fwd(const void* x, void* y, int32_t n, int32_t h, int32_t w, int32_t c, void* stream);
int glnn_up2_bwd(const void* dy, void* dx, int32_t n, int32_t h, int32_t w, int32_t c, void* stream);

/* out = a + b (bfloat16, count elements). */
int glnn_add(const void* a, const void* b, void* out, int64_t count, void* stream);

/* Weighted squared error of the first ct channels of pred (npix x cp, bf16)
 * against target (npix x ct, float32) with per-channel weights cw[ct]:
 * loss = sum cw[c] (pred - target)^2 / npix, dpred = its gradient (bf16, the
 * other cp - ct channels zero).  loss: one float written on the device; work:
 * float32 scratch of at least 1024 floats. */
int glnn_mse(const void* pred, int32_t cp, const float* target, int32_t ct, const float* cw, void* dpred, float* loss,
             float* work, int64_t npix, void* stream);

/* Adam (with decoupled weight decay) on float32 parameters; step counts from 1. */
int glnn_adam(float* w, const float* g, float* m, float* v, int64_t count, float lr, float beta1, float beta2,
              float eps, float weight_decay, int32_t step, void* stream);

/* float32 <-> bfloat16 conversion of count elements. */
int glnn_f32_to_bf16(const float* x, void* y, int64_t count, void* stream);
int glnn_bf16_to_f32(const void* x, float* y, int64_t count, void* stream);

#ifdef __cplusplus
}
#endif

#endif
