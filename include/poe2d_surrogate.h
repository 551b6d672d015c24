/*
 * poe2d_surrogate.h -- C ABI of the learned surrogate: a small network that
 * maps a downsampled porosity / gas-saturation map of a patchy model plus
 * its source and grid parameters to the receiver gather the solver would
 * record.  No reference counterpart: thejatmik/poe2d has no learned part.
 *
 * Network (about 2.4 M parameters; bf16 weights and activations, FP32
 * accumulation on the tensor cores, FP32 master weights and Adam state):
 *   input   map [B, 64, 64, 2] (channels last: porosity, gas fraction) and
 *           scalars [B, 3]
 *   encoder four 3x3 stride-2 convolutions with ReLU: 2 -> 64 -> 128 -> 128
 *           -> 256 channels, 64x64 -> 4x4
 *   latent  [4*4*256 | scalars] -> 256 -> 2048 (= 16 samples x 128 channels),
 *           fully connected with ReLU
 *   decoder six nearest x2 upsampling + k=3 convolutions with ReLU:
 *           128 -> 128 -> 128 -> 128 -> 64 -> 64 -> 64 channels, 16 -> 1024
 *           samples, then a k=3 convolution to 384 channels (128 receivers x
 *           vx, vz, p) without activation
 *   output  gather [B, 1024, 384] FP32, time-major; channel c means what it
 *           means in the training targets (the data generator stores
 *           c = 128 * component + receiver, components vx, vz, p)
 * Loss: mean squared error against bf16 targets of the same layout.
 *
 * All tensors passed to these calls are DEVICE pointers on the context's
 * device; parameters move through host arrays.  Training batches must be a
 * multiple of 8; inference batches up to max_batch.
 */
#ifndef POE2D_SURROGATE_H
#define POE2D_SURROGATE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct poe_sg poe_sg;

enum { POE_SG_MAP = 64, POE_SG_MAP_CH = 2, POE_SG_SCALARS = 3, POE_SG_SAMPLES = 1024, POE_SG_CHANNELS = 384 };

/* Network with He-normal weights drawn from seed, buffers for batches up to
 * max_batch, on the current device; stream: a cudaStream_t or NULL (private). */
int poe_sg_create(int32_t max_batch, uint64_t seed, void *stream, poe_sg **out);

/* Trainable parameters (count) and the length of the flat parameter array
 * used by get/set_params and get_grads: per layer, the weights [Cout][K]
 * then the biases [Cout], layers in network order. */
int poe_sg_param_count(const poe_sg *net, int64_t *count);
int poe_sg_get_params(poe_sg *net, float *host, int64_t n);
int poe_sg_set_params(poe_sg *net, const float *host, int64_t n);   /* resets Adam state */
int poe_sg_get_grads(poe_sg *net, float *host, int64_t n);

/* Inference: out [B, 1024, 384] FP32 (device, 16-byte aligned; NULL: the
 * network's own buffer). */
int poe_sg_forward(poe_sg *net, const void *maps_bf16, const float *scalars, int32_t B, float *out);

/* Forward, loss and backward: gradients stay in the network; *loss_out (host)
 * receives the mean squared error. */
int poe_sg_loss_grad(poe_sg *net, const void *maps_bf16, const float *scalars, const void *targets_bf16,
                     int32_t B, float *loss_out);

/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) with the current gradients. */
int poe_sg_adam(poe_sg *net, float lr);

/* The optimiser state, for inspection and training checkpoints, in the
 * layout of get_params (each pointer may be NULL): Adam's first and second
 * moments m and v, the bf16 weight copy the forward pass reads (widened to
 * FP32, exactly), and the number of Adam steps taken since the parameters
 * were last set. */
int poe_sg_get_state(poe_sg *net, float *m, float *v, float *w16_f32, int64_t n, int32_t *step);

/* loss_grad + adam. */
int poe_sg_train_step(poe_sg *net, const void *maps_bf16, const float *scalars, const void *targets_bf16,
                      int32_t B, float lr, float *loss_out);

/* Kernel launches issued by this network since creation. */
int poe_sg_launches(const poe_sg *net, int64_t *count);
const char *poe_sg_last_error(const poe_sg *net);
void poe_sg_destroy(poe_sg *net);

/* The GEMM on its own: C = alpha A . B^T (+ bias[n]) (ReLU) (+= C), A: M x K,
 * B: N x K, bf16 with K contiguous (pitches lda, ldb multiples of 8); outputs
 * FP32 and/or bf16 with pitch ldc.  ws (may be NULL) of ws_floats >= 16 M ldc
 * lets long-K products split K across CTAs.  err_dev: device int set to 1 if
 * a bounded wait gave up.  All pointers device pointers. */
int poe_sg_gemm(const void *A, int32_t lda, const void *B, int32_t ldb, int32_t M, int32_t N, int32_t K,
                float alpha, const float *bias, int32_t relu, float *out_f32, void *out_bf16, int32_t ldc,
                int32_t accumulate, float *ws, int64_t ws_floats, int32_t *err_dev, void *stream);

/* Batch assembly for training: dst row r = src row idx[r] for r < n, rows of
 * row_bytes bytes (a multiple of 4; src and dst 4-byte aligned); idx holds
 * n int64 row indices, each below the caller's row count.  All pointers
 * device pointers; runs on `stream`. */
int poe_sg_gather_rows(const void *src, int64_t row_bytes, const int64_t *idx, int32_t n, void *dst,
                       void *stream);

#ifdef __cplusplus
}
#endif
#endif
