// sg_internal.h -- device-side interfaces of the surrogate network kernels.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace sg {

constexpr int kMaxSplits = 16;

// C = alpha * A . B^T: A is M x K (pitch lda), B is N x K (pitch ldb), bf16, K contiguous
struct Gemm {
    const __nv_bfloat16 *A;
    int lda;
    const __nv_bfloat16 *B;
    int ldb;
    int M, N, K;
};

struct Epilogue {
    float alpha = 1.0f;
    const float *bias = nullptr;          // [N]
    int relu = 0;
    float *out_f32 = nullptr;             // [M x ldc]
    __nv_bfloat16 *out_bf16 = nullptr;    // [M x ldc]
    int ldc = 0;
    int accumulate = 0;                   // out_f32 += result
};

// Launch on st; ws (may be null: no split-K) holds kMaxSplits * M * ldc floats.
// Returns a cudaError_t value.  A bounded wait that gave up sets *err = 1.
int gemm(const Gemm &g, const Epilogue &e, float *ws, int64_t ws_floats, int *err, cudaStream_t st);

// One output phase of a k = 3 convolution over time of x [B, T, cin] (dense
// rows, channels last) upsampled `up` times (1 or 2, nearest), without an
// im2col matrix: out[b, up*s + phase, :] = sum over taps k of
// W[:, k*cin .. k*cin+cin) . xu[b, up*s + phase + k - 1, :] for s < T, xu the
// upsampled input (zero outside [0, up*T)).  The GEMM's producer loads each
// tap's rows of x directly (a row offset per tap and phase), so the result
// equals the GEMM over im2col1d's matrix bit for bit.  W is cout x 3*cin
// (K-major); cin a multiple of 64, T a power of two; e: a plain output (no
// accumulation), FP32 or bf16, ldc a multiple of 16 bytes.
int gemm_conv1d(const __nv_bfloat16 *x, int B, int T, int cin, int up, int phase, const __nv_bfloat16 *W, int cout,
                const Epilogue &e, int *err, cudaStream_t st);

}  // namespace sg
