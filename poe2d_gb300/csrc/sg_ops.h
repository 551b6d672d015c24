// sg_ops.h -- non-GEMM kernels of the surrogate network (sg_ops.cu).
// Every function launches on st and returns a cudaError_t value.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace sg {

constexpr int kMseBlocks = 512;          // partial sums of the loss
constexpr int kColChunkRows = 1024;      // rows per partial column sum

// conv 3x3 / stride 2 / pad 1 over NHWC x [B, H, W, C] -> col [B*H/2*W/2, ld], ld >= 9C
int im2col2d(const __nv_bfloat16 *x, int B, int H, int W, int C, __nv_bfloat16 *col, int ld, cudaStream_t st);
int col2im2d(const __nv_bfloat16 *dcol, int ld, int B, int H, int W, int C, __nv_bfloat16 *dx, cudaStream_t st);
// conv1d k=3 / pad 1 over x [B, T, C] repeated `up` times in time -> col [B*T*up, ld], ld >= 3C
int im2col1d(const __nv_bfloat16 *x, int B, int T, int C, int up, __nv_bfloat16 *col, int ld, cudaStream_t st);
int col2im1d(const __nv_bfloat16 *dcol, int ld, int B, int T, int C, int up, __nv_bfloat16 *dx, cudaStream_t st);
int relu_bwd(const __nv_bfloat16 *dy, int ldy, const __nv_bfloat16 *y, int64_t rows, int cols, __nv_bfloat16 *dz,
             cudaStream_t st);
// db[n] = sum_r dz[r, n]; partial holds ceil(rows / kColChunkRows) * cols floats
int colsum(const __nv_bfloat16 *dz, int64_t rows, int cols, int ld, float *db, float *partial, cudaStream_t st);
int transpose(const __nv_bfloat16 *in, int64_t R, int C, int ldi, __nv_bfloat16 *out, int64_t ldo, cudaStream_t st);
// loss_sum = sum (out - tgt)^2; dout = grad_scale * (out - tgt) (dout may be null); partial: kMseBlocks floats
int mse(const float *out, const __nv_bfloat16 *tgt, int64_t n, float grad_scale, __nv_bfloat16 *dout, float *partial,
        float *loss_sum, cudaStream_t st);
int adam(float *w, const float *g, float *m, float *v, int64_t n, float lr_t, float b1, float b2, float eps_t,
         __nv_bfloat16 *w16, cudaStream_t st);
int to_bf16(const float *x, int64_t n, __nv_bfloat16 *y, cudaStream_t st);
int concat(const __nv_bfloat16 *src, int ns, const float *extra, int ne, int B, __nv_bfloat16 *dst, int ldd,
           cudaStream_t st);
// dst row r = src row idx[r] for r < n (rows of row_bytes, a multiple of 4)
int gather_rows(const void *src, int64_t row_bytes, const int64_t *idx, int n, void *dst, cudaStream_t st);

}  // namespace sg
