// sg_ops.cu -- the surrogate network's non-GEMM kernels: im2col / col2im for
// the 2-D encoder convolutions and the 1-D (optionally upsampling) decoder
// convolutions, ReLU backward, bias gradients, transposes, the MSE loss and
// its gradient, Adam.  Everything is channels-last; bf16 activations, FP32
// gradients of parameters, FP32 optimizer state.  Reductions run in a fixed
// order so training is deterministic.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "sg_ops.h"

namespace sg {
namespace {

__device__ __forceinline__ float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ __nv_bfloat16 tobf(float v) { return __float2bfloat16_rn(v); }

int grid_for(int64_t n, int block)
{
    int64_t g = (n + block - 1) / block;
    if (g > 65535LL * 16) g = 65535LL * 16;
    return (int)(g < 1 ? 1 : g);
}

// Index arithmetic is 32-bit (every tensor here has fewer than 2^31 elements,
// checked by the launchers) and the channel-vectorised kernels move 8 bf16
// (16 bytes) per thread: channel counts that are multiples of 8 keep a group
// of 8 consecutive columns inside one tap and one source pixel.

__device__ __forceinline__ void add8(float (&acc)[8], const uint4 v)
{
    const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&v);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float2 f = __bfloat1622float2(h[i]);
        acc[2 * i] += f.x;
        acc[2 * i + 1] += f.y;
    }
}

__device__ __forceinline__ uint4 pack8(const float (&acc)[8])
{
    uint4 v;
    __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&v);
#pragma unroll
    for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(acc[2 * i], acc[2 * i + 1]);
    return v;
}

// conv 3x3, stride 2, pad 1: col[(b, oy, ox), (ky*3 + kx)*C + c], zero past 9C up to ld
__global__ void k_im2col2d(const __nv_bfloat16 *x, int B, int H, int W, int C, __nv_bfloat16 *col, int ld)
{
    const int Ho = H / 2, Wo = W / 2;
    const int total = B * Ho * Wo * ld;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int k = i % ld, r = i / ld;
        float v = 0.0f;
        if (k < 9 * C) {
            const int tap = k / C, c = k - tap * C;
            const int ky = tap / 3, kx = tap - ky * 3;
            const int ox = r % Wo, oy = (r / Wo) % Ho, b = r / (Wo * Ho);
            const int y = 2 * oy - 1 + ky, xx = 2 * ox - 1 + kx;
            if (y >= 0 && y < H && xx >= 0 && xx < W) v = bf(x[((b * H + y) * W + xx) * C + c]);
        }
        col[i] = tobf(v);
    }
}

// the same for C % 8 == 0, 8 columns per thread
__global__ void k_im2col2d_v8(const __nv_bfloat16 *x, int B, int H, int W, int C, __nv_bfloat16 *col, int ld)
{
    const int Ho = H / 2, Wo = W / 2, U = ld / 8;
    const int total = B * Ho * Wo * U;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int u = i % U, r = i / U;
        const int k = 8 * u;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (k < 9 * C) {
            const int tap = k / C, c = k - tap * C;
            const int ky = tap / 3, kx = tap - ky * 3;
            const int ox = r % Wo, oy = (r / Wo) % Ho, b = r / (Wo * Ho);
            const int y = 2 * oy - 1 + ky, xx = 2 * ox - 1 + kx;
            if (y >= 0 && y < H && xx >= 0 && xx < W)
                v = *reinterpret_cast<const uint4 *>(x + ((b * H + y) * W + xx) * C + c);
        }
        *reinterpret_cast<uint4 *>(col + r * ld + k) = v;
    }
}

// gradient of the im2col above: dx[b, y, x, c0..c0+7] = sum of the col entries that copied
// it (C % 8 == 0)
__global__ void k_col2im2d_v8(const __nv_bfloat16 *dcol, int ld, int B, int H, int W, int C, __nv_bfloat16 *dx)
{
    const int Ho = H / 2, Wo = W / 2, U = C / 8;
    const int total = B * H * W * U;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int c = 8 * (i % U), p = i / U;
        const int xx = p % W, y = (p / W) % H, b = p / (W * H);
        float acc[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        for (int ky = 0; ky < 3; ++ky) {
            const int ty = y + 1 - ky;
            if (ty < 0 || (ty & 1) || ty / 2 >= Ho) continue;
            for (int kx = 0; kx < 3; ++kx) {
                const int tx = xx + 1 - kx;
                if (tx < 0 || (tx & 1) || tx / 2 >= Wo) continue;
                const int r = (b * Ho + ty / 2) * Wo + tx / 2;
                add8(acc, *reinterpret_cast<const uint4 *>(dcol + r * ld + (ky * 3 + kx) * C + c));
            }
        }
        *reinterpret_cast<uint4 *>(dx + p * C + c) = pack8(acc);
    }
}

// conv1d k=3, pad 1, over x repeated `up` times in time:
// col[(b, t), tap*C + c] = u[b, t + tap - 1, c], u[t] = x[t / up], To = T * up (C % 8 == 0)
__global__ void k_im2col1d_v8(const __nv_bfloat16 *x, int B, int T, int C, int up, __nv_bfloat16 *col, int ld)
{
    const int To = T * up, U = ld / 8;
    const int total = B * To * U;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int u = i % U, r = i / U;
        const int k = 8 * u;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (k < 3 * C) {
            const int tap = k / C, c = k - tap * C;
            const int t = r % To, b = r / To;
            const int s = t + tap - 1;
            if (s >= 0 && s < To) v = *reinterpret_cast<const uint4 *>(x + (b * T + s / up) * C + c);
        }
        *reinterpret_cast<uint4 *>(col + r * ld + k) = v;
    }
}

__global__ void k_col2im1d_v8(const __nv_bfloat16 *dcol, int ld, int B, int T, int C, int up, __nv_bfloat16 *dx)
{
    const int To = T * up, U = C / 8;
    const int total = B * T * U;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int c = 8 * (i % U), p = i / U;
        const int t = p % T, b = p / T;
        float acc[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        for (int q = 0; q < up; ++q) {
            const int su = t * up + q;                    // a time of the upsampled input
            for (int tap = 0; tap < 3; ++tap) {
                const int to = su - tap + 1;              // output time that read su through this tap
                if (to < 0 || to >= To) continue;
                add8(acc, *reinterpret_cast<const uint4 *>(dcol + (b * To + to) * ld + tap * C + c));
            }
        }
        *reinterpret_cast<uint4 *>(dx + p * C + c) = pack8(acc);
    }
}

// dz = dy * (y > 0); dy rows have pitch ldy, y and dz are dense rows x cols
// (cols and ldy multiples of 8: 8 elements per thread)
__global__ void k_relu_bwd_v8(const __nv_bfloat16 *dy, int ldy, const __nv_bfloat16 *y, int rows, int cols,
                              __nv_bfloat16 *dz)
{
    const int U = cols / 8, total = rows * U;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int r = i / U, c = 8 * (i - r * U);
        const uint4 g = *reinterpret_cast<const uint4 *>(dy + r * ldy + c);
        const uint4 a = *reinterpret_cast<const uint4 *>(y + r * cols + c);
        const __nv_bfloat16 *gh = reinterpret_cast<const __nv_bfloat16 *>(&g);
        const __nv_bfloat16 *ah = reinterpret_cast<const __nv_bfloat16 *>(&a);
        uint4 o;
        __nv_bfloat16 *oh = reinterpret_cast<__nv_bfloat16 *>(&o);
#pragma unroll
        for (int j = 0; j < 8; ++j) oh[j] = bf(ah[j]) > 0.0f ? gh[j] : tobf(0.0f);
        *reinterpret_cast<uint4 *>(dz + r * cols + c) = o;
    }
}

// column sums of dz in two fixed-order passes: partial[chunk][n] over
// kColChunkRows rows each, then the chunks in order
__global__ void k_colsum_part(const __nv_bfloat16 *dz, int64_t rows, int cols, int ld, float *partial)
{
    __shared__ float part[8][33];
    const int c = blockIdx.x * 32 + threadIdx.x;
    const int64_t r0 = (int64_t)blockIdx.y * kColChunkRows;
    int64_t r1 = r0 + kColChunkRows;
    if (r1 > rows) r1 = rows;
    float s = 0.0f;
    if (c < cols)
        for (int64_t r = r0 + threadIdx.y; r < r1; r += 8) s += bf(dz[r * ld + c]);
    part[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.y == 0 && c < cols) {
        float t = 0.0f;
        for (int k = 0; k < 8; ++k) t += part[k][threadIdx.x];
        partial[(int64_t)blockIdx.y * cols + c] = t;
    }
}

__global__ void k_colsum_fin(const float *partial, int chunks, int cols, float *db)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float t = 0.0f;
    for (int k = 0; k < chunks; ++k) t += partial[(int64_t)k * cols + c];
    db[c] = t;
}

// out[c, r] = in[r, c] for an R x C bf16 matrix (pitches ldi, ldo)
__global__ void k_transpose(const __nv_bfloat16 *in, int64_t R, int C, int ldi, __nv_bfloat16 *out, int64_t ldo)
{
    __shared__ __nv_bfloat16 t[32][33];
    const int64_t r0 = (int64_t)blockIdx.y * 32;
    const int c0 = blockIdx.x * 32;
    for (int k = threadIdx.y; k < 32; k += 8) {
        const int64_t r = r0 + k;
        const int c = c0 + threadIdx.x;
        t[k][threadIdx.x] = (r < R && c < C) ? in[r * ldi + c] : tobf(0.0f);
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += 8) {
        const int c = c0 + k;
        const int64_t r = r0 + threadIdx.x;
        if (c < C && r < R) out[(int64_t)c * ldo + r] = t[threadIdx.x][k];
    }
}

// per-block partial sums of (out - tgt)^2 and the gradient scale * (out - tgt)
__global__ void k_mse(const float *out, const __nv_bfloat16 *tgt, int64_t n, float scale, __nv_bfloat16 *dout,
                      float *partial)
{
    __shared__ float red[256];
    float s = 0.0f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float d = out[i] - bf(tgt[i]);
        s += d * d;
        if (dout) dout[i] = tobf(scale * d);
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void k_sum(const float *partial, int n, float *out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        float s = 0.0f;
        for (int i = 0; i < n; ++i) s += partial[i];
        *out = s;
    }
}

// Adam (Kingma & Ba 2015) with the bias corrections folded into lr_t and eps_t
__global__ void k_adam(float *w, const float *g, float *m, float *v, int64_t n, float lr_t, float b1, float b2,
                       float eps_t, __nv_bfloat16 *w16)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr_t * mi / (sqrtf(vi) + eps_t);
        w[i] = wi;
        if (w16) w16[i] = tobf(wi);
    }
}

__global__ void k_to_bf16(const float *x, int64_t n, __nv_bfloat16 *y)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = tobf(x[i]);
}

// dst[b, :] = [src[b, 0:ns] | extra[b, 0:ne] | 0 ...] with dst pitch ldd
__global__ void k_concat(const __nv_bfloat16 *src, int ns, const float *extra, int ne, int B, __nv_bfloat16 *dst,
                         int ldd)
{
    const int64_t total = (int64_t)B * ldd;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int b = (int)(i / ldd), k = (int)(i - (int64_t)b * ldd);
        __nv_bfloat16 v = tobf(0.0f);
        if (k < ns) v = src[(int64_t)b * ns + k];
        else if (k - ns < ne) v = tobf(extra[(int64_t)b * ne + (k - ns)]);
        dst[i] = v;
    }
}
}  // namespace

namespace {
bool small(int64_t n) { return n < ((int64_t)1 << 31); }
}  // namespace

int im2col2d(const __nv_bfloat16 *x, int B, int H, int W, int C, __nv_bfloat16 *col, int ld, cudaStream_t st)
{
    const int64_t n = (int64_t)B * (H / 2) * (W / 2) * ld;
    if (!small(n) || !small((int64_t)B * H * W * C)) return (int)cudaErrorInvalidValue;
    if (C % 8 == 0 && ld % 8 == 0) k_im2col2d_v8<<<grid_for(n / 8, 256), 256, 0, st>>>(x, B, H, W, C, col, ld);
    else k_im2col2d<<<grid_for(n, 256), 256, 0, st>>>(x, B, H, W, C, col, ld);
    return (int)cudaGetLastError();
}

int col2im2d(const __nv_bfloat16 *dcol, int ld, int B, int H, int W, int C, __nv_bfloat16 *dx, cudaStream_t st)
{
    const int64_t n = (int64_t)B * H * W * C;
    if (!small(n) || !small((int64_t)B * (H / 2) * (W / 2) * ld) || C % 8 || ld % 8) return (int)cudaErrorInvalidValue;
    k_col2im2d_v8<<<grid_for(n / 8, 256), 256, 0, st>>>(dcol, ld, B, H, W, C, dx);
    return (int)cudaGetLastError();
}

int im2col1d(const __nv_bfloat16 *x, int B, int T, int C, int up, __nv_bfloat16 *col, int ld, cudaStream_t st)
{
    const int64_t n = (int64_t)B * T * up * ld;
    if (!small(n) || C % 8 || ld % 8) return (int)cudaErrorInvalidValue;
    k_im2col1d_v8<<<grid_for(n / 8, 256), 256, 0, st>>>(x, B, T, C, up, col, ld);
    return (int)cudaGetLastError();
}

int col2im1d(const __nv_bfloat16 *dcol, int ld, int B, int T, int C, int up, __nv_bfloat16 *dx, cudaStream_t st)
{
    const int64_t n = (int64_t)B * T * C;
    if (!small(n) || !small((int64_t)B * T * up * ld) || C % 8 || ld % 8) return (int)cudaErrorInvalidValue;
    k_col2im1d_v8<<<grid_for(n / 8, 256), 256, 0, st>>>(dcol, ld, B, T, C, up, dx);
    return (int)cudaGetLastError();
}

int relu_bwd(const __nv_bfloat16 *dy, int ldy, const __nv_bfloat16 *y, int64_t rows, int cols, __nv_bfloat16 *dz,
             cudaStream_t st)
{
    if (!small(rows * (int64_t)(cols > ldy ? cols : ldy)) || cols % 8 || ldy % 8) return (int)cudaErrorInvalidValue;
    k_relu_bwd_v8<<<grid_for(rows * cols / 8, 256), 256, 0, st>>>(dy, ldy, y, (int)rows, cols, dz);
    return (int)cudaGetLastError();
}

int colsum(const __nv_bfloat16 *dz, int64_t rows, int cols, int ld, float *db, float *partial, cudaStream_t st)
{
    const int64_t chunks = (rows + kColChunkRows - 1) / kColChunkRows;
    if (chunks < 1 || chunks > 65535) return (int)cudaErrorInvalidValue;
    k_colsum_part<<<dim3((cols + 31) / 32, (unsigned)chunks), dim3(32, 8), 0, st>>>(dz, rows, cols, ld, partial);
    k_colsum_fin<<<(cols + 127) / 128, 128, 0, st>>>(partial, (int)chunks, cols, db);
    return (int)cudaGetLastError();
}

int transpose(const __nv_bfloat16 *in, int64_t R, int C, int ldi, __nv_bfloat16 *out, int64_t ldo, cudaStream_t st)
{
    const dim3 grid((C + 31) / 32, (unsigned)((R + 31) / 32));
    if (grid.y > 65535) return (int)cudaErrorInvalidValue;
    k_transpose<<<grid, dim3(32, 8), 0, st>>>(in, R, C, ldi, out, ldo);
    return (int)cudaGetLastError();
}

int mse(const float *out, const __nv_bfloat16 *tgt, int64_t n, float grad_scale, __nv_bfloat16 *dout, float *partial,
        float *loss_sum, cudaStream_t st)
{
    k_mse<<<kMseBlocks, 256, 0, st>>>(out, tgt, n, grad_scale, dout, partial);
    k_sum<<<1, 32, 0, st>>>(partial, kMseBlocks, loss_sum);
    return (int)cudaGetLastError();
}

int adam(float *w, const float *g, float *m, float *v, int64_t n, float lr_t, float b1, float b2, float eps_t,
         __nv_bfloat16 *w16, cudaStream_t st)
{
    k_adam<<<grid_for(n, 256), 256, 0, st>>>(w, g, m, v, n, lr_t, b1, b2, eps_t, w16);
    return (int)cudaGetLastError();
}

int to_bf16(const float *x, int64_t n, __nv_bfloat16 *y, cudaStream_t st)
{
    k_to_bf16<<<grid_for(n, 256), 256, 0, st>>>(x, n, y);
    return (int)cudaGetLastError();
}

int concat(const __nv_bfloat16 *src, int ns, const float *extra, int ne, int B, __nv_bfloat16 *dst, int ldd,
           cudaStream_t st)
{
    k_concat<<<grid_for((int64_t)B * ldd, 256), 256, 0, st>>>(src, ns, extra, ne, B, dst, ldd);
    return (int)cudaGetLastError();
}


// dst row r = src row idx[r] (rows of vecs_per_row V's): one V per thread step
template <class V>
__global__ void k_gather_rows(const V *src, int64_t vecs_per_row, const int64_t *idx, int n, V *dst)
{
    const int64_t total = (int64_t)n * vecs_per_row;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / vecs_per_row, v = i - r * vecs_per_row;
        dst[i] = src[idx[r] * vecs_per_row + v];
    }
}

int gather_rows(const void *src, int64_t row_bytes, const int64_t *idx, int n, void *dst, cudaStream_t st)
{
    if (n < 0 || row_bytes <= 0 || row_bytes % 4 || ((uintptr_t)src & 3) || ((uintptr_t)dst & 3))
        return (int)cudaErrorInvalidValue;
    if (n == 0) return 0;
    // 16-byte vectors where rows and bases allow, else 4-byte words
    const bool v16 = row_bytes % 16 == 0 && ((uintptr_t)src & 15) == 0 && ((uintptr_t)dst & 15) == 0;
    const int64_t vecs = row_bytes / (v16 ? 16 : 4), total = (int64_t)n * vecs;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 8 * 152) blocks = 8 * 152;
    if (v16)
        k_gather_rows<uint4><<<blocks, 256, 0, st>>>(static_cast<const uint4 *>(src), vecs, idx, n,
                                                      static_cast<uint4 *>(dst));
    else
        k_gather_rows<uint32_t><<<blocks, 256, 0, st>>>(static_cast<const uint32_t *>(src), vecs, idx, n,
                                                         static_cast<uint32_t *>(dst));
    return (int)cudaGetLastError();
}

}  // namespace sg

// ---- C ABI: the row gather on its own (device pointers; idx: n row indices
// into src, each < the caller's row count)
extern "C" int poe_sg_gather_rows(const void *src, int64_t row_bytes, const int64_t *idx, int32_t n, void *dst,
                                  void *stream)
{
    if (!src || !dst || (n > 0 && !idx)) return 1;   // POE_EINVAL
    const int rc = sg::gather_rows(src, row_bytes, idx, n, dst, (cudaStream_t)stream);
    return rc == 0 ? 0 : (rc == (int)cudaErrorInvalidValue ? 1 : 5);
}
