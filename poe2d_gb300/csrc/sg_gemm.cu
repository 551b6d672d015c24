// sg_gemm.cu -- BF16 tensor-core GEMM for the surrogate network (sm_103a).
//
//   C[M x N] = alpha * A[M x K] . B[N x K]^T (+ bias[n]) (ReLU) (+= C)
//
// A and B are bf16, row-major with K contiguous (K-major), FP32 accumulation
// in tensor memory.  One CTA of 128 threads computes a 128 x BN tile:
//   thread 0    TMA producer: a 2- or 3-stage ring of 128x64 (A) and BNx64 (B)
//               tiles, 128-byte swizzled, one mbarrier per stage;
//   thread 32   MMA issuer: four tcgen05.mma (K = 16 each) per stage, then
//               tcgen05.commit frees the stage; a last commit signals the end;
//   warps 0-3   epilogue: each warp reads its 32 TMEM lanes (rows) with
//               tcgen05.ld and applies alpha, bias, ReLU; a plain output
//               (FP32 or bf16, not accumulated, one K split) is staged in the
//               freed pipeline stages as 128-byte-swizzled 128 x 128-byte
//               blocks and written by TMA tensor stores (coalesced whole
//               rows, asynchronous), otherwise each thread stores its row.
// K may be split over blockIdx.z (ksplit > 1): each split writes an FP32
// partial tile to a workspace and a reduction kernel applies the epilogue in
// a fixed order, so results do not depend on scheduling.
//
// Out-of-range rows and K columns of a TMA box are zero-filled by the copy
// engine, so M, N and K need no padding; the global row pitches must be
// multiples of 8 elements (16 bytes) and the bases 16-byte aligned.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>

#include "launch_attr.h"
#include "sg_internal.h"
#include "sm103_ptx.cuh"

namespace sg {
using namespace sm103;

namespace {
constexpr int BM = 128, BK = 64, NT = 128;

// ST pipeline stages: 3 for long reductions (2 CTAs per SM); 2 when a CTA
// sees at most 4 k-blocks, which keeps shared memory small enough for 3 CTAs
// per SM, so one CTA's epilogue overlaps another's loads and MMAs
template <int BN, int ST>
struct GemmSmem {
    static constexpr int STAGES = ST;
    static constexpr int A_BYTES = BM * BK * 2;             // 16 KB
    static constexpr int B_BYTES = BN * BK * 2;
    static constexpr int STAGE = A_BYTES + B_BYTES;
    static_assert(BM * BN * 4 <= STAGES * STAGE, "an FP32 output tile fits in the pipeline stages");
    static constexpr int BAR_OFF = STAGES * STAGE;
    static constexpr int BIAS_OFF = BAR_OFF + (2 * STAGES + 1) * 8 + 8;
    static constexpr int TOTAL = BIAS_OFF + BN * 4 + 1024;   // + alignment slack
    static constexpr uint32_t TX = (uint32_t)STAGE;
    static constexpr uint32_t TMEM_COLS = BN < 32 ? 32 : BN;
};

// output through TMA stores: OUT_F32 (32-column blocks) or OUT_BF16 (64-column blocks)
enum { OUT_THREADS = 0, OUT_F32 = 1, OUT_BF16 = 2 };

// A operand of a k = 3 time convolution read in place (T > 0): tA is the 3-D
// map {cin, T, B} of x, k-block kk = 64 j of K = 3 cin reads tap kk / cin,
// channels kk % cin, rows s + off[tap] of the tile's items; the output rows
// are the phase's rows of the upsampled time axis (tC 3-D {N, up, M})
struct ConvA {
    int T = 0, cin = 0, up = 1, phase = 0;
    int off[3] = {0, 0, 0};
};

template <int BN, int STAGES>
__global__ void __launch_bounds__(NT, 1)
k_gemm(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tB,
       const __grid_constant__ CUtensorMap tC, int out_mode, const ConvA ca, int M, int N, int K,
       int kblocks_per_split, Epilogue e, float *partial, int *err)
{
    using L = GemmSmem<BN, STAGES>;
    extern __shared__ unsigned char smraw[];
    unsigned char *sm = (unsigned char *)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = reinterpret_cast<uint64_t *>(sm + L::BAR_OFF);
    uint64_t *empty = full + STAGES;
    uint64_t *done = empty + STAGES;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(done + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int nkb_total = (K + BK - 1) / BK;
    const int kb0 = blockIdx.z * kblocks_per_split;
    int kb1 = kb0 + kblocks_per_split;
    if (kb1 > nkb_total) kb1 = nkb_total;
    const int nkb = kb1 > kb0 ? kb1 - kb0 : 0;

    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        mbar_fence_init();
    }
    if (warp == 2) tmem_alloc(tslot, L::TMEM_COLS);
    // the tile's bias once, for the epilogue (zero past N or without a bias)
    float *sbias = reinterpret_cast<float *>(sm + L::BIAS_OFF);
    for (int i = tid; i < BN; i += NT) sbias[i] = (e.bias && n0 + i < N) ? e.bias[n0 + i] : 0.0f;
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    bool ok = true;

    if (tid == 0) {   // producer
        int issued = 0;
        for (int i = 0; i < nkb; ++i) {
            const int s = i % STAGES;
            if (i >= STAGES && !mbar_wait(&empty[s], (uint32_t)(((i / STAGES) - 1) & 1))) {
                ok = false;
                break;
            }
            unsigned char *a = sm + s * L::STAGE;
            mbar_expect_tx(&full[s], L::TX);
            if (ca.T > 0) {
                // the tile's 128 rows of x: one item's rows m0 % T .. +127 (T >= 128) or
                // 128 / T whole items (T < 128), shifted by the tap's offset (rows
                // outside an item arrive as zeros: the convolution's padding)
                const int kk = (kb0 + i) * BK, tap = kk / ca.cin, b0 = m0 / ca.T;
                const int off = tap == 0 ? ca.off[0] : (tap == 1 ? ca.off[1] : ca.off[2]);
                tma_load_3d(a, &tA, kk - tap * ca.cin, m0 - b0 * ca.T + off, b0, &full[s]);
            } else {
                tma_load_2d(a, &tA, (kb0 + i) * BK, m0, &full[s]);
            }
            tma_load_2d(a + L::A_BYTES, &tB, (kb0 + i) * BK, n0, &full[s]);
            issued = i + 1;
        }
        // copies still in flight must land before the CTA can leave
        for (int i = issued - STAGES < 0 ? 0 : issued - STAGES; i < issued; ++i)
            if (!mbar_wait(&full[i % STAGES], (uint32_t)((i / STAGES) & 1))) ok = false;
    } else if (tid == 32) {   // MMA issuer
        constexpr uint32_t idesc = idesc_bf16_f32(BM, BN);
        for (int i = 0; i < nkb; ++i) {
            const int s = i % STAGES;
            if (!mbar_wait(&full[s], (uint32_t)((i / STAGES) & 1))) {
                ok = false;
                break;
            }
            tc_fence_after();
            const uint32_t a = smem_u32(sm + s * L::STAGE);
            const uint64_t ad = desc_k_sw128(a), bd = desc_k_sw128(a + L::A_BYTES);
#pragma unroll
            for (int k = 0; k < BK / 16; ++k)
                tc_mma_f16(tmem, ad + 2 * k, bd + 2 * k, idesc, (i | k) ? 1u : 0u);
            tc_commit(&empty[s]);
        }
        tc_commit(done);   // arrives once every MMA above has completed
    }
    __syncwarp();

    // epilogue: warp w owns TMEM lanes (tile rows) 32w .. 32w+31
    if (!mbar_wait(done, 0)) ok = false;
    tc_fence_after();
    if (!ok) atomicExch(err, 1);
    const int row = m0 + warp * 32 + lane;
    const bool row_ok = row < M && nkb > 0;
    // 16-byte vector stores where the row pitch keeps 16-column chunks aligned
    const bool vec32 = (e.ldc % 4) == 0 && (((uintptr_t)(partial ? (void *)partial : (void *)e.out_f32)) & 15) == 0;
    const bool vec16 = (e.ldc % 8) == 0 && (((uintptr_t)e.out_bf16) & 15) == 0;
    // a staged output goes out block by block as soon as every warp has put its
    // rows of the block in (the stores overlap the remaining TMEM reads); every
    // thread's waits are over, so whether any gave up is known now
    const bool staged = out_mode != OUT_THREADS;
    const bool store_ok = staged ? __syncthreads_and(ok) != 0 : false;
#pragma unroll 1
    for (int c2 = 0; c2 < BN / 32; ++c2) {
        // two 16-column TMEM loads in flight per wait
        uint32_t vv[2][16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c2 * 32), vv[0]);
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c2 * 32 + 16), vv[1]);
        tmem_ld_wait();
        if (row_ok && ok) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint32_t (&v)[16] = vv[h];
            const int c = 2 * c2 + h;
            const int nb = n0 + c * 16;
            const bool full = nb + 16 <= N;
            if (partial) {   // split-K: raw partial sums
                float *p = partial + ((size_t)blockIdx.z * M + row) * e.ldc + nb;
                if (full && vec32) {
    #pragma unroll
                    for (int q = 0; q < 4; ++q)
                        reinterpret_cast<float4 *>(p)[q] = make_float4(__uint_as_float(v[4 * q]), __uint_as_float(v[4 * q + 1]),
                                                                       __uint_as_float(v[4 * q + 2]), __uint_as_float(v[4 * q + 3]));
                } else {
    #pragma unroll
                    for (int j = 0; j < 16; ++j)
                        if (nb + j < N) p[j] = __uint_as_float(v[j]);
                }
                continue;
            }
            float x[16];
    #pragma unroll
            for (int j = 0; j < 16; ++j) {
                float t = e.alpha * __uint_as_float(v[j]);
                t += sbias[c * 16 + j];
                if (e.relu) t = fmaxf(t, 0.0f);
                x[j] = t;
            }
            if (out_mode != OUT_THREADS) {
                // 128 x 128-byte block of this column range; 16-byte piece q of
                // row r sits at piece q ^ (r & 7) (the 128-byte swizzle)
                const int r = warp * 32 + lane, sw = r & 7;
                if (out_mode == OUT_F32) {
                    unsigned char *blk = sm + (c >> 1) * (BM * 128) + r * 128;
    #pragma unroll
                    for (int q = 0; q < 4; ++q)
                        *reinterpret_cast<float4 *>(blk + ((((c & 1) * 4 + q) ^ sw) << 4)) =
                            make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
                } else {
                    unsigned char *blk = sm + (c >> 2) * (BM * 128) + r * 128;
    #pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        uint4 w;
                        __nv_bfloat162 *h2 = reinterpret_cast<__nv_bfloat162 *>(&w);
    #pragma unroll
                        for (int i = 0; i < 4; ++i) h2[i] = __floats2bfloat162_rn(x[8 * q + 2 * i], x[8 * q + 2 * i + 1]);
                        *reinterpret_cast<uint4 *>(blk + ((((c & 3) * 2 + q) ^ sw) << 4)) = w;
                    }
                }
                continue;
            }
            const size_t o = (size_t)row * e.ldc + nb;
            if (e.out_f32) {
                float *p = e.out_f32 + o;
                if (full && vec32) {
    #pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        float4 w = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
                        if (e.accumulate) {
                            const float4 a = reinterpret_cast<const float4 *>(p)[q];
                            w.x += a.x; w.y += a.y; w.z += a.z; w.w += a.w;
                        }
                        reinterpret_cast<float4 *>(p)[q] = w;
                        x[4 * q] = w.x; x[4 * q + 1] = w.y; x[4 * q + 2] = w.z; x[4 * q + 3] = w.w;
                    }
                } else {
    #pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        if (nb + j >= N) continue;
                        if (e.accumulate) x[j] += p[j];
                        p[j] = x[j];
                    }
                }
            }
            if (e.out_bf16) {
                __nv_bfloat16 *p = e.out_bf16 + o;
                if (full && vec16) {
    #pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        uint4 w;
                        __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&w);
    #pragma unroll
                        for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(x[8 * q + 2 * i], x[8 * q + 2 * i + 1]);
                        reinterpret_cast<uint4 *>(p)[q] = w;
                    }
                } else {
    #pragma unroll
                    for (int j = 0; j < 16; ++j)
                        if (nb + j < N) p[j] = __float2bfloat16_rn(x[j]);
                }
            }
        }
        }
        // the 128-byte block this chunk completes: a 32-column block (FP32) after
        // every chunk, a 64-column block (bf16) after every second one
        if (staged && (out_mode == OUT_F32 || (c2 & 1))) {
            fence_proxy_async_smem();
            __syncthreads();
            const int cols = out_mode == OUT_F32 ? 32 : 64, j = out_mode == OUT_F32 ? c2 : c2 >> 1;
            if (tid == 0 && store_ok && nkb > 0 && n0 + j * cols < N) {
                if (ca.T > 0) tma_store_3d(&tC, n0 + j * cols, ca.phase, m0, sm + j * (BM * 128));
                else tma_store_2d(&tC, n0 + j * cols, m0, sm + j * (BM * 128));
                bulk_commit();
            }
        }
    }
    if (staged && tid == 0 && store_ok && nkb > 0)
        bulk_wait_read_all();   // the stores have read the stage buffers (the writes complete on their own)
    tc_fence_before();
    __syncthreads();
    if (warp == 2) tmem_dealloc(tmem, L::TMEM_COLS);
}

// sum of the split-K partials in split order, then the epilogue
__global__ void k_splitk_reduce(const float *partial, int splits, int M, int N, Epilogue e)
{
    const size_t total = (size_t)M * N;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int row = (int)(i / N), n = (int)(i - (size_t)row * N);
        const size_t o = (size_t)row * e.ldc + n;
        float x = 0.0f;
        for (int s = 0; s < splits; ++s) x += partial[(size_t)s * M * e.ldc + o];
        x *= e.alpha;
        if (e.bias) x += e.bias[n];
        if (e.relu) x = fmaxf(x, 0.0f);
        if (e.out_f32) {
            if (e.accumulate) x += e.out_f32[o];
            e.out_f32[o] = x;
        }
        if (e.out_bf16) e.out_bf16[o] = __float2bfloat16_rn(x);
    }
}

typedef CUresult (*EncodeFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                             const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                             CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encode_fn()
{
    static EncodeFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeFn)p;
    });
    return fn;
}

// bf16 rows x cols (cols contiguous, pitch ld elements), box 64 x box_rows, 128-B swizzle
bool make_map(CUtensorMap *m, const void *base, int rows, int cols, int ld, int box_rows)
{
    EncodeFn fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the output C as the TMA store's tensor: N columns x M rows (pitch ldc
// elements), 128 x 128-byte boxes, 128-byte swizzle
bool make_out_map(CUtensorMap *m, void *base, bool f32, int rows, int cols, int ldc)
{
    EncodeFn fn = encode_fn();
    if (!fn) return false;
    const int es = f32 ? 4 : 2;
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ldc * es};
    const cuuint32_t box[2] = {(cuuint32_t)(128 / es), (cuuint32_t)BM};
    const cuuint32_t estr[2] = {1, 1};
    return fn(m, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box,
              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_NONE,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int sm_count()
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

template <int BN, int ST>
int launch(const CUtensorMap &ta, const CUtensorMap &tb, const CUtensorMap &tc, int out_mode, const ConvA &ca, int M,
           int N, int K, int splits, int kper, const Epilogue &e, float *ws, int *err, cudaStream_t st)
{
    using L = GemmSmem<BN, ST>;
    static std::atomic<uint64_t> done{0};
    poe::smem_attr_once(k_gemm<BN, ST>, L::TOTAL, done);
    const dim3 grid((M + BM - 1) / BM, (N + BN - 1) / BN, splits);
    k_gemm<BN, ST><<<grid, NT, L::TOTAL, st>>>(ta, tb, tc, out_mode, ca, M, N, K, kper, e,
                                               splits > 1 ? ws : nullptr, err);
    return (int)cudaGetLastError();
}

// the tile kernel for BN columns and a stage count by the k-blocks per CTA
int launch_any(int BN, bool short_k, const CUtensorMap &ta, const CUtensorMap &tb, const CUtensorMap &tc,
               int out_mode, const ConvA &ca, int M, int N, int K, int splits, int kper, const Epilogue &e, float *ws,
               int *err, cudaStream_t st)
{
    return BN == 128
               ? (short_k ? launch<128, 2>(ta, tb, tc, out_mode, ca, M, N, K, splits, kper, e, ws, err, st)
                          : launch<128, 3>(ta, tb, tc, out_mode, ca, M, N, K, splits, kper, e, ws, err, st))
               : (short_k ? launch<64, 2>(ta, tb, tc, out_mode, ca, M, N, K, splits, kper, e, ws, err, st)
                          : launch<64, 3>(ta, tb, tc, out_mode, ca, M, N, K, splits, kper, e, ws, err, st));
}
}  // namespace

int gemm(const Gemm &g, const Epilogue &e, float *ws, int64_t ws_floats, int *err, cudaStream_t st)
{
    if (g.M <= 0 || g.N <= 0 || g.K <= 0) return (int)cudaErrorInvalidValue;
    if (g.lda % 8 || g.ldb % 8 || g.lda < g.K || g.ldb < g.K || ((uintptr_t)g.A & 15) || ((uintptr_t)g.B & 15))
        return (int)cudaErrorInvalidValue;
    if (e.ldc < g.N) return (int)cudaErrorInvalidValue;
    const int BN = g.N > 64 ? 128 : 64;
    CUtensorMap ta, tb;
    if (!make_map(&ta, g.A, g.M, g.K, g.lda, BM) || !make_map(&tb, g.B, g.N, g.K, g.ldb, BN))
        return (int)cudaErrorInvalidValue;
    // split K when the tile grid leaves most SMs idle and K is long
    const int tiles = ((g.M + BM - 1) / BM) * ((g.N + BN - 1) / BN);
    const int nkb = (g.K + BK - 1) / BK;
    int splits = 1;
    if (ws && tiles < sm_count() / 2 && nkb >= 8) {
        splits = sm_count() / tiles;
        if (splits > kMaxSplits) splits = kMaxSplits;
        if (splits > nkb / 4) splits = nkb / 4;
        if (splits < 1) splits = 1;
        while (splits > 1 && (int64_t)splits * g.M * e.ldc > ws_floats) --splits;
    }
    const int kper = (nkb + splits - 1) / splits;
    splits = (nkb + kper - 1) / kper;
    const bool short_k = kper <= 4;
    // one plain output (no accumulation, one K split, 16-byte rows and base):
    // written by TMA stores from the stage buffers
    CUtensorMap tc;
    std::memset(&tc, 0, sizeof(tc));
    int out_mode = OUT_THREADS;
    if (splits == 1 && !e.accumulate && (e.out_f32 == nullptr) != (e.out_bf16 == nullptr)) {
        const bool f32 = e.out_f32 != nullptr;
        void *base = f32 ? (void *)e.out_f32 : (void *)e.out_bf16;
        if ((e.ldc % (f32 ? 4 : 8)) == 0 && ((uintptr_t)base & 15) == 0 &&
            make_out_map(&tc, base, f32, g.M, g.N, e.ldc))
            out_mode = f32 ? OUT_F32 : OUT_BF16;
    }
    int rc = launch_any(BN, short_k, ta, tb, tc, out_mode, ConvA{}, g.M, g.N, g.K, splits, kper, e, ws, err, st);
    if (rc || splits == 1) return rc;
    const int64_t total = (int64_t)g.M * g.N;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 4 * sm_count()) blocks = 4 * sm_count();
    k_splitk_reduce<<<blocks, 256, 0, st>>>(ws, splits, g.M, g.N, e);
    return (int)cudaGetLastError();
}

int gemm_conv1d(const __nv_bfloat16 *x, int B, int T, int cin, int up, int phase, const __nv_bfloat16 *W, int cout,
                const Epilogue &e, int *err, cudaStream_t st)
{
    if (B <= 0 || T <= 0 || (T & (T - 1)) || cin <= 0 || cin % BK || cout <= 0 || (up != 1 && up != 2) ||
        phase < 0 || phase >= up || e.accumulate || (e.out_f32 == nullptr) == (e.out_bf16 == nullptr) ||
        e.ldc < cout || ((uintptr_t)x & 15) || ((uintptr_t)W & 15))
        return (int)cudaErrorInvalidValue;
    const bool f32 = e.out_f32 != nullptr;
    void *out = f32 ? (void *)e.out_f32 : (void *)e.out_bf16;
    const int es = f32 ? 4 : 2;
    if ((e.ldc * es) % 16 || ((uintptr_t)out & 15)) return (int)cudaErrorInvalidValue;
    EncodeFn fn = encode_fn();
    if (!fn) return (int)cudaErrorInvalidValue;
    const int K = 3 * cin, M = B * T, rows = T < BM ? T : BM;
    // x as {cin, T, B}: a box of 64 channels x `rows` times x BM / rows items (128 rows in all)
    CUtensorMap ta, tb, tc;
    {
        const cuuint64_t dims[3] = {(cuuint64_t)cin, (cuuint64_t)T, (cuuint64_t)B};
        const cuuint64_t strides[2] = {(cuuint64_t)cin * 2, (cuuint64_t)T * cin * 2};
        const cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)rows, (cuuint32_t)(BM / rows)};
        const cuuint32_t estr[3] = {1, 1, 1};
        if (fn(&ta, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<__nv_bfloat16 *>(x), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return (int)cudaErrorInvalidValue;
    }
    const int BN = cout > 64 ? 128 : 64;
    if (!make_map(&tb, W, cout, K, K, BN)) return (int)cudaErrorInvalidValue;
    // the output as {cout, up, M}: row up*r + phase of the upsampled time axis
    {
        const cuuint64_t dims[3] = {(cuuint64_t)cout, (cuuint64_t)up, (cuuint64_t)M};
        const cuuint64_t strides[2] = {(cuuint64_t)e.ldc * es, (cuuint64_t)up * e.ldc * es};
        const cuuint32_t box[3] = {(cuuint32_t)(128 / es), 1u, (cuuint32_t)BM};
        const cuuint32_t estr[3] = {1, 1, 1};
        if (fn(&tc, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, out, dims, strides,
               box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_NONE,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return (int)cudaErrorInvalidValue;
    }
    // tap k of output time up*s + phase reads upsampled time up*s + phase + k - 1,
    // which is x row floor((up*s + phase + k - 1) / up) = s + off[k]
    ConvA ca;
    ca.T = T;
    ca.cin = cin;
    ca.up = up;
    ca.phase = phase;
    for (int k = 0; k < 3; ++k) {
        const int d = phase + k - 1;   // up*s + d
        ca.off[k] = d >= 0 ? d / up : -1;
    }
    const int nkb = K / BK;
    return launch_any(BN, nkb <= 4, ta, tb, tc, f32 ? OUT_F32 : OUT_BF16, ca, M, cout, K, 1, nkb, e, nullptr, err,
                      st);
}

}  // namespace sg

// ---- C ABI: the GEMM on its own (device pointers), for tests and callers
// that drive the tensor cores directly
extern "C" int poe_sg_gemm(const void *A, int32_t lda, const void *B, int32_t ldb, int32_t M, int32_t N, int32_t K,
                           float alpha, const float *bias, int32_t relu, float *out_f32, void *out_bf16, int32_t ldc,
                           int32_t accumulate, float *ws, int64_t ws_floats, int32_t *err_dev, void *stream)
{
    if (!A || !B || !err_dev || (!out_f32 && !out_bf16)) return 1;   // POE_EINVAL
    sg::Gemm g{static_cast<const __nv_bfloat16 *>(A), lda, static_cast<const __nv_bfloat16 *>(B), ldb, M, N, K};
    sg::Epilogue e;
    e.alpha = alpha;
    e.bias = bias;
    e.relu = relu;
    e.out_f32 = out_f32;
    e.out_bf16 = static_cast<__nv_bfloat16 *>(out_bf16);
    e.ldc = ldc;
    e.accumulate = accumulate;
    const int rc = sg::gemm(g, e, ws, ws_floats, err_dev, (cudaStream_t)stream);
    return rc == 0 ? 0 : (rc == (int)cudaErrorInvalidValue ? 1 : 5);   // POE_OK / POE_EINVAL / POE_ECUDA
}
