// poe2d_tile.cu -- launches of the fused step kernel, one step per launch or
// a step-spanning launch of several (its variants are compiled in
// poe2d_tile_fast.cu, poe2d_tile_exact.cu and poe2d_tile_exact_any.cu from
// poe2d_tile.cuh), and the small kernels around it: step clocks, the
// bounded-wait check, derived fields.
#include <cuda_runtime.h>

#include <mutex>

#include "poe2d_tile.cuh"

namespace poe {

namespace {
using tile::mbar_fence_init;
using tile::mbar_init;
using tile::mbar_wait_n;

// the stencil mode of a launch: FAST, or EXACT for the spacings of its models
int stencil_mode(bool exact, bool few)
{
    return !exact ? SM_FAST : (few ? SM_EXACT_FEW : SM_EXACT_ANY);
}

int step_mode(int sm, const ModelDev &m, const ModelDev *models, const StreamShot *shots, const int4 *items,
              int nitems, int k, int nk, bool kone, bool coef, int *queue, void *stream)
{
    switch (sm) {
    case SM_FAST: return tile_step_fast(m, models, shots, items, nitems, k, nk, kone, coef, queue, stream);
    case SM_EXACT_FEW: return tile_step_exact(m, models, shots, items, nitems, k, nk, kone, coef, queue, stream);
    default: return tile_step_exact_any(m, models, shots, items, nitems, k, nk, kone, coef, queue, stream);
    }
}
}  // namespace

int launch_tile_step(const ModelDev &m, const StreamShot *shots_dev, int nshots, const int4 *items, int nitems, int k,
                     int nk, bool exact, bool kone, int tile_z, int *queue, void *stream)
{
    (void)nshots;
    if (tile_z == PAL_TZ_SMALL) {
        if (exact) return (int)cudaErrorInvalidValue;   // built for FAST stencils only
        return tile_step_fast16(m, shots_dev, items, nitems, k, nk, kone, m.ids == nullptr, queue, stream);
    }
    if (tile_z != PAL_TZ) return (int)cudaErrorInvalidValue;
    return step_mode(stencil_mode(exact, m.qx.few_bits && m.qz.few_bits), m, nullptr, shots_dev, items, nitems, k,
                     nk, kone, m.ids == nullptr, queue, stream);
}

int launch_batch_step(const ModelDev *models_dev, const StreamShot *shots_dev, const int4 *items, int nitems, int k,
                      int nk, bool exact, bool exact_few, bool coef, bool kone, int *queue, void *stream)
{
    const ModelDev dummy{};
    return step_mode(stencil_mode(exact, exact_few), dummy, models_dev, shots_dev, items, nitems, k, nk, kone, coef,
                     queue, stream);
}

// the step kernel's bounded waits, on the GPU: (1) an mbarrier phase that
// never completes (no thread arrives), (2) tile flags one of which nothing
// sets (flags[0] = 0; flags[1..8] hold 5), (3) the same flags with the unset
// one not watched, which must pass.  err: bit 0 and bit 1 when waits (1) and
// (2) gave up after `polls` polls, bit 2 if wait (3) did
__global__ void k_wait_limit(int *err, const int *flags, int polls)
{
    __shared__ uint64_t bar;
    const int lane = threadIdx.x;
    if (lane == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (lane == 0 && !mbar_wait_n(&bar, 0, polls)) atomicOr(err, 1);
    __syncwarp();
    if (!tile::wait_flags(lane < 9 ? flags + lane : nullptr, 1, polls) && lane == 0) atomicOr(err, 2);
    if (!tile::wait_flags(lane >= 1 && lane < 9 ? flags + lane : nullptr, 5, polls) && lane == 0) atomicOr(err, 4);
}

int launch_wait_limit(int *err, const int *flags, int polls, void *stream)
{
    k_wait_limit<<<1, 32, 0, (cudaStream_t)stream>>>(err, flags, polls);
    return (int)cudaGetLastError();
}

__global__ void k_advance_shots(const StreamShot *shots, int nshots, int64_t by)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nshots) *const_cast<int64_t *>(shots[i].step) += by;
}

int launch_advance_shots(const StreamShot *shots_dev, int nshots, int64_t by, void *stream)
{
    if (nshots <= 0) return 0;
    k_advance_shots<<<(nshots + 127) / 128, 128, 0, (cudaStream_t)stream>>>(shots_dev, nshots, by);
    return (int)cudaGetLastError();
}

// ---- small helpers: step counters and derived fields ----
__global__ void k_advance(int64_t *steps, int nshots, int64_t by)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nshots) steps[i] += by;
}

int launch_advance(int64_t *steps_dev, int nshots, int64_t by, void *stream)
{
    k_advance<<<(nshots + 127) / 128, 128, 0, (cudaStream_t)stream>>>(steps_dev, nshots, by);
    return (int)cudaGetLastError();
}

// sigma_xx, sigma_zz, p of a shot's current state (they are not stored by the
// step kernel); n = steps done, the source term of step n is included.
__global__ void k_derive(const ModelDev m, const StreamShot *__restrict__ shots, int shot, int64_t n, float *out)
{
    const StreamShot &S = shots[shot];
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.y;
    if (x > m.NX || z > m.NZ) return;
    const int NX = m.NX, NZ = m.NZ;
    const int64_t P = m.P, PL = m.plane;
    const int64_t o = (int64_t)(z + ZH) * P + (x + XH);
    const float *F = S.f[n & 1];
    // coefficient c (plane order) from the planes or the palette table
    auto coef = [&](int c) {
        const int mt = c == C_LC ? MT_LC : (c == C_MU ? MT_MU : (c == C_AL ? MT_AL : MT_M));
        return m.ids ? m.mtab[MT_W * m.ids[o] + mt] : m.coef[c * PL + o];
    };
    const bool g1 = x >= 1 && x <= NX - 1 && z >= 2 && z <= NZ - 2;
    const bool g3 = x >= 1 && x <= NX - 2 && z >= 2 && z <= NZ - 1;
    const float g11 = F[SF_G11 * PL + o], g22 = F[SF_G22 * PL + o];
    const float al = coef(C_AL), M = coef(C_M);
    float pv = 0.0f;
    if (g1) pv = -al * M * (g11 + g22) + M * (F[SF_XI1 * PL + o] + F[SF_XI2 * PL + o]);
    const bool is_src = o == S.src_off;
    if (is_src) {
        if (!g1) pv = S.acc[n & 1];
        else if (S.src_where == SRC_P && n >= 1 && n <= S.src_n) pv = pv + S.src_tab[n - 1];
    }
    float sxx = 0.0f, szz = 0.0f;
    if (g3) sxx_szz_exact(coef(C_LC), coef(C_MU), g11, g22, al, pv, sxx, szz);
    out[0 * PL + o] = sxx;
    out[1 * PL + o] = szz;
    out[2 * PL + o] = pv;
}

int launch_derive(const ModelDev &m, const StreamShot *shots_dev, int shot, int64_t n, float *out, void *stream)
{
    dim3 grd((m.NX + 1 + 127) / 128, m.NZ + 1);
    k_derive<<<grd, 128, 0, (cudaStream_t)stream>>>(m, shots_dev, shot, n, out);
    return (int)cudaGetLastError();
}

// ---- allocation-free read-out of one derived field ----
// For callers that cannot allocate device memory: the one-plane scratch lives
// in this file-scope array, loaded with the library and held by every device
// that loads it until the process exits.  32 MiB: padded planes of up to
// 8 Mi floats (grids up to about 2850 x 2850 cells).
static __device__ __align__(256) float g_noalloc_scratch[NOALLOC_SCRATCH_FLOATS];

// sigma_xx (which = 0), sigma_zz (1) or p (2) of one shot's current state into
// one padded plane; the same arithmetic as k_derive
__global__ void k_derive_one(const ModelDev m, const float *__restrict__ F, const float *__restrict__ acc,
                             int64_t src_off, int src_where, int64_t src_n, const float *__restrict__ src_tab,
                             int64_t n, int which, float *out)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.y;
    if (x > m.NX || z > m.NZ) return;
    const int NX = m.NX, NZ = m.NZ;
    const int64_t P = m.P, PL = m.plane;
    const int64_t o = (int64_t)(z + ZH) * P + (x + XH);
    auto coef = [&](int c) {
        const int mt = c == C_LC ? MT_LC : (c == C_MU ? MT_MU : (c == C_AL ? MT_AL : MT_M));
        return m.ids ? m.mtab[MT_W * m.ids[o] + mt] : m.coef[c * PL + o];
    };
    const bool g1 = x >= 1 && x <= NX - 1 && z >= 2 && z <= NZ - 2;
    const bool g3 = x >= 1 && x <= NX - 2 && z >= 2 && z <= NZ - 1;
    const float g11 = F[SF_G11 * PL + o], g22 = F[SF_G22 * PL + o];
    const float al = coef(C_AL), M = coef(C_M);
    float pv = 0.0f;
    if (g1) pv = -al * M * (g11 + g22) + M * (F[SF_XI1 * PL + o] + F[SF_XI2 * PL + o]);
    if (o == src_off) {
        if (!g1) pv = acc[n & 1];
        else if (src_where == SRC_P && n >= 1 && n <= src_n) pv = pv + src_tab[n - 1];
    }
    float sxx = 0.0f, szz = 0.0f;
    if (g3) sxx_szz_exact(coef(C_LC), coef(C_MU), g11, g22, al, pv, sxx, szz);
    out[o] = which == 0 ? sxx : (which == 1 ? szz : pv);
}

namespace {
std::mutex g_noalloc_mu;
float *g_noalloc_ptr[256] = {};   // device address of g_noalloc_scratch, per device ordinal
}  // namespace

int derive_noalloc(const ModelDev &m, const float *F, const float *acc, int64_t src_off, int src_where,
                   int64_t src_n, const float *src_tab, int64_t n, int which, float *host_out, void *stream)
{
    if (m.plane > NOALLOC_SCRATCH_FLOATS) return (int)cudaErrorInvalidValue;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return (int)e;
    if (dev < 0 || dev >= 256) return (int)cudaErrorInvalidDevice;
    float *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            // the array's name is a host-side stand-in: its device address is
            // looked up once per device, with that device current
            e = cudaGetSymbolAddress((void **)&g_noalloc_ptr[dev], g_noalloc_scratch);
            if (e != cudaSuccess) {
                g_noalloc_ptr[dev] = nullptr;
                return (int)e;
            }
        }
        scratch = g_noalloc_ptr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    dim3 grd((m.NX + 1 + 127) / 128, m.NZ + 1);
    k_derive_one<<<grd, 128, 0, st>>>(m, F, acc, src_off, src_where, src_n, src_tab, n, which, scratch);
    if ((e = cudaGetLastError()) != cudaSuccess) return (int)e;
    const int nx = m.NX + 1, nz = m.NZ + 1;
    e = cudaMemcpy2DAsync(host_out, sizeof(float) * nx, scratch + (int64_t)ZH * m.P + XH, sizeof(float) * m.P,
                          sizeof(float) * nx, nz, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return (int)e;
    return (int)cudaStreamSynchronize(st);
}

}  // namespace poe
