// poe2d_tile.cuh -- the fused time step: stress + velocity in one kernel, one
// step per launch or (step-spanning) many.  Included by one instantiation
// unit per stencil mode (poe2d_tile_fast.cu, poe2d_tile_exact.cu,
// poe2d_tile_exact_any.cu) and by poe2d_tile_fast16.cu (FAST, 60 x 16 tiles),
// which compile in parallel.
//
// k_tile_pal: a persistent, warp-specialised kernel (one CTA per SM) takes
// 60 x 32 (or 60 x 16) tiles of any number of shots (and, for batches, of
// models) from a work queue.  Per tile: stress on the tile + 2-cell halo
// (64 x 36 cells for 32 rows):
// strains, fluid content, sigma2 = p, sigma_xz, sigma_xx, sigma_zz (cu:49-112,
// 202-229, 231-244) -> shared memory, the integrated state of the tile's own
// cells -> HBM; the tile's receivers (before the velocity update, as
// save1_kernel runs, cu:1629); velocity on the tile (cu:279-386) -> HBM.  The
// halo is recomputed so no tile waits for another.  sigma_xx, sigma_zz and p
// never touch HBM.  Tiles re-read this step's inputs in their halos, so the
// state is double-buffered: step n reads buffer (n-1)&1 and writes buffer n&1
// (the stress C-PML memory too; the velocity C-PML memory is per-cell private
// and updated in place).  Coefficients come from a material palette (one byte
// per cell, a table row per material) or, for models with more distinct
// materials, per cell from the 8 coefficient planes (COEF).
//
// Arithmetic per cell is the reference's, in the same order, with its FP64
// sub-expressions rounded as in poe2d_math.cuh (EXACT) or plain FP32
// stencils (FAST); compiled with -fmad=false.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <type_traits>

#include "launch_attr.h"
#include "poe2d_internal.h"

namespace poe {

// stencil modes: plain FP32, and the reference's FP64 rounding for a spacing
// whose 24 h is a float of few bits (0.5, 1, 1.25, ...) or for any spacing
enum { SM_FAST = 0, SM_EXACT_FEW = 1, SM_EXACT_ANY = 2 };

namespace tile {

template <int SM>
__device__ __forceinline__ float D4(float a, float b, float c, float d, const Div24 &q)
{
    return SM == SM_FAST ? d4_fast(a, b, c, d, q)
                         : (SM == SM_EXACT_FEW ? d4_exact_few(a, b, c, d, q) : d4_exact_any(a, b, c, d, q));
}

template <bool KONE>
__device__ __forceinline__ float KDIV(float v, float K)
{
    return KONE ? v : v / K;
}

// ---- mbarrier / TMA primitives (sm_90+ PTX) ----
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait for a phase: false if it did not complete within `polls`
// polls (each poll may suspend the thread for a short, system-dependent time)
__device__ __forceinline__ bool mbar_wait_n(uint64_t *bar, uint32_t parity, int polls)
{
    for (int i = 0; i < polls; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// the kernels' waits: 2^20 polls, far beyond any wait of a working step
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) { return mbar_wait_n(bar, parity, 1 << 20); }

__device__ __forceinline__ void tma_load_2d(void *dst, const void *desc, int c0, int c1, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"(desc), "r"(c0), "r"(c1), "r"(smem_u32(bar))
        : "memory");
}

// bytes (a multiple of 16, both addresses 16-byte aligned) global -> shared
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tma_load_3d(void *dst, const void *desc, int c0, int c1, int c2, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"(desc), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

// ===================================================================== palette
// For models whose 8 coefficient planes take at most MAX_PALETTE distinct
// values (patchy models: 2) each cell carries a one-byte material id and every
// per-cell coefficient the reference computes (co, c1, c2, rhof*eta/kappa,
// 1/co, 1/c1) comes from a table row in shared memory; other models (COEF)
// read the 8 coefficient planes per cell.
//
// Persistent, warp-specialised and double-buffered: one CTA per SM takes
// (model, shot, tile) items from the work list.  A producer warp runs one item
// ahead: it resolves the item's model and shot (a chain of dependent global
// loads that would otherwise stall every warp at each item), writes the
// item's parameters to shared memory, and fills the free buffer with five TMA
// copies (the 4 velocity planes and the 5 state planes with halos, one box
// each; the material ids; the two C-PML profile slices) and, for a batch item,
// a bulk copy of its material table.  Each copy costs the producer about 120
// cycles to issue, so the copies are few and large.  Eighteen compute warps
// (ten for 16-row tiles) compute the items from the buffers: a warp task is
// 32 consecutive columns (conflict-free shared-memory rows) of a band of 4
// consecutive rows, so the z-stencils of a column reuse the values of the
// rows before them in registers.  Stress: 9 bands x 2 halves cover the
// 64 x 36 stress cells; velocity: 8 bands x 2 halves cover the 60 x 32 tile,
// while the remaining two warps record the tile's receivers.  The warps may run one item ahead
// of each other.  (Splitting them into two groups of 9 that each own one
// buffer and alternate items, so that one group's mid-item barrier overlaps
// the other's work, measured 20 % slower: each group then waits for its own
// buffer's copies.)  Buffers are handed over with mbarriers (full: producer
// -> compute, empty: compute -> producer); every wait is bounded.
constexpr int ROWS = 4;                            // consecutive rows per compute task
constexpr int QX = PAL_TX;                         // 60 output columns
constexpr int IW = PAL_IDS_W;                      // ids: column x0-4 at (x0 & 15)
constexpr int PXW = TMA_VW;                        // x profile slice: x0-4 .. x0+63
constexpr int RING = 4;                            // MS: producer -> publisher ring slots
// The geometry of a tile of TZ rows (60 x 32: every variant; 60 x 16: the
// FAST single-model variants).  Shared memory per buffer: the 4 velocity
// planes (68 x TZ+8), the 5 state planes (68 x TZ+4), the material ids
// (80 x TZ+5 bytes), the two profile slices (6 x 68 and 6 x TZ+8 floats), a
// material table, the item's parameters and (batch) its model descriptor.
template <int TZ>
struct Geo {
    static constexpr int QZ = TZ;                              // output rows
    static constexpr int NST = 2 * ((QZ + 4) / ROWS);          // stress tasks: (TZ+4)/4 bands x 2 halves
    static constexpr int NVT = 2 * (QZ / ROWS);                // velocity tasks: TZ/4 bands x 2 halves
    static constexpr int PCT = 32 * NST;                       // compute threads: one stress task per warp
    static constexpr int PNT = PCT + 32;                       // + the producer warp
    static constexpr int IH = TZ + 5;                          // id rows z0-2 .. z0+TZ+2
    static constexpr int PV_FLOATS = TMA_VW * (TZ + 8);        // per velocity plane
    static constexpr int PS_BOX = TMA_VW * (TZ + 4);           // delivered per state plane
    static constexpr int PS_FLOATS = PS_BOX;                   // slot stride: the 5 slots are one dense TMA box
    static constexpr int PZH = TZ + 8;                         // z profile slice: z0-4 .. z0+TZ+3
    static constexpr int BUF_OFF_S = 4 * PV_FLOATS * 4;
    static constexpr int BUF_OFF_I = (BUF_OFF_S + 5 * PS_FLOATS * 4 + 127) / 128 * 128;
    static constexpr int BUF_OFF_PX = BUF_OFF_I + (IW * IH + 127) / 128 * 128;
    static constexpr int BUF_OFF_PZ = BUF_OFF_PX + (6 * PXW * 4 + 127) / 128 * 128;
    static constexpr int BUF_OFF_T = BUF_OFF_PZ + (6 * PZH * 4 + 127) / 128 * 128;
    static constexpr int BUF_OFF_M = BUF_OFF_T + MAX_PALETTE * MT_W * 4;
    static constexpr int BUF_OFF_MD = BUF_OFF_M + 128;
    static constexpr int BUF_BYTES = (BUF_OFF_MD + (int)sizeof(ModelDev) + 127) / 128 * 128;
    static constexpr int PAL_OFF_B = 2 * BUF_BYTES;            // mbarriers and counters
    static constexpr int PAL_OFF_R = PAL_OFF_B + 64;           // MS: the producer -> publisher ring
    static constexpr size_t PAL_SMEM = PAL_OFF_R + 128;
    // every box arrives whole (out-of-range parts zero-filled): 9 state boxes, ids, profile slices
    static constexpr uint32_t PAL_TX_BYTES =
        4 * PV_FLOATS * 4 + 5 * PS_BOX * 4 + IW * IH + 6 * PXW * 4 + 6 * PZH * 4;
    static_assert((QZ + 4) % ROWS == 0 && QZ % ROWS == 0 && NST > NVT, "task grid");
    static_assert(PV_FLOATS == TMA_VW * tile_vh(TZ) && PS_BOX == TMA_VW * tile_sh(TZ) && IH == tile_ids_h(TZ),
                  "the boxes the host encodes");
    static_assert(BUF_OFF_S % 128 == 0 && BUF_OFF_I % 128 == 0 && BUF_BYTES % 128 == 0, "TMA smem alignment");
    static_assert(BUF_OFF_PX % 128 == 0 && BUF_OFF_PZ % 128 == 0 && BUF_OFF_T % 16 == 0 && BUF_OFF_MD % 16 == 0,
                  "TMA and bulk-copy destinations");
    static_assert(PXW % 4 == 0 && PZH % 4 == 0 && IW % 16 == 0 && IW >= 12 + 4 + 64 && PAL_SMEM <= 232448,
                  "16-byte box rows; the id box covers x0-4 .. x0+63 from any 16-byte start; shared memory budget");
};
// state slots in shared memory; after the stress phase they hold its outputs
// (the planes SF_SXZ .. SF_XI2 in order: one TMA box of depth 5 fills them)
enum { PS_SXZ = 0, PS_G11, PS_G22, PS_XI1, PS_XI2 };
static_assert(SF_VX + 1 == SF_VZ && SF_VZ + 1 == SF_WX && SF_WX + 1 == SF_WZ && SF_SXZ + 1 == SF_G11 &&
                  SF_G11 + 1 == SF_G22 && SF_G22 + 1 == SF_XI1 && SF_XI1 + 1 == SF_XI2,
              "velocity planes and stress-state planes are consecutive in the state array");
enum { PO_SXX = PS_G11, PO_SZZ = PS_G22, PO_P = PS_XI1, PO_SXZ = PS_SXZ };

// Global accesses through the pointers the producer resolved for an item
// (read back from shared memory, so the compiler sees generic pointers):
// stated as global, they take the global path and are not taken for possible
// writes to the shared-memory tile, so later tile reads need not wait for them.
__device__ __forceinline__ void gst(float *p, float v) { __stwb(p, v); }
__device__ __forceinline__ float gld(const float *p) { return __ldca(p); }
// data no thread writes during the launch (the previous step's stress C-PML
// memory): non-coherent loads, which the compiler may issue ahead of earlier
// stores since they cannot alias them
__device__ __forceinline__ float gld_ro(const float *p) { return __ldg(p); }

// Step-spanning launches (MS): the C-PML memory a tile reads was written by
// other CTAs of the same launch at the previous step, so it is read through
// L2 only (this SM's L1 could still hold a line of an older step) and
// prefetched to L2; one launch per step reads it as above.
template <bool MS>
__device__ __forceinline__ float gld_m(const float *p)
{
    return MS ? __ldcg(p) : gld(p);
}
template <bool MS>
__device__ __forceinline__ float gld_ro_m(const float *p)
{
    return MS ? __ldcg(p) : gld_ro(p);
}
template <bool MS>
__device__ __forceinline__ void prefetch_m(const float *p)
{
    if (MS) asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
    else asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}
// a tile flag of a step-spanning launch: read with acquire, published with
// release, both at GPU scope
__device__ __forceinline__ int ld_acquire(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int *p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// orders generic-proxy global accesses against later async-proxy (TMA) ones
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }
// a CTA-scope counter in shared memory: added to with release, read with acquire
__device__ __forceinline__ void red_add_release_cta(int *p, int v)
{
    asm volatile("red.release.cta.shared::cta.add.s32 [%0], %1;" ::"r"(smem_u32(p)), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_acquire_cta(const int *p)
{
    int v;
    asm volatile("ld.acquire.cta.shared::cta.b32 %0, [%1];" : "=r"(v) : "r"(smem_u32(p)) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_cta(int *p, int v)
{
    asm volatile("st.release.cta.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(p)), "r"(v) : "memory");
}
// the warp waits until every lane's flag (a lane with a null flag watches
// none) reads at least want, each lane polling its own with ld.acquire.gpu;
// false when the flags still fall short after `polls` rounds (bounded)
__device__ __forceinline__ bool wait_flags(const int *flag, int want, int polls)
{
    bool ok = flag == nullptr;
    for (int poll = 0;; ++poll) {
        if (!ok) ok = ld_acquire(flag) >= want;
        if (__all_sync(0xffffffffu, ok)) return true;
        if (poll >= polls) return false;
    }
}

// new w and v of one cell from its coefficient planes (c at the cell, planes
// pl apart), with the reference's float operations in its order (cu:293-311,
// 330-353): co = (rho m - rhof^2)/dt, c1,2 = co +- rho (eta/kappa)/2
__device__ __forceinline__ void velocity_coef(const float *__restrict__ c, int64_t pl, float dt, float A, float B,
                                              float w0, float v0, float &w1, float &v1)
{
    const float rho = gld(c + C_RHO * pl), rhof = gld(c + C_RHOF * pl);
    const float rsm = gld(c + C_RSM * pl), eok = gld(c + C_EOK * pl);
    const float co = (rho * rsm - rhof * rhof) / dt;
    const float c1 = co + rho * eok * 0.5f;
    const float c2 = co - rho * eok * 0.5f;
    w1 = (c2 * w0 + (-rhof * A - rho * B)) / c1;
    v1 = v0 + (rsm * A + rhof * B + rhof * eok * ((w0 + w1) * 0.5f)) / co;
}

// what the producer resolves for one item (shared memory, per buffer)
struct ItemMeta {
    float *FB;                 // state buffer written by this step
    const float *mxr, *mzr;    // stress C-PML memory read / written by this step
    float *mxw, *mzw;
    float *mxv, *mzv;          // velocity C-PML memory (in place)
    float *acc_w;              // sigma2 at the source cell, written
    float *trace_row;          // this step's trace row, or null
    const int4 *rec;           // receivers of this tile
    int nrec_q;
    int src_off, src_where, src_on;
    float src_val, pacc;
    int x0, z0, interior;
    int g;                     // the item's index in the launch; -1: the work list has ended
};
static_assert(sizeof(ItemMeta) <= 128, "item parameters fit their slot");

// add bytes to the current phase's transaction count without arriving
__device__ __forceinline__ void mbar_expect_tx_only(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// orders this thread's generic-proxy shared-memory accesses before later
// async-proxy (TMA) writes to the same buffer
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// barrier 1: every compute warp (NT compute threads)
template <int NT>
__device__ __forceinline__ void compute_sync() { asm volatile("bar.sync 1, %0;" ::"n"(NT) : "memory"); }
// the same barrier, returning whether v held in every compute thread
template <int NT>
__device__ __forceinline__ bool compute_sync_and(bool v)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, 1, %2, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)v), "n"(NT)
        : "memory");
    return r != 0;
}

}  // namespace tile

// Work queue: the CTAs take the launch's items in order from one counter
// (queue[0]; queue[1] counts the CTAs that found it exhausted, and the last
// of them sets both back to 0 for the next launch), so the tiles that run at
// the same time are neighbours in the work list however long the launch
// (their halos meet in L2) and a CTA that drew heavy tiles simply takes
// fewer.  Tiles are independent within a step: the results do not depend on
// which CTA computes which tile.
//
// MS (step-spanning launch): the launch runs steps k .. k+nk-1 and walks
// (step, tile) items step by step: item g is tile g % nitems of step
// k + g / nitems.  Before the producer fills a buffer with a tile of step n it
// waits until the tile's 3 x 3 neighbourhood (the cells its boxes read, and
// the readers of the buffer it will overwrite) has completed step n-1, by
// the shots' done flags; a publisher warp publishes each of the CTA's tiles
// once the compute warps have released its buffer, whatever the producer is
// waiting for.  A producer only ever waits for items of the previous step,
// which were taken from the queue before its own, and a CTA issues its items
// in the order it takes them; the first step of a launch waits for none, so
// by induction on the step every item is issued and finishes: the waits
// cannot close a cycle.  Without MS (nk = 1) no tile waits for another.
template <int SM, bool KONE, bool MULTI, bool COEF, bool MS, int TZ>
__global__ void __launch_bounds__(tile::Geo<TZ>::PNT + (MS ? 32 : 0), 1)
k_tile_pal(const ModelDev mp, const ModelDev *__restrict__ models, const StreamShot *__restrict__ shots,
           const int4 *__restrict__ items, int nitems, int k, int nk, int prefetch, int *__restrict__ queue)
{
    using namespace tile;
    using G = Geo<TZ>;
    constexpr int QZ = G::QZ, NST = G::NST, NVT = G::NVT, PCT = G::PCT, IH = G::IH;
    constexpr int PV_FLOATS = G::PV_FLOATS, PS_BOX = G::PS_BOX, PS_FLOATS = G::PS_FLOATS, PZH = G::PZH;
    constexpr int BUF_OFF_S = G::BUF_OFF_S, BUF_OFF_I = G::BUF_OFF_I, BUF_OFF_PX = G::BUF_OFF_PX;
    constexpr int BUF_OFF_PZ = G::BUF_OFF_PZ, BUF_OFF_T = G::BUF_OFF_T, BUF_OFF_M = G::BUF_OFF_M;
    constexpr int BUF_OFF_MD = G::BUF_OFF_MD, BUF_BYTES = G::BUF_BYTES;
    constexpr int PAL_OFF_B = G::PAL_OFF_B, PAL_OFF_R = G::PAL_OFF_R;
    constexpr uint32_t PAL_TX_BYTES = G::PAL_TX_BYTES;
    (void)PS_BOX;
    (void)IH;
    constexpr bool EXACT = SM != SM_FAST;
    constexpr int NW = PCT / 32;             // compute warps: one stress task each
    static_assert(NST == NW && NW > NVT, "one stress task per warp; velocity warps, then receiver warps");
    extern __shared__ __align__(128) unsigned char smp[];
    uint64_t *full = reinterpret_cast<uint64_t *>(smp + PAL_OFF_B);
    uint64_t *empty = full + 2;
    // MS: compute-warp releases of each buffer, counted (monotonic, so the
    // publisher may lag behind the buffer's reuse without losing count)
    int *released = reinterpret_cast<int *>(full + 4);
    // MS: the producer hands each item's tile flag and step to the publisher
    // through a ring of RING slots (slot j % RING holds item j once its
    // sequence number reads j + 1; a null flag ends the list), and refills a
    // slot only after the publisher has taken its previous item (published)
    int *published = released + 2;
    int **ring_flag = reinterpret_cast<int **>(smp + PAL_OFF_R);
    int *ring_val = reinterpret_cast<int *>(ring_flag + RING);
    int *ring_seq = ring_val + RING;
    const int tid = threadIdx.x;
    // the error flag for a failure no item can be named for (read where needed)
    auto err0 = [&]() { return MULTI ? models[0].err : mp.err; };

    if (tid == 0) {
        for (int b = 0; b < 2; ++b) {
            mbar_init(&full[b], 1);
            mbar_init(&empty[b], NW);
            released[b] = 0;
        }
        *published = 0;
        for (int r = 0; r < RING; ++r) ring_seq[r] = 0;
        mbar_fence_init();
    }
    __syncthreads();

    const int total = MS ? nk * nitems : nitems;   // items of this launch

    // ------------------------------------------------------------ publisher (MS)
    // Publishes each item's tile flag once all compute warps have released its
    // buffer: a warp of its own, off the path from a buffer's release to its
    // refill, so neither the producer's copies nor its waits for other tiles
    // hold it up, and it holds up neither.
    if (MS && tid >= PCT + 32) {
        if (tid != PCT + 32) return;
        // polls sleep between reads: this warp shares its SM's issue slots with
        // the compute warps, and a tile's flag is needed only steps later
        for (int j = 0;; ++j) {
            const int r = j % RING;
            int poll = 0;
            while (ld_acquire_cta(&ring_seq[r]) != j + 1) {
                if (++poll > (1 << 22)) {
                    atomicExch(err0(), 1);
                    return;
                }
                __nanosleep(128);
            }
            int *flag = ring_flag[r];
            const int nval = ring_val[r];
            st_release_cta(published, j + 1);   // slot r may be refilled
            if (!flag) return;
            const int b = j & 1;
            const int want = NW * ((j >> 1) + 1);   // releases of buffer b once item j is done
            poll = 0;
            while (ld_acquire_cta(&released[b]) < want) {
                if (++poll > (1 << 22)) {
                    atomicExch(err0(), 1);
                    return;
                }
                __nanosleep(128);
            }
            // the compute warps' global stores, acquired through the counter, are
            // released with the flag (to generic and TMA readers)
            fence_proxy_async_global();
            st_release(flag, nval);
        }
    }

    // ------------------------------------------------------------ producer
    if (tid >= PCT) {   // (the warp after the compute warps)
        const int lane = tid - PCT;
        int j = 0;
        bool gave_up = false;
        // ring slot j % RING for item j (MS, lane 0), once the publisher has taken item j - RING
        auto ring_put = [&](int jj, int *flag, int val) -> bool {
            const int r = jj % RING;
            for (int poll = 0; ld_acquire_cta(published) < jj - RING + 1; ++poll)
                if (poll >= (1 << 20)) return false;
            ring_flag[r] = flag;
            ring_val[r] = val;
            st_release_cta(&ring_seq[r], jj + 1);
            return true;
        };
        int gnext = lane == 0 ? atomicAdd(queue, 1) : 0;
        for (;; ++j) {
            const int g = __shfl_sync(0xffffffffu, gnext, 0);
            if (g >= total) break;
            if (lane == 0) gnext = atomicAdd(queue, 1);   // the next item, fetched while this one is set up
            const int b = j & 1;
            const int w = MS ? g % nitems : g;
            const int kk = MS ? k + g / nitems : k;
            // Resolve the item (a chain of dependent global loads) while buffer b
            // is still being computed on, so the copies start the moment it frees.
            const int4 it = items[w];
            const ModelDev &m = MULTI ? models[it.x] : mp;
            const StreamShot &S = shots[it.y];
            const int x0 = it.z, z0 = it.w;
            const int P = m.P;
            ItemMeta M;
            const void *tm_v = nullptr, *tm_s = nullptr;
            int cv = 0;
            int64_t n = 0;
            if (lane == 0) {
                n = *S.step + kk + 1;
                const int rd = (int)((n - 1) & 1), wr = (int)(n & 1);
                M.FB = S.f[wr];
                M.mxr = S.mx[rd];
                M.mxw = S.mx[wr];
                M.mzr = S.mz[rd];
                M.mzw = S.mz[wr];
                M.mxv = S.mxv;
                M.mzv = S.mzv;
                M.acc_w = S.acc + wr;
                M.pacc = __ldcg(S.acc + rd);   // written at the previous step, maybe by another CTA
                M.src_off = (int)S.src_off;
                M.src_where = S.src_where;
                M.src_on = n <= S.src_n;
                M.src_val = n <= S.src_n ? S.src_tab[n - 1] : 0.0f;
                const bool rec_on = S.nrec > 0 && n <= S.trace_cap;
                const int tile = (z0 / QZ) * m.ntx + x0 / QX;
                const int qb = rec_on ? S.rec_start[tile] : 0, qe = rec_on ? S.rec_start[tile + 1] : 0;
                M.rec = S.rec_sorted + qb;
                M.nrec_q = qe - qb;
                M.trace_row = rec_on ? S.trace + (n - 1) * S.nrec : nullptr;
                M.x0 = x0;
                M.z0 = z0;
                M.g = g;
                // interior: no grid edge, C-PML strip or source within the tile and its halo
                int sx = -1000000, sz = -1000000;
                if (S.src_off >= 0) {
                    sz = (int)(S.src_off / P) - ZH;
                    sx = (int)(S.src_off - (int64_t)(sz + ZH) * P) - XH;
                }
                const int xa = x0 - 2, xb = x0 + QX + 1, za = z0 - 2, zb = z0 + QZ + 1;
                M.interior = xa >= 2 && xa >= m.xL && xb <= m.NX - 2 && xb < m.xR && za >= 2 && za >= m.zT &&
                             zb <= m.NZ - 2 && zb < m.zB && !(sx >= xa && sx <= xb && sz >= za && sz <= zb);
                tm_v = S.tm_v;
                tm_s = S.tm_s;
                cv = rd * NSF;
            }
            // what the fills below need from the model, read now: past the wait
            // (a compiler barrier) a batch item's descriptor would be re-read from
            // global memory on the copies' critical path
            const void *m_tmi = m.tm_ids, *m_tmx = m.tm_px, *m_tmz = m.tm_pz;
            const float *m_mtab = m.mtab;
            const int m_nmat = m.nmat;
            // batch items: this lane's words of the model descriptor, read now
            constexpr int MDW = (int)(sizeof(ModelDev) / 4);
            static_assert(MDW <= 64, "two descriptor words per producer lane");
            uint32_t md0 = 0, md1 = 0;
            if (MULTI) {
                const uint32_t *msrc = reinterpret_cast<const uint32_t *>(&m);
                if (lane < MDW) md0 = msrc[lane];
                if (lane + 32 < MDW) md1 = msrc[lane + 32];
            }
            if (MS) {
                // the 3 x 3 neighbourhood of the tile must have completed step n-1:
                // lane l < 9 watches the tile (tx + l % 3 - 1, tz + l / 3 - 1).  The
                // launch's first step waits for none: the previous launch ended
                // (the flags may lag behind the shot, never lead it).
                const int nn = __shfl_sync(0xffffffffu, (int)n, 0);
                const int tx = x0 / QX, tz = z0 / QZ, ntx = m.ntx, ntz = m.ntz;
                const int ux = tx + lane % 3 - 1, uz = tz + lane / 3 - 1;
                const int *flag = (kk > k && lane < 9 && ux >= 0 && ux < ntx && uz >= 0 && uz < ntz)
                                      ? S.done + uz * ntx + ux
                                      : nullptr;
                if (!wait_flags(flag, nn - 1, 1 << 20)) gave_up = true;
                if (gave_up) {
                    if (lane == 0) atomicExch(mp.err ? mp.err : models[it.x].err, 1);
                    break;
                }
                // lanes 0-8 acquired the flags, lane 0 issues the copies: the warp
                // barrier orders the one after the other
                __syncwarp();
                // the item's tile flag and step, for the publisher
                if (lane == 0 && !ring_put(j, S.done + (z0 / QZ) * m.ntx + x0 / QX, (int)nn)) gave_up = true;
                if (__shfl_sync(0xffffffffu, (int)gave_up, 0)) {
                    if (lane == 0) atomicExch(mp.err ? mp.err : models[it.x].err, 1);
                    gave_up = true;
                    break;
                }
            }
            // buffer b free again: released by the compute warps
            if (j >= 2 && !mbar_wait(&empty[b], (uint32_t)(((j - 2) >> 1) & 1))) {
                if (lane == 0) atomicExch(mp.err ? mp.err : models[it.x].err, 1);
                gave_up = true;
                break;
            }
            unsigned char *buf = smp + b * BUF_BYTES;
            if (lane == 0) {
                if (MS && kk > k) fence_proxy_async_global();   // the neighbours' stores, acquired above, before the copies
                // the big copies first: the 4 velocity planes with a 4-cell halo and
                // the 5 state planes with a 2-row halo, one box each (bytes
                // announced, no arrival yet)
                const uint32_t tab_bytes = (MULTI && !COEF) ? (uint32_t)(m_nmat * MT_W * 4) : 0u;
                mbar_expect_tx_only(&full[b], PAL_TX_BYTES - (COEF ? (uint32_t)(IW * IH) : 0u) + tab_bytes);
                tma_load_3d(buf, tm_v, x0, z0, cv + SF_VX, &full[b]);
                tma_load_3d(buf + BUF_OFF_S, tm_s, x0, z0 + 2, cv + SF_SXZ, &full[b]);
                // ids from padded column x0 (grid x0-4) rounded down to 16 bytes,
                // rows from padded z0+2 (grid z0-2); profile slices from padded
                // x0 / z0 (grid x0-4 / z0-4), all 6 rows
                if (!COEF) tma_load_2d(buf + BUF_OFF_I, m_tmi, x0 & ~15, z0 + 2, &full[b]);
                tma_load_2d(buf + BUF_OFF_PX, m_tmx, x0, 0, &full[b]);
                tma_load_2d(buf + BUF_OFF_PZ, m_tmz, z0, 0, &full[b]);
                if (MULTI && !COEF) bulk_load(buf + BUF_OFF_T, m_mtab, tab_bytes, &full[b]);
            }
            if (MULTI) {
                // the model descriptor, for the compute warps
                uint32_t *mdst = reinterpret_cast<uint32_t *>(buf + BUF_OFF_MD);
                if (lane < MDW) mdst[lane] = md0;
                if (lane + 32 < MDW) mdst[lane + 32] = md1;
            }
            // every lane's descriptor words are written before lane 0's arrival,
            // the phase's only one, can complete it
            __syncwarp();
            if (lane == 0) {
                *reinterpret_cast<ItemMeta *>(buf + BUF_OFF_M) = M;
                mbar_arrive(&full[b]);
            }
            __syncwarp();
        }
        // the end of the work list, as item j of the buffers: once buffer j & 1 is
        // free (its fill j - 2 then landed too), its parameters say so (and, MS,
        // so does the ring)
        int drain_from = j - 2;
        if (!gave_up) {
            const int b = j & 1;
            if (j >= 2 && !mbar_wait(&empty[b], (uint32_t)(((j - 2) >> 1) & 1))) {
                if (lane == 0) atomicExch(err0(), 1);
            } else {
                drain_from = j - 1;
                if (lane == 0) {
                    reinterpret_cast<ItemMeta *>(smp + b * BUF_BYTES + BUF_OFF_M)->g = -1;
                    if (MS && !ring_put(j, nullptr, 0)) atomicExch(err0(), 1);
                    mbar_arrive(&full[b]);
                }
            }
        }
        // the last CTA to find the queue exhausted sets it back for the next launch
        if (lane == 0) {
            __threadfence();
            if (atomicAdd(queue + 1, 1) == (int)gridDim.x - 1) {
                __threadfence();
                atomicExch(queue, 0);
                atomicExch(queue + 1, 0);
            }
        }
        // copies in flight land before the CTA may exit
        for (int i = drain_from < 0 ? 0 : drain_from; i < j; ++i) mbar_wait(&full[i & 1], (uint32_t)((i >> 1) & 1));
        return;
    }

    // ------------------------------------------------------------ compute
    const int wid = tid >> 5, lane = tid & 31;
    // this warp's stress task, which is also its velocity task if wid < NVT:
    // column lx of the 64-wide stress tile, rows zb0 .. zb0+3
    const int lx = (wid & 1) * 32 + lane, zb0 = (wid >> 1) * ROWS;
    if (!MULTI) {
        // single model: one material table for every item, in buffer 0's slot
        float *t0 = reinterpret_cast<float *>(smp + BUF_OFF_T);
        for (int i = tid; i < mp.nmat * MT_W; i += PCT) t0[i] = mp.mtab[i];
        compute_sync<PCT>();
    }
    for (int j = 0;; ++j) {
        const int b = j & 1;
        unsigned char *buf = smp + b * BUF_BYTES;
        // No barrier here: warps run ahead into the item as soon as its data
        // has landed.  A wait that gave up leaves the buffer's contents (item
        // parameters included) untrusted: touch nothing, join the item's
        // mid-point barrier, which then ends every compute thread together.
        if (!mbar_wait(&full[b], (uint32_t)((j >> 1) & 1))) {
            compute_sync_and<PCT>(false);
            if (tid == 0) atomicExch(err0(), 1);
            return;
        }
        if (reinterpret_cast<const ItemMeta *>(buf + BUF_OFF_M)->g < 0) break;   // every compute warp ends here
        const ModelDev &m = MULTI ? *reinterpret_cast<const ModelDev *>(buf + BUF_OFF_MD) : mp;
        // the stencil divisors in registers: the model descriptor of a batch item
        // sits in shared memory, where the loops' own stores would force re-reads
        const Div24 qx = m.qx, qz = m.qz;
        const ItemMeta &IM = *reinterpret_cast<const ItemMeta *>(buf + BUF_OFF_M);
        const float *st = reinterpret_cast<const float *>(MULTI ? buf + BUF_OFF_T : smp + BUF_OFF_T);
        // COEF: the 8 coefficient planes, read per cell (padded like the state: zero outside the grid)
        const float *__restrict__ cf = m.coef;
        const float *PXs = reinterpret_cast<const float *>(buf + BUF_OFF_PX);
        const float *PZs = reinterpret_cast<const float *>(buf + BUF_OFF_PZ);
        const int NX = m.NX, NZ = m.NZ;
        const int P = m.P;
        const int64_t PL = m.plane;
        const float dt = m.dt;
        const int Wx = m.Wx, nzx = (NZ + 1) * m.Wx, hzp = m.Hz * P;
        const int x0 = IM.x0, z0 = IM.z0;
        float *__restrict__ FB = IM.FB;
        const int src_off = IM.src_off;
        const int src_where = IM.src_where;
        const bool src_on = IM.src_on != 0;
        const float src_val = IM.src_val;
        const float pacc = IM.pacc;
        float *sv = reinterpret_cast<float *>(buf);                 // 4 x 40 x 68, from (x0-4, z0-4)
        float *ss = reinterpret_cast<float *>(buf + BUF_OFF_S);     // 5 x 36 x 68, from (x0-4, z0-2)
        const uint8_t *si = buf + BUF_OFF_I + (x0 & 15);            // 37 x 80,     from (x0-4, z0-2)

        // Interior tiles (no grid edge, C-PML strip or source within the tile
        // and its halo) take a copy of the code with every guard constant-true.
        auto compute = [&](auto interior_tag) -> bool {
            constexpr bool IN = decltype(interior_tag)::value;
            // v + m for a C-PML memory term m.  In interior tiles every m is an
            // exact zero; with FAST stencils the addition is skipped there (it
            // could only turn a -0 into +0), EXACT keeps the reference's sum.
            auto addm = [](float v, float mv) { return (SM == SM_FAST && IN) ? v : v + mv; };
            // The velocity C-PML memory this thread updates in place after the
            // barrier (rows zb0 .. zb0+3 of column lx, on the strips), to L1.  A
            // single model's per-step launch prefetches it just before the
            // barrier, while the other warps finish their stress rows: prefetched
            // at the tile start together with the stress phase's memory it
            // overflows the L1 that the tile buffers leave (about 28 KB beside
            // 205 KB of shared memory).  The batch kernel prefetches it at the
            // tile start, where it spills no registers, and so does a
            // step-spanning launch, whose prefetches go to L2 (+0.3 %).
            auto prefetch_velocity_memory = [&]() {
                if (IN || !prefetch || wid >= NVT || lx >= QX || x0 + lx > NX) return;
                const int x = x0 + lx;
                const int xc = xcol(m, x);
#pragma unroll
                for (int r = 0; r < ROWS; ++r) {
                    const int tz = z0 + zb0 + r;
                    if (tz > NZ) break;
                    const int zr = zrow(m, tz);
                    if (xc >= 0)
#pragma unroll
                        for (int a = 0; a < 3; ++a)
                            prefetch_m<MS>(IM.mxv + a * nzx + tz * Wx + xc);
                    if (zr >= 0)
#pragma unroll
                        for (int a = 0; a < 3; ++a)
                            prefetch_m<MS>(IM.mzv + a * hzp + zr * P + x + XH);
                }
            };
            if (MULTI || MS) prefetch_velocity_memory();
            if (COEF && wid < NVT && lx < QX) {
                // the density coefficients this thread's velocity rows read (rows
                // zb0 .. zb0+4 of column lx): to L1 now, read after the stress phase
                const float *c = cf + (int64_t)(z0 + zb0 + ZH) * P + x0 + lx + XH;
#pragma unroll
                for (int r = 0; r < ROWS + 1; ++r)
#pragma unroll
                    for (int pl = C_RHO; pl <= C_EOK; ++pl)
                        asm volatile("prefetch.global.L1 [%0];" ::"l"(c + pl * PL + (int64_t)r * P));
            }
            if (!IN && prefetch && x0 - 2 + lx >= 0 && x0 - 2 + lx <= NX) {
                // the stress C-PML memory of this thread's stress rows: to L1 before
                // the first row needs it
                const int x = x0 - 2 + lx;
                const int xc = xcol(m, x);
#pragma unroll
                for (int r = 0; r < ROWS; ++r) {
                    const int z = z0 - 2 + zb0 + r;
                    if (z < 0 || z > NZ) continue;
                    const int zr = zrow(m, z);
                    if (xc >= 0)
#pragma unroll
                        for (int a = 0; a < 3; ++a)
                            prefetch_m<MS>(IM.mxr + a * nzx + z * Wx + xc);
                    if (zr >= 0)
#pragma unroll
                        for (int a = 0; a < 3; ++a)
                            prefetch_m<MS>(IM.mzr + a * hzp + zr * P + x + XH);
                }
            }
            // ---- stress on the tile + 2-cell halo: column lx, rows zb0 .. zb0+3
            {
                const int x = x0 - 2 + lx;
                const bool x_ok = IN || (x >= 0 && x <= NX);
                const bool x_g1 = IN || (x >= 1 && x <= NX - 1), x_g2 = IN || (x >= 2 && x <= NX - 1);
                const bool x_g3 = IN || (x >= 1 && x <= NX - 2);
                const bool x_own = x_ok && lx >= 2 && lx < QX + 2;
                const int xc = (!IN && x_ok) ? xcol(m, x) : -1;
                const int xi = x + XH;
                const int pxo = lx + 2;                          // x in the profile slice
                const float bxh = PXs[PBH * PXW + pxo], axh = PXs[PAH * PXW + pxo];
                const float bx = PXs[PB * PXW + pxo], ax = PXs[PA * PXW + pxo];
                const float Kxh = KONE ? 1.0f : PXs[PKH * PXW + pxo];
                const float Kx = KONE ? 1.0f : PXs[PK * PXW + pxo];
                // this column's values along z, shared by the 4 rows' z-stencils:
                // vz, wz at velocity-tile rows zb0 .. zb0+6, vx at rows zb0+1 .. zb0+7
                const float *VXc = sv + 0 * PV_FLOATS + lx + 2, *VZc = sv + 1 * PV_FLOATS + lx + 2;
                const float *WXc = sv + 2 * PV_FLOATS + lx + 2, *WZc = sv + 3 * PV_FLOATS + lx + 2;
                float vzc[ROWS + 3], wzc[ROWS + 3], vxc[ROWS + 3];
                uint8_t idc[ROWS + 1];
#pragma unroll
                for (int r = 0; r < ROWS + 3; ++r) {
                    vzc[r] = VZc[(zb0 + r) * TMA_VW];
                    wzc[r] = WZc[(zb0 + r) * TMA_VW];
                    vxc[r] = VXc[(zb0 + 1 + r) * TMA_VW];
                }
#pragma unroll
                for (int r = 0; r < ROWS + 1; ++r) idc[r] = COEF ? 0 : si[(zb0 + r) * IW + lx + 2];
#pragma unroll
                for (int r = 0; r < ROWS; ++r) {
                    const int zl = zb0 + r;
                    const int z = z0 - 2 + zl;
                    const int pzo = zl + 2;                      // z in the profile slice
                    const int vr = (zl + 2) * TMA_VW;            // row of the velocity tile
                    const int so = zl * TMA_VW + lx + 2;         // in the state tile
                    const bool z_ok = IN || (z >= 0 && z <= NZ);
                    const bool cell_ok = x_ok && z_ok;
                    const bool g1 = IN || (cell_ok && x_g1 && z >= 2 && z <= NZ - 2);   // cu:60-62
                    const bool g2 = IN || (cell_ok && x_g2 && z >= 1 && z <= NZ - 2);   // cu:212-214
                    const bool g3 = IN || (cell_ok && x_g3 && z >= 2 && z <= NZ - 1);   // cu:237-239
                    const bool own = x_own && z_ok && zl >= 2 && zl < QZ + 2;
                    const int o = (z + ZH) * P + xi;
                    const float vdx = D4<SM>(VXc[vr + 1], vxc[r + 1], VXc[vr + 2], VXc[vr - 1], qx);
                    const float vdz = D4<SM>(vzc[r + 2], vzc[r + 1], vzc[r + 3], vzc[r], qz);
                    const float wdx = D4<SM>(WXc[vr + 1], WXc[vr], WXc[vr + 2], WXc[vr - 1], qx);
                    const float wdz = D4<SM>(wzc[r + 2], wzc[r + 1], wzc[r + 3], wzc[r], qz);
                    const float sdx = D4<SM>(vzc[r + 2], VZc[vr - 1], VZc[vr + 1], VZc[vr - 2], qx);
                    const float sdz = D4<SM>(vxc[r + 2], vxc[r + 1], vxc[r + 3], vxc[r], qz);
                    float g11 = ss[PS_G11 * PS_FLOATS + so], g22 = ss[PS_G22 * PS_FLOATS + so];
                    float xi1 = ss[PS_XI1 * PS_FLOATS + so], xi2 = ss[PS_XI2 * PS_FLOATS + so];
                    float sxz = ss[PS_SXZ * PS_FLOATS + so];
                    float lc, mu, al, M, mu_top;
                    if (COEF) {
                        const float *c = cf + o;
                        lc = gld(c + C_LC * PL);
                        mu = gld(c + C_MU * PL);
                        al = gld(c + C_AL * PL);
                        M = gld(c + C_M * PL);
                        mu_top = gld(c + C_MU * PL + P);             // rmu[top] (cu:218)
                    } else {
                        const float4 ma = *reinterpret_cast<const float4 *>(st + MT_W * idc[r]);
                        mu_top = st[MT_W * idc[r + 1] + MT_MU];      // rmu[top] (cu:218)
                        lc = ma.x;
                        mu = ma.y;
                        al = ma.z;
                        M = ma.w;
                    }
                    const int zr = (!IN && z_ok) ? zrow(m, z) : -1;
                    float m1 = 0.0f, m2 = 0.0f, m3 = 0.0f, m4 = 0.0f, m5 = 0.0f, m6 = 0.0f;
                    if (xc >= 0 && (g1 || g2)) {
                        const int ix = z * Wx + xc;
                        const float *MA = IM.mxr;
                        m1 = bxh * gld_ro_m<MS>(MA + MXS_SXX * nzx + ix) + axh * vdx;
                        m3 = bxh * gld_ro_m<MS>(MA + MXS_S2 * nzx + ix) + axh * wdx;
                        m5 = bx * gld_ro_m<MS>(MA + MXS_SXZ * nzx + ix) + ax * sdx;
                        if (own) {
                            float *MB = IM.mxw;
                            if (g1) {
                                gst(MB + MXS_SXX * nzx + ix, m1);
                                gst(MB + MXS_S2 * nzx + ix, m3);
                            }
                            if (g2) gst(MB + MXS_SXZ * nzx + ix, m5);
                        }
                    }
                    if (zr >= 0 && (g1 || g2)) {
                        const int iz = zr * P + xi;
                        const float *MA = IM.mzr;
                        const float bz = PZs[PB * PZH + pzo], az = PZs[PA * PZH + pzo];
                        m2 = bz * gld_ro_m<MS>(MA + MZS_SXX * hzp + iz) + az * vdz;
                        m4 = bz * gld_ro_m<MS>(MA + MZS_S2 * hzp + iz) + az * wdz;
                        m6 = PZs[PBH * PZH + pzo] * gld_ro_m<MS>(MA + MZS_SXZ * hzp + iz) + PZs[PAH * PZH + pzo] * sdz;
                        if (own) {
                            float *MB = IM.mzw;
                            if (g1) {
                                gst(MB + MZS_SXX * hzp + iz, m2);
                                gst(MB + MZS_S2 * hzp + iz, m4);
                            }
                            if (g2) gst(MB + MZS_SXZ * hzp + iz, m6);
                        }
                    }
                    const float Kz = KONE ? 1.0f : PZs[PK * PZH + pzo];
                    if (g1) {   // cu:71-86
                        g11 = g11 + dt * addm(KDIV<KONE>(vdx, Kxh), m1);
                        g22 = g22 + dt * addm(KDIV<KONE>(vdz, Kz), m2);
                        xi1 = xi1 - addm(KDIV<KONE>(wdx, Kxh), m3) * dt;
                        xi2 = xi2 - addm(KDIV<KONE>(wdz, Kz), m4) * dt;
                    }
                    float pv = g1 ? (-al * M * (g11 + g22) + M * (xi1 + xi2)) : 0.0f;
                    const bool is_src = !IN && cell_ok && o == src_off;
                    if (is_src && !g1) pv = pacc;                    // sigma2 never overwritten there
                    if (is_src && src_where == SRC_P && src_on) pv = pv + src_val;   // cu:107-109
                    if (is_src && own) gst(IM.acc_w, pv);
                    if (g2) {   // cu:223-226
                        const float Ssum = addm(addm(KDIV<KONE>(sdx, Kx), m5) + KDIV<KONE>(sdz, Kz), m6);
                        sxz = EXACT ? sxz_exact(sxz, mu_top, Ssum, dt) : sxz_fast(sxz, mu_top, Ssum, dt);
                    }
                    float sxx = 0.0f, szz = 0.0f;
                    if (g3) {   // cu:241-242
                        if (EXACT) sxx_szz_exact(lc, mu, g11, g22, al, pv, sxx, szz);
                        else sxx_szz_fast(lc, mu, g11, g22, al, pv, sxx, szz);
                    }
                    if (own) {
                        gst(FB + SF_G11 * PL + o, g11);
                        gst(FB + SF_G22 * PL + o, g22);
                        gst(FB + SF_XI1 * PL + o, xi1);
                        gst(FB + SF_XI2 * PL + o, xi2);
                        gst(FB + SF_SXZ * PL + o, sxz);
                    }
                    // this thread alone reads these slots of this cell: outputs overwrite inputs
                    ss[PO_SXX * PS_FLOATS + so] = sxx;
                    ss[PO_SZZ * PS_FLOATS + so] = szz;
                    ss[PO_P * PS_FLOATS + so] = pv;
                    ss[PO_SXZ * PS_FLOATS + so] = sxz;
                }
            }
            if (!MULTI && !MS) prefetch_velocity_memory();
            if (!compute_sync_and<PCT>(true)) return false;   // false: a thread's wait for this item gave up

            if (wid >= NVT) {
                // ---- receivers of this tile (vx, vz before the update; p of this step)
                if (IM.nrec_q > 0) {
                    float *trace_row = IM.trace_row;
                    for (int q = tid - 32 * NVT; q < IM.nrec_q; q += PCT - 32 * NVT) {
                        const int4 Rq = IM.rec[q];               // (x, comp, slot, z)
                        const int xl = Rq.x - x0, zl = Rq.w - z0;
                        float v;
                        if (Rq.y == 2) v = ss[PO_P * PS_FLOATS + (zl + 2) * TMA_VW + xl + 4];
                        else v = sv[(Rq.y == 0 ? 0 : 1) * PV_FLOATS + (zl + 4) * TMA_VW + xl + 4];
                        gst(trace_row + Rq.z, v);
                    }
                }
                return true;
            }
            // ---- velocity on the tile: column lx (< 60), rows zb0 .. zb0+3
            float *__restrict__ MXV = IM.mxv;
            float *__restrict__ MZV = IM.mzv;
            if (lx < QX) {
                const int x = x0 + lx;
                const bool x_in = IN || x <= NX;
                const bool x_vx = IN || (x >= 2 && x <= NX - 1), x_vz = IN || (x >= 1 && x <= NX - 2);   // cu:289, 326
                const int xc = (!IN && x_in) ? xcol(m, x) : -1;
                const int xi = x + XH;
                const int pxo = lx + 4;
                const float bx = PXs[PB * PXW + pxo], ax = PXs[PA * PXW + pxo];
                const float bxh = PXs[PBH * PXW + pxo], axh = PXs[PAH * PXW + pxo];
                const float Kx = KONE ? 1.0f : PXs[PK * PXW + pxo], Kxh = KONE ? 1.0f : PXs[PKH * PXW + pxo];
                // this column's stress values along z: sxz at stress-tile rows
                // zb0 .. zb0+6, szz and p at rows zb0+1 .. zb0+7
                const float *SXXc = ss + PO_SXX * PS_FLOATS + lx + 4, *SZZc = ss + PO_SZZ * PS_FLOATS + lx + 4;
                const float *SXZc = ss + PO_SXZ * PS_FLOATS + lx + 4, *PPc = ss + PO_P * PS_FLOATS + lx + 4;
                float sxzc[ROWS + 3], szzc[ROWS + 3], ppc[ROWS + 3];
                uint8_t idc[ROWS + 1];
#pragma unroll
                for (int r = 0; r < ROWS + 3; ++r) {
                    sxzc[r] = SXZc[(zb0 + r) * TMA_VW];
                    szzc[r] = SZZc[(zb0 + 1 + r) * TMA_VW];
                    ppc[r] = PPc[(zb0 + 1 + r) * TMA_VW];
                }
#pragma unroll
                for (int r = 0; r < ROWS + 1; ++r) idc[r] = COEF ? 0 : si[(zb0 + 2 + r) * IW + lx + 4];
#pragma unroll
                for (int r = 0; r < ROWS; ++r) {
                    const int zl = zb0 + r;
                    const int tz = z0 + zl;
                    if (!IN && (!x_in || tz > NZ)) continue;
                    const int pzo = zl + 4;
                    const int sr = (zl + 2) * TMA_VW;            // row of the stress tile
                    const int vo = (zl + 4) * TMA_VW + lx + 4;
                    const float vx0 = sv[0 * PV_FLOATS + vo], vz0 = sv[1 * PV_FLOATS + vo];
                    const float wx0 = sv[2 * PV_FLOATS + vo], wz0 = sv[3 * PV_FLOATS + vo];
                    const int o = (tz + ZH) * P + xi;
                    const float d1x = D4<SM>(SXXc[sr], SXXc[sr - 1], SXXc[sr + 1], SXXc[sr - 2], qx);
                    const float d2x = D4<SM>(ppc[r + 1], PPc[sr - 1], PPc[sr + 1], PPc[sr - 2], qx);
                    const float d3x = D4<SM>(sxzc[r + 2], sxzc[r + 1], sxzc[r + 3], sxzc[r], qz);
                    const float d1z = D4<SM>(SXZc[sr + 1], sxzc[r + 2], SXZc[sr + 2], SXZc[sr - 1], qx);
                    const float d2z = D4<SM>(szzc[r + 2], szzc[r + 1], szzc[r + 3], szzc[r], qz);
                    const float d3z = D4<SM>(ppc[r + 2], ppc[r + 1], ppc[r + 3], ppc[r], qz);
                    const bool gvx = IN || (x_vx && tz >= 2 && tz <= NZ - 1);   // cu:289-291
                    const bool gvz = IN || (x_vz && tz >= 1 && tz <= NZ - 2);   // cu:326-328
                    const int zr = IN ? -1 : zrow(m, tz);
                    float m1 = 0.0f, m2 = 0.0f, m3 = 0.0f, m4 = 0.0f, m5 = 0.0f, m6 = 0.0f;
                    if (xc >= 0 && (gvx || gvz)) {
                        const int ix = tz * Wx + xc;
                        float *M1 = MXV + MXV_VX1 * nzx + ix, *M2 = MXV + MXV_VX2 * nzx + ix;
                        float *M4 = MXV + MXV_VZ * nzx + ix;
                        m1 = bx * gld_m<MS>(M1) + ax * d1x;
                        m2 = bx * gld_m<MS>(M2) + ax * d2x;
                        m4 = bxh * gld_m<MS>(M4) + axh * d1z;
                        if (gvx) {
                            gst(M1, m1);
                            gst(M2, m2);
                        }
                        if (gvz) gst(M4, m4);
                    }
                    if (zr >= 0 && (gvx || gvz)) {
                        const int iz = zr * P + xi;
                        float *M3 = MZV + MZV_VX * hzp + iz, *M5 = MZV + MZV_VZ1 * hzp + iz;
                        float *M6 = MZV + MZV_VZ2 * hzp + iz;
                        const float bh = PZs[PBH * PZH + pzo], ah = PZs[PAH * PZH + pzo];
                        m3 = PZs[PB * PZH + pzo] * gld_m<MS>(M3) + PZs[PA * PZH + pzo] * d3x;
                        m5 = bh * gld_m<MS>(M5) + ah * d2z;
                        m6 = bh * gld_m<MS>(M6) + ah * d3z;
                        if (gvx) gst(M3, m3);
                        if (gvz) {
                            gst(M5, m5);
                            gst(M6, m6);
                        }
                    }
                    const float Kz = KONE ? 1.0f : PZs[PK * PZH + pzo], Kzh = KONE ? 1.0f : PZs[PKH * PZH + pzo];
                    float vx1 = vx0, wx1 = wx0, vz1 = vz0, wz1 = wz0;
                    {   // vx, wx, material at (x, t) (cu:293-311)
                        const float A = addm(addm(KDIV<KONE>(d1x, Kx), m1) + KDIV<KONE>(d3x, Kz), m3);
                        const float B = addm(KDIV<KONE>(d2x, Kx), m2);
                        float w1, v1;
                        if (COEF)
                            velocity_coef(cf + o, PL, dt, A, B, wx0, vx0, w1, v1);
                        else {
                            const float *mt = st + MT_W * idc[r];
                            const float4 bb = *reinterpret_cast<const float4 *>(mt + 4);    // c2 rhof rho c1
                            const float4 cc = *reinterpret_cast<const float4 *>(mt + 8);    // 1/c1 m rhof*eok co
                            const float rco = mt[MT_RCO];
                            w1 = div_by(bb.x * wx0 + (-bb.y * A - bb.z * B), bb.w, cc.x);
                            v1 = vx0 + div_by(cc.y * A + bb.y * B + cc.z * ((wx0 + w1) * 0.5f), cc.w, rco);
                        }
                        if (gvx) { wx1 = w1; vx1 = v1; }
                    }
                    {   // vz, wz, material at (x, t+1) (cu:330-353)
                        float A = addm(addm(KDIV<KONE>(d1z, Kxh), m4) + KDIV<KONE>(d2z, Kzh), m5);
                        const float B = addm(KDIV<KONE>(d3z, Kzh), m6);
                        if (!IN && o == src_off && src_where == SRC_FZ && src_on) A = A + src_val;
                        float w1, v1;
                        if (COEF)
                            velocity_coef(cf + o + P, PL, dt, A, B, wz0, vz0, w1, v1);
                        else {
                            const float *mt = st + MT_W * idc[r + 1];
                            const float4 bb = *reinterpret_cast<const float4 *>(mt + 4);
                            const float4 cc = *reinterpret_cast<const float4 *>(mt + 8);
                            const float rco = mt[MT_RCO];
                            w1 = div_by(bb.x * wz0 + (-bb.y * A - bb.z * B), bb.w, cc.x);
                            v1 = vz0 + div_by(cc.y * A + bb.y * B + cc.z * ((wz0 + w1) * 0.5f), cc.w, rco);
                        }
                        if (gvz) { wz1 = w1; vz1 = v1; }
                    }
                    gst(FB + SF_VX * PL + o, vx1);
                    gst(FB + SF_WX * PL + o, wx1);
                    gst(FB + SF_VZ * PL + o, vz1);
                    gst(FB + SF_WZ * PL + o, wz1);
                }
            }
            return true;
        };
        if (!(IM.interior ? compute(std::true_type{}) : compute(std::false_type{}))) {
            if (tid == 0) atomicExch(m.err, 1);
            return;
        }
        // hand buffer b back to the producer (and, MS, count the release for the
        // publisher; the warp barrier orders every lane's stores before both)
        fence_proxy_async();
        __syncwarp();
        if (lane == 0) {
            if (MS) red_add_release_cta(&released[b], 1);
            mbar_arrive(&empty[b]);
        }
    }
}

// SMs of the current device (the persistent grid: one CTA per SM)
inline int sm_count()
{
    static std::atomic<int> sms[64];
    int dev = 0;
    cudaGetDevice(&dev);
    std::atomic<int> &n = sms[dev & 63];
    if (!n.load(std::memory_order_relaxed)) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        n.store(v > 0 ? v : 1, std::memory_order_relaxed);
    }
    return n.load(std::memory_order_relaxed);
}

// Edge tiles prefetch their C-PML memory variables to L1 when each SM walks
// at least 8 tiles per step (a 2001^2 shot: 14, +6 %; 16 shots of 1001^2:
// 57, +4 %); with fewer (one 1001^2 shot: 3.6, every SM on the strip rows at
// once at the step start) the prefetches cost 10 %.
inline int prefetch_strips(int nitems) { return nitems >= 8 * sm_count() ? 1 : 0; }

// one launch of the step kernel of stencil mode SM: a single model (models
// null) or a batch (models: device array; m unused)
template <int SM, bool KONE, bool MULTI, bool COEF, bool MS, int TZ>
int tile_launch(const ModelDev &m, const ModelDev *models, const StreamShot *shots, const int4 *items, int nitems,
                int k, int nk, int *queue, cudaStream_t st)
{
    using G = tile::Geo<TZ>;
    static std::atomic<uint64_t> done{0};
    auto kern = k_tile_pal<SM, KONE, MULTI, COEF, MS, TZ>;
    smem_attr_once(kern, (int)G::PAL_SMEM, done);
    // persistent: one CTA per SM, fewer if the launch has fewer items (a
    // step-spanning launch counts every step's: CTAs past a step's tile count
    // take the next step's tiles as their neighbourhoods finish)
    const int64_t items_all = MS ? (int64_t)nk * nitems : nitems;
    const int grid = items_all < sm_count() ? (int)items_all : sm_count();
    if (grid <= 0) return (int)cudaGetLastError();
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(G::PNT + (MS ? 32 : 0));   // MS: + the publisher warp
    cfg.dynamicSmemBytes = G::PAL_SMEM;
    cfg.stream = st;
    // a step-spanning launch's CTAs wait for one another's tiles: a
    // cooperative launch guarantees that all of them are resident at once
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = MS ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return (int)cudaLaunchKernelEx(&cfg, kern, m, models, shots, items, nitems, k, MS ? nk : 1,
                                   prefetch_strips(nitems), queue);
}

// every (KONE, MULTI, COEF, step-spanning) variant of one stencil mode and
// tile height (MULTI: batches, built for 32-row tiles only)
template <int SM, int TZ>
int tile_launch_mode(const ModelDev &m, const ModelDev *models, const StreamShot *shots, const int4 *items,
                     int nitems, int k, int nk, bool kone, bool coef, int *queue, cudaStream_t st)
{
    const bool multi = models != nullptr;
    if (multi && TZ != PAL_TZ) return (int)cudaErrorInvalidValue;
    constexpr bool MU_OK = TZ == PAL_TZ;   // batch variants exist for the 32-row tile
    switch ((kone ? 8 : 0) | (multi ? 4 : 0) | (coef ? 2 : 0) | (nk > 1 ? 1 : 0)) {
#define POE_TILE_CASE(s, KO, MU, CO, MS) \
    case s: return tile_launch<SM, KO, MU && MU_OK, CO, MS, TZ>(m, models, shots, items, nitems, k, nk, queue, st);
        POE_TILE_CASE(0, false, false, false, false) POE_TILE_CASE(1, false, false, false, true)
        POE_TILE_CASE(2, false, false, true, false) POE_TILE_CASE(3, false, false, true, true)
        POE_TILE_CASE(4, false, true, false, false) POE_TILE_CASE(5, false, true, false, true)
        POE_TILE_CASE(6, false, true, true, false) POE_TILE_CASE(7, false, true, true, true)
        POE_TILE_CASE(8, true, false, false, false) POE_TILE_CASE(9, true, false, false, true)
        POE_TILE_CASE(10, true, false, true, false) POE_TILE_CASE(11, true, false, true, true)
        POE_TILE_CASE(12, true, true, false, false) POE_TILE_CASE(13, true, true, false, true)
        POE_TILE_CASE(14, true, true, true, false) POE_TILE_CASE(15, true, true, true, true)
#undef POE_TILE_CASE
    }
    return (int)cudaErrorInvalidValue;
}

}  // namespace poe
