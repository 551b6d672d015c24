// poe2d_api.cpp -- solver contexts behind the C ABI (include/poe2d.h).
//
// A context is one model on one GPU: its coefficient planes and C-PML
// profiles live in HBM once and are shared by all of its shots.  poe_run
// advances every shot together; the per-step launch sequence is captured
// once into a CUDA graph of kGraphSteps steps and replayed (the step number
// is read from each shot's device counter, so the graph never changes).
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/poe2d.h"
#include "poe2d_internal.h"
#include "poe2d_palette.h"
#include "poe2d_plan.h"

using namespace poe;

namespace {
constexpr int kGraphSteps = 64;
// POE_SPAN_AUTO: step-spanning launches for steps of at most this many tiles
// per SM (measured against a launch per step: a 2001^2 shot, 14 per SM,
// +22 %; one 1001^2 shot, 3.6 per SM, +78 %; 16 shots of 1001^2, 57 per SM,
// +4 %; 64 shots of 1001^2, 229 per SM, -3 %: with many tiles per step the
// step tail the spanning removes is small and its per-tile costs remain)
constexpr int kSpanTilesPerSM = 96;
}

struct ShotHost {
    float *f[2] = {nullptr, nullptr};       // NSF planes each, one allocation (f[0])
    // device copies of the tile boxes: [0] velocity, [1] state for 32-row
    // tiles, [2], [3] the same for PAL_TZ_SMALL-row tiles
    CUtensorMap *tm = nullptr;
    float *mx[2] = {nullptr, nullptr}, *mz[2] = {nullptr, nullptr};
    float *mxv = nullptr, *mzv = nullptr, *acc = nullptr;
    float *src_tab = nullptr, *trace = nullptr;
    // receivers as CSR over tiles, for each tile height ([0] PAL_TZ, [1] PAL_TZ_SMALL)
    int *rec_start[2] = {nullptr, nullptr};
    int4 *rec_sorted[2] = {nullptr, nullptr};
    int nrec = 0;
    int64_t trace_cap = 0;
    int64_t src_cap = 0;     // entries computed in src_tab
    int64_t src_n = 0;       // active entries
    bool src_complete = false;
    poe_source src{};
    int64_t src_off = -1;
    int src_where = SRC_NONE;
    int64_t steps = 0;
    uint64_t rec_hash = 0;   // of the receiver list (checkpoint identity)
    int *done = nullptr;     // per tile: a step it has completed (step-spanning launches); sized for
                             // the smaller tile height's tiling
};

struct poe_ctx {
    poe_grid g{};
    ModelDev m{};
    bool exact = true, kone = true;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int device = 0;
    float *coef = nullptr, *px = nullptr, *pz = nullptr;
    std::vector<ShotHost> shots;
    StreamShot *shots_dev = nullptr;
    int64_t *steps_dev = nullptr;
    int shots_dev_cap = 0;
    std::vector<StreamShot> shots_host;    // what shots_dev holds
    std::vector<int4> items;               // palette mode: (0, shot, x0, z0) per tile and shot
    int4 *items_dev = nullptr;
    int items_dev_cap = 0;
    bool shots_dirty = true;
    int max_rec = 0;
    cudaGraphExec_t graph = nullptr;
    int graph_kernels = 0;
    int64_t launches = 0;
    float *derived = nullptr;   // 3 planes: sigma_xx, sigma_zz, p on demand
    int *err_dev = nullptr;     // set by a kernel whose bounded wait gave up
    int *queue_dev = nullptr;   // the step kernel's work queue (2 ints, zero between launches)
    uint8_t *ids = nullptr;     // palette mode: material id plane
    CUtensorMap *tm_model = nullptr;   // palette mode: TMA descriptors of ids, px, pz (device)
    float *mtab = nullptr;      // palette mode: material table
    int nmat = 0;
    int ntx = 1, ntz = 1;       // tiles across x and z (at the context's tile height)
    int ncell_max = 1;          // tiles at the smaller tile height (the shots' flag arrays)
    int order = POE_ORDER_ROWS;      // work-list order (POE_ORDER_*; EXACT contexts start BALANCED)
    int graph_steps = kGraphSteps;   // steps per captured graph
    int span = POE_SPAN_AUTO;        // step-spanning launches (POE_SPAN_*)
    int tile_x = PAL_TX, tile_z = PAL_TZ;   // the step kernel's tile (tile_z: PAL_TZ or PAL_TZ_SMALL)
    poe_batch *batch = nullptr;   // the batch this context belongs to, if any
    uint64_t prof_hash = 0;       // of the C-PML profiles given to poe_create
    uint64_t coef_hash = 0;       // of the 8 coefficient planes, computed on first checkpoint use
    bool coef_hashed = false;
    std::string err;
};

namespace {
void batch_forget(poe_batch *b, poe_ctx *ctx);   // a member context is being destroyed
}

namespace {

int fail(poe_ctx *c, int code, const std::string &msg)
{
    if (c) c->err = msg;
    return code;
}

// 64-bit hash of a stream of 32-bit words (checkpoint identities and payload)
struct Hash64 {
    uint64_t h = 0x9e3779b97f4a7c15ull;
    void word(uint32_t w)
    {
        h = (h ^ w) * 0x100000001b3ull;
        h ^= h >> 29;
    }
    void floats(const float *v, size_t n)
    {
        for (size_t i = 0; i < n; ++i) {
            uint32_t w;
            std::memcpy(&w, v + i, 4);
            word(w);
        }
    }
};

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? POE_ENOMEM : POE_ECUDA,   \
                        std::string(#call) + ": " + cudaGetErrorString(e_));             \
    } while (0)

#define CKL(rc)                                                                           \
    do {                                                                                  \
        int r_ = (rc);                                                                    \
        if (r_ != 0)                                                                      \
            return fail(ctx, POE_ECUDA, std::string("kernel launch: ") +                  \
                                            cudaGetErrorString((cudaError_t)r_));         \
    } while (0)

void free_shot(ShotHost &s)
{
    cudaFree(s.f[0]);
    cudaFree(s.tm);
    for (int i = 0; i < 2; ++i) {
        cudaFree(s.mx[i]);
        cudaFree(s.mz[i]);
    }
    cudaFree(s.mxv);
    cudaFree(s.mzv);
    cudaFree(s.acc);
    cudaFree(s.src_tab);
    cudaFree(s.trace);
    for (int t = 0; t < 2; ++t) {
        cudaFree(s.rec_start[t]);
        cudaFree(s.rec_sorted[t]);
    }
    cudaFree(s.done);
    s = ShotHost{};
}

void drop_graph(poe_ctx *ctx)
{
    if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
    ctx->graph = nullptr;
}

// strip extents from the profiles: a column carries C-PML memory only where
// a != 0 in one of its profiles (elsewhere b = 1, a = 0 keeps it zero)
void strips(const float *prof, int n1, int &lo, int &hi)
{
    const float *a = prof + POE_PA * n1, *ah = prof + POE_PA_HALF * n1;
    lo = 0;
    hi = n1;
    for (int i = 0; i < n1 / 2; ++i)
        if (a[i] != 0.0f || ah[i] != 0.0f) lo = i + 1;
    for (int i = n1 - 1; i >= n1 / 2; --i)
        if (a[i] != 0.0f || ah[i] != 0.0f) hi = i;
    if (lo >= hi) {   // strips meet: store the full axis
        lo = n1;
        hi = n1;
    }
}


// SMs of a device: the number of CTAs of a persistent step launch
int device_sms(int device)
{
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || v < 1) v = 1;
    return v;
}

// whether the step kernel takes its guarded (edge) path for the tile at
// (x0, z0) of a shot: a grid edge, a C-PML strip or the source within the
// tile and its halo; the same test as the kernel's interior flag
bool tile_is_edge(const poe_ctx *ctx, int shot, int x0, int z0)
{
    const ModelDev &m = ctx->m;
    const ShotHost &s = ctx->shots[(size_t)shot];
    const int xa = x0 - 2, xb = x0 + ctx->tile_x + 1, za = z0 - 2, zb = z0 + ctx->tile_z + 1;
    const bool src_in = s.src_where != SRC_NONE && s.src.ix >= xa && s.src.ix <= xb && s.src.iz >= za &&
                        s.src.iz <= zb;
    const bool interior = xa >= 2 && xa >= m.xL && xb <= m.NX - 2 && xb < m.xR && za >= 2 && za >= m.zT &&
                          zb <= m.NZ - 2 && zb < m.zB && !src_in;
    return !interior;
}

// the step kernel's tile height (PAL_TZ or PAL_TZ_SMALL): tile counts and the
// model's id and z-profile boxes; the work list and the shots' tile data
// follow at the next sync
void set_tile(poe_ctx *ctx, int tz)
{
    const int nz = ctx->g.NZ + 1;
    const int t = tz == PAL_TZ ? 0 : 1;
    ctx->tile_z = tz;
    ctx->ntz = (nz + tz - 1) / tz;
    ctx->m.ntx = ctx->ntx;
    ctx->m.ntz = ctx->ntz;
    ctx->m.tm_ids = ctx->tm_model && ctx->ids ? (const void *)&ctx->tm_model[t ? 3 : 0] : nullptr;
    ctx->m.tm_pz = ctx->tm_model ? (const void *)&ctx->tm_model[t ? 4 : 2] : nullptr;
    ctx->shots_dirty = true;
}

int sync_shots(poe_ctx *ctx)
{
    if (!ctx->shots_dirty) return POE_OK;
    const int ns = (int)ctx->shots.size();
    if (ns > ctx->shots_dev_cap) {
        const int cap = std::max(ns, 2 * ctx->shots_dev_cap);
        cudaFree(ctx->shots_dev);
        cudaFree(ctx->steps_dev);
        ctx->shots_dev = nullptr;
        ctx->steps_dev = nullptr;
        ctx->shots_dev_cap = 0;   // a failed allocation below leaves no stale capacity
        CK(cudaMalloc(&ctx->shots_dev, sizeof(StreamShot) * cap));
        CK(cudaMalloc(&ctx->steps_dev, sizeof(int64_t) * cap));
        ctx->shots_dev_cap = cap;
    }
    std::vector<StreamShot> sd(ns);
    std::vector<int64_t> st(ns);
    ctx->max_rec = 0;
    for (int i = 0; i < ns; ++i) {
        const ShotHost &s = ctx->shots[i];
        StreamShot &d = sd[i];
        for (int b = 0; b < 2; ++b) {
            d.f[b] = s.f[b];
            d.mx[b] = s.mx[b];
            d.mz[b] = s.mz[b];
        }
        d.mxv = s.mxv;
        d.mzv = s.mzv;
        d.acc = s.acc;
        d.step = ctx->steps_dev + i;
        d.src_off = s.src_off;
        d.src_where = s.src_where;
        d.src_n = s.src_n;
        d.src_tab = s.src_tab;
        const int ti = ctx->tile_z == PAL_TZ ? 0 : 1;
        d.rec_start = s.rec_start[ti];
        d.rec_sorted = s.rec_sorted[ti];
        d.nrec = s.nrec;
        d.trace = s.trace;
        d.trace_cap = s.trace_cap;
        d.tm_v = s.tm ? (const void *)&s.tm[2 * ti] : nullptr;
        d.tm_s = s.tm ? (const void *)&s.tm[2 * ti + 1] : nullptr;
        d.done = s.done;
        st[i] = s.steps;
        ctx->max_rec = std::max(ctx->max_rec, s.nrec);
    }
    // step kernel work list: every tile of every shot, in the context's order
    ctx->items.clear();
    {
        auto add = [&](int i, int tx, int tz) {
            ctx->items.push_back(make_int4(0, i, tx * ctx->tile_x, tz * ctx->tile_z));
        };
        if (ctx->order == POE_ORDER_TILE_MAJOR) {        // the same tile of every shot side by side
            for (int tz = 0; tz < ctx->ntz; ++tz)
                for (int tx = 0; tx < ctx->ntx; ++tx)
                    for (int i = 0; i < ns; ++i) add(i, tx, tz);
        } else if (ctx->order == POE_ORDER_COLUMNS) {    // per shot, tile columns
            for (int i = 0; i < ns; ++i)
                for (int tx = 0; tx < ctx->ntx; ++tx)
                    for (int tz = 0; tz < ctx->ntz; ++tz) add(i, tx, tz);
        } else {                                         // per shot, tile rows
            for (int i = 0; i < ns; ++i)
                for (int tz = 0; tz < ctx->ntz; ++tz)
                    for (int tx = 0; tx < ctx->ntx; ++tx) add(i, tx, tz);
        }
        if (ctx->order == POE_ORDER_BALANCED) {
            // the same tiles, dealt so every CTA of the persistent launch gets
            // an even share of edge tiles (poe2d_plan.h)
            std::vector<uint8_t> edge(ctx->items.size());
            for (size_t j = 0; j < ctx->items.size(); ++j)
                edge[j] = tile_is_edge(ctx, ctx->items[j].y, ctx->items[j].z, ctx->items[j].w) ? 1 : 0;
            const std::vector<int> perm = balanced_order(edge, device_sms(ctx->device));
            std::vector<int4> dealt(ctx->items.size());
            for (size_t p = 0; p < perm.size(); ++p) dealt[p] = ctx->items[(size_t)perm[p]];
            ctx->items.swap(dealt);
        }
    }
    const int ni = (int)ctx->items.size();
    if (ni > ctx->items_dev_cap) {
        const int cap = std::max(ni, 2 * ctx->items_dev_cap);
        cudaFree(ctx->items_dev);
        ctx->items_dev = nullptr;
        ctx->items_dev_cap = 0;
        CK(cudaMalloc(&ctx->items_dev, sizeof(int4) * cap));
        ctx->items_dev_cap = cap;
    }
    if (ns) {
        CK(cudaMemcpyAsync(ctx->shots_dev, sd.data(), sizeof(StreamShot) * ns, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(ctx->steps_dev, st.data(), sizeof(int64_t) * ns, cudaMemcpyHostToDevice, ctx->stream));
        if (ni)
            CK(cudaMemcpyAsync(ctx->items_dev, ctx->items.data(), sizeof(int4) * ni, cudaMemcpyHostToDevice,
                               ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));   // host vectors go out of scope
    }
    ctx->shots_host = sd;
    drop_graph(ctx);
    ctx->shots_dirty = false;
    return POE_OK;
}

// make the source table of shot s cover steps up to need (1-based)
int ensure_source(poe_ctx *ctx, ShotHost &s, int64_t need)
{
    if (s.src_where == SRC_NONE || s.src_complete || s.src_cap >= need) return POE_OK;
    int64_t cap = std::max<int64_t>(need, std::max<int64_t>(1024, 2 * s.src_cap));
    std::vector<float> tab((size_t)cap);
    int64_t nact = 0;
    int rc = poe_source_table(&ctx->g, &s.src, cap, tab.data(), &nact);
    if (rc != POE_OK) return fail(ctx, rc, "source table");
    // the new table replaces the old one only once it is on the device: the
    // shots' device records keep pointing at a live table if anything fails
    float *nt = nullptr;
    if (nact > 0) {
        cudaError_t e = cudaMalloc(&nt, sizeof(float) * nact);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(nt, tab.data(), sizeof(float) * nact, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) {
            cudaFree(nt);
            return fail(ctx, e == cudaErrorMemoryAllocation ? POE_ENOMEM : POE_ECUDA,
                        std::string("source table: ") + cudaGetErrorString(e));
        }
    }
    CK(cudaStreamSynchronize(ctx->stream));   // no launch still reads the old table
    cudaFree(s.src_tab);
    s.src_tab = nt;
    s.src_n = nact;
    s.src_cap = cap;
    s.src_complete = nact < cap;
    ctx->shots_dirty = true;
    return POE_OK;
}

int ensure_trace(poe_ctx *ctx, ShotHost &s, int64_t need)
{
    if (s.nrec == 0 || s.trace_cap >= need) return POE_OK;
    const int64_t cap = std::max<int64_t>(need, std::max<int64_t>(256, s.trace_cap + s.trace_cap / 2));
    float *nt = nullptr;
    CK(cudaMalloc(&nt, sizeof(float) * cap * s.nrec));
    cudaError_t e = cudaMemsetAsync(nt, 0, sizeof(float) * cap * s.nrec, ctx->stream);
    if (e == cudaSuccess && s.trace && s.trace_cap)
        e = cudaMemcpyAsync(nt, s.trace, sizeof(float) * s.trace_cap * s.nrec, cudaMemcpyDeviceToDevice,
                            ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {   // the shot keeps its old trace buffer
        cudaFree(nt);
        return fail(ctx, POE_ECUDA, std::string("trace buffer: ") + cudaGetErrorString(e));
    }
    cudaFree(s.trace);
    s.trace = nt;
    s.trace_cap = cap;
    ctx->shots_dirty = true;
    return POE_OK;
}

// steps k .. k+nk-1 in one launch (nk > 1: step-spanning)
int step_launch(poe_ctx *ctx, int k, int nk)
{
    return launch_tile_step(ctx->m, ctx->shots_dev, (int)ctx->shots.size(), ctx->items_dev, (int)ctx->items.size(), k,
                            nk, ctx->exact, ctx->kone, ctx->tile_z, ctx->queue_dev, ctx->stream);
}

// the context's launches for nsteps steps (one step-spanning launch, or one
// per step); returns the launches issued, or -1 with ctx->err set
int64_t issue_steps(poe_ctx *ctx, int64_t nsteps)
{
    const bool span = ctx->span == POE_SPAN_ALWAYS ||
                      (ctx->span == POE_SPAN_AUTO &&
                       (int64_t)ctx->items.size() <= (int64_t)kSpanTilesPerSM * device_sms(ctx->device));
    if (span && nsteps > 1) {
        const int r = step_launch(ctx, 0, (int)nsteps);
        if (r) return fail(ctx, POE_ECUDA, std::string("kernel launch: ") + cudaGetErrorString((cudaError_t)r)), -1;
        return 1;
    }
    for (int64_t k = 0; k < nsteps; ++k) {
        const int r = step_launch(ctx, (int)k, 1);
        if (r) return fail(ctx, POE_ECUDA, std::string("kernel launch: ") + cudaGetErrorString((cudaError_t)r)), -1;
    }
    return nsteps;
}

int run_direct(poe_ctx *ctx, int64_t nsteps)
{
    const int ns = (int)ctx->shots.size();
    const int64_t l = issue_steps(ctx, nsteps);
    if (l < 0) return POE_ECUDA;
    ctx->launches += l;
    CKL(launch_advance(ctx->steps_dev, ns, nsteps, ctx->stream));
    ctx->launches += 1;
    return POE_OK;
}

int build_graph(poe_ctx *ctx)
{
    const int ns = (int)ctx->shots.size();
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int rc = 0;
    const int64_t l = issue_steps(ctx, ctx->graph_steps);
    if (l < 0) rc = (int)cudaErrorLaunchFailure;
    if (rc == 0) rc = launch_advance(ctx->steps_dev, ns, ctx->graph_steps, ctx->stream);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (rc != 0 || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail(ctx, POE_ECUDA, std::string("graph capture: ") +
                                        cudaGetErrorString(rc ? (cudaError_t)rc : e));
    }
    e = cudaGraphInstantiate(&ctx->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        ctx->graph = nullptr;
        return fail(ctx, POE_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    }
    ctx->graph_kernels = (int)l + 1;   // the step launches and one clock advance
    return POE_OK;
}

// after a stream sync: POE_ETIMEOUT if a kernel reported a bounded wait that gave up
int device_status(poe_ctx *ctx)
{
    int h = 0;
    CK(cudaMemcpyAsync(&h, ctx->err_dev, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (h) {
        CK(cudaMemsetAsync(ctx->err_dev, 0, sizeof(int), ctx->stream));
        // a launch that gave up may have left its work queue mid-way
        CK(cudaMemsetAsync(ctx->queue_dev, 0, 2 * sizeof(int), ctx->stream));
        return fail(ctx, POE_ETIMEOUT, "a kernel's bounded wait for its shared-memory copies gave up");
    }
    return POE_OK;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no -lcuda)
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn()
{
    // contexts may be created on several threads at once: the entry point is
    // published atomically (a failed lookup is retried by the next caller)
    static std::atomic<EncodeTiledFn> fn{nullptr};
    EncodeTiledFn f = fn.load(std::memory_order_acquire);
    if (!f) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess) {
            f = (EncodeTiledFn)p;
            fn.store(f, std::memory_order_release);
        }
    }
    return f;
}

// TMA descriptor of a 2-D array (d0 elements per row, d1 rows, rows stride
// bytes apart) with a (box_w x box_h) box
bool encode_2d(CUtensorMap *out, CUtensorMapDataType type, void *base, int64_t d0, int64_t d1, int64_t stride,
               int box_w, int box_h)
{
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)d0, (cuuint64_t)d1};
    cuuint64_t strides[1] = {(cuuint64_t)stride};
    cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
    cuuint32_t es[2] = {1, 1};
    return fn(out, type, 2, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// TMA descriptor of a stack of float planes (pitch P, R rows, nplanes) with a
// (box_w x box_h x box_d) box: box_d consecutive planes in one copy
bool encode_planes(CUtensorMap *out, float *base, const ModelDev &m, int nplanes, int box_w, int box_h, int box_d)
{
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[3] = {(cuuint64_t)m.P, (cuuint64_t)m.R, (cuuint64_t)nplanes};
    cuuint64_t strides[2] = {(cuuint64_t)m.P * 4, (cuuint64_t)m.plane * 4};
    cuuint32_t box[3] = {(cuuint32_t)box_w, (cuuint32_t)box_h, (cuuint32_t)box_d};
    cuuint32_t es[3] = {1, 1, 1};
    return fn(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

ShotHost *get_shot(poe_ctx *ctx, int32_t shot)
{
    if (!ctx || shot < 0 || shot >= (int32_t)ctx->shots.size()) return nullptr;
    return &ctx->shots[shot];
}

}  // namespace

extern "C" {

int poe_create(const poe_grid *grid, const float *coef, const float *prof_x, const float *prof_z,
               void *stream, uint32_t flags, poe_ctx **out)
{
    if (!out) return POE_EINVAL;
    *out = nullptr;
    if (!grid || !coef || !prof_x || !prof_z || grid->NX < 4 || grid->NZ < 4 || !(grid->dx > 0.0f) ||
        !(grid->dz > 0.0f) || !(grid->dt > 0.0f))
        return POE_EINVAL;
    poe_ctx *ctx = new poe_ctx();
    ctx->g = *grid;
    ctx->exact = !(flags & POE_CTX_FAST_STENCIL);
    // the CTAs take the work list in order: with FAST stencils (bandwidth
    // bound) rows keep the tiles in flight neighbours, whose halos meet in L2
    // (2001^2 shot: 63.7 against 61.8 Gcell/s balanced); with EXACT stencils
    // (about twice the instructions) an even mix of edge and interior tiles in
    // flight wins (27.8 against 25.1)
    ctx->order = ctx->exact ? POE_ORDER_BALANCED : POE_ORDER_ROWS;
    cudaGetDevice(&ctx->device);
    if (stream) {
        ctx->stream = (cudaStream_t)stream;
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            delete ctx;
            return POE_ECUDA;
        }
        ctx->own_stream = true;
    }
    const int nx = grid->NX + 1, nz = grid->NZ + 1;
    ModelDev &m = ctx->m;
    m.NX = grid->NX;
    m.NZ = grid->NZ;
    // tiles (60 x 32) read columns x0-4 .. x0+63 and rows z0-4 .. z0+35; the
    // pitch also rounds the grid up to 64-cell tiles (the 2001-cell benchmark
    // rows: 2080 floats, not a power of two)
    {
        const int px1 = ((nx + TILE_X - 1) / TILE_X) * TILE_X + 8;
        const int px2 = ((nx + PAL_TX - 1) / PAL_TX) * PAL_TX + 8;
        m.P = (std::max(std::max(px1, px2), XH + nx + 4) + 31) / 32 * 32;
        m.R = std::max((nz + TILE_Z - 1) / TILE_Z * TILE_Z, (nz + PAL_TZ - 1) / PAL_TZ * PAL_TZ) + 8;
    }
    m.plane = (int64_t)m.P * m.R;
    {
        Hash64 hp;
        hp.floats(prof_x, (size_t)6 * nx);
        hp.floats(prof_z, (size_t)6 * nz);
        ctx->prof_hash = hp.h;
    }
    m.dt = grid->dt;
    m.qx = make_div24(grid->dx);
    m.qz = make_div24(grid->dz);
    strips(prof_x, nx, m.xL, m.xR);
    strips(prof_z, nz, m.zT, m.zB);
    m.Wx = m.xL + (nx - m.xR);
    m.Hz = m.zT + (nz - m.zB);
    // K == 1 everywhere (K_max = 1, cu:843) lets the kernels skip value / K
    ctx->kone = true;
    for (int r : {POE_PK, POE_PK_HALF}) {
        for (int i = 0; i < nx; ++i) ctx->kone &= prof_x[r * nx + i] == 1.0f;
        for (int i = 0; i < nz; ++i) ctx->kone &= prof_z[r * nz + i] == 1.0f;
    }
    auto up_planes = [&](float **dst, const float *src, int nplanes) -> int {
        CK(cudaMalloc(dst, sizeof(float) * m.plane * nplanes));
        CK(cudaMemsetAsync(*dst, 0, sizeof(float) * m.plane * nplanes, ctx->stream));
        for (int p = 0; p < nplanes; ++p)
            CK(cudaMemcpy2DAsync(*dst + p * m.plane + (int64_t)ZH * m.P + XH, sizeof(float) * m.P,
                                 src + (int64_t)p * nx * nz, sizeof(float) * nx, sizeof(float) * nx, nz,
                                 cudaMemcpyHostToDevice, ctx->stream));
        return POE_OK;
    };
    int rc = POE_OK;
    // palette mode when the model has few distinct materials (patchy models)
    std::vector<uint8_t> hid;
    std::vector<float> htab;
    const bool pal = !(flags & POE_CTX_NO_PALETTE) && encode_fn() &&
                     build_palette(coef, (int64_t)nx * nz, grid->dt, hid, htab);
    if (pal) {
        ctx->nmat = (int)(htab.size() / MT_W);
        cudaError_t e = cudaMalloc(&ctx->ids, (size_t)m.P * m.R);
        if (e == cudaSuccess) e = cudaMemsetAsync(ctx->ids, 0, (size_t)m.P * m.R, ctx->stream);
        if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(ctx->ids + (size_t)ZH * m.P + XH, m.P, hid.data(), nx, nx, nz,
                                  cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaMalloc(&ctx->mtab, sizeof(float) * htab.size());
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(ctx->mtab, htab.data(), sizeof(float) * htab.size(), cudaMemcpyHostToDevice,
                                ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = fail(ctx, POE_ECUDA, std::string("palette upload: ") + cudaGetErrorString(e));
    } else {
        rc = up_planes(&ctx->coef, coef, POE_NCOEF);
    }
    if (rc == POE_OK) {
        std::vector<float> hx((size_t)6 * m.P, 0.0f), hz((size_t)6 * m.R, 0.0f);
        for (int r = 0; r < 6; ++r) {
            // outside the grid: b = 1, K = 1, a = 0 (no memory update, no scaling)
            const bool one = r == POE_PB || r == POE_PB_HALF || r == POE_PK || r == POE_PK_HALF;
            for (int i = 0; i < m.P; ++i) hx[(size_t)r * m.P + i] = one ? 1.0f : 0.0f;
            for (int i = 0; i < m.R; ++i) hz[(size_t)r * m.R + i] = one ? 1.0f : 0.0f;
            for (int i = 0; i < nx; ++i) hx[(size_t)r * m.P + XH + i] = prof_x[(size_t)r * nx + i];
            for (int i = 0; i < nz; ++i) hz[(size_t)r * m.R + ZH + i] = prof_z[(size_t)r * nz + i];
        }
        cudaError_t e = cudaMalloc(&ctx->px, sizeof(float) * hx.size());
        if (e == cudaSuccess) e = cudaMalloc(&ctx->err_dev, sizeof(int));
        if (e == cudaSuccess) e = cudaMemsetAsync(ctx->err_dev, 0, sizeof(int), ctx->stream);
        if (e == cudaSuccess) e = cudaMalloc(&ctx->queue_dev, 2 * sizeof(int));
        if (e == cudaSuccess) e = cudaMemsetAsync(ctx->queue_dev, 0, 2 * sizeof(int), ctx->stream);
        if (e == cudaSuccess) e = cudaMalloc(&ctx->pz, sizeof(float) * hz.size());
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(ctx->px, hx.data(), sizeof(float) * hx.size(), cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(ctx->pz, hz.data(), sizeof(float) * hz.size(), cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = fail(ctx, POE_ECUDA, std::string("upload: ") + cudaGetErrorString(e));
    }
    if (rc == POE_OK) {
        // the step kernel's producer fetches each tile's ids (palette models)
        // and profile slices with TMA (rows of P bytes / P floats / R floats)
        // [0] ids, [1] x profiles, [2] z profiles for 32-row tiles; [3] ids, [4] z
        // profiles for PAL_TZ_SMALL-row tiles
        CUtensorMap tm[5];
        std::memset(tm, 0, sizeof(tm));
        bool ok = encode_2d(&tm[1], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, ctx->px, m.P, 6, (int64_t)m.P * 4, TMA_VW, 6);
        for (int t = 0; t < 2 && ok; ++t) {
            const int tz = t ? PAL_TZ_SMALL : PAL_TZ;
            ok = (!ctx->ids || encode_2d(&tm[t ? 3 : 0], CU_TENSOR_MAP_DATA_TYPE_UINT8, ctx->ids, m.P, m.R, m.P,
                                         PAL_IDS_W, tile_ids_h(tz))) &&
                 encode_2d(&tm[t ? 4 : 2], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, ctx->pz, m.R, 6, (int64_t)m.R * 4,
                           tile_vh(tz), 6);
        }
        cudaError_t e = ok ? cudaMalloc(&ctx->tm_model, sizeof(tm)) : cudaErrorInvalidValue;
        if (e == cudaSuccess) e = cudaMemcpy(ctx->tm_model, tm, sizeof(tm), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) rc = fail(ctx, POE_ECUDA, std::string("TMA descriptors: ") + cudaGetErrorString(e));
    }
    if (rc != POE_OK) {
        poe_destroy(ctx);
        return rc;
    }
    m.coef = ctx->coef;
    m.px = ctx->px;
    m.pz = ctx->pz;
    m.err = ctx->err_dev;
    m.ids = ctx->ids;
    m.mtab = ctx->mtab;
    m.nmat = ctx->nmat;
    m.tm_px = ctx->tm_model ? (const void *)&ctx->tm_model[1] : nullptr;
    // tile geometry of the step kernel (receiver lists and flags are per tile)
    ctx->tile_x = PAL_TX;
    ctx->ntx = (nx + ctx->tile_x - 1) / ctx->tile_x;
    ctx->ncell_max = ctx->ntx * ((nz + PAL_TZ_SMALL - 1) / PAL_TZ_SMALL);
    set_tile(ctx, PAL_TZ);
    *out = ctx;
    return POE_OK;
}

int poe_add_shot(poe_ctx *ctx, const poe_source *src, const poe_receiver *rec, int32_t nrec, int32_t *shot_id)
{
    if (!ctx) return POE_EINVAL;
    if (nrec < 0 || (nrec > 0 && !rec)) return fail(ctx, POE_EINVAL, "receivers");
    const int NX = ctx->g.NX, NZ = ctx->g.NZ;
    const ModelDev &m = ctx->m;
    ShotHost s;
    if (src) {
        if (src->ix < 0 || src->ix > NX || src->iz < 0 || src->iz > NZ)
            return fail(ctx, POE_EINVAL, "source outside the grid");
        if (src->kind != POE_SRC_REF_DGAUSS_P && src->kind != POE_SRC_RICKER_FZ)
            return fail(ctx, POE_EINVAL, "source kind");
        if (!(src->f0 > 0.0f)) return fail(ctx, POE_EINVAL, "source f0");
        s.src = *src;
        s.src_where = src->kind == POE_SRC_REF_DGAUSS_P ? SRC_P : SRC_FZ;
        s.src_off = (int64_t)(src->iz + ZH) * m.P + (src->ix + XH);
    }
    // receivers: CSR over tiles, so each tile records its own (for either tile height)
    for (int i = 0; i < nrec; ++i) {
        const poe_receiver &r = rec[i];
        if (r.comp == POE_REC_NONE) continue;
        if (r.comp < 0 || r.comp > 2 || r.ix < 0 || r.ix > NX || r.iz < 0 || r.iz > NZ)
            return fail(ctx, POE_EINVAL, "receiver " + std::to_string(i) + " outside the grid");
    }
    std::vector<int> start[2];
    std::vector<int4> sorted[2];
    for (int t = 0; t < 2; ++t) {
        const int tz = t ? PAL_TZ_SMALL : PAL_TZ;
        const int ncell = ctx->ntx * ((NZ + tz) / tz);
        start[t].assign((size_t)ncell + 1, 0);
        for (int i = 0; i < nrec; ++i)
            if (rec[i].comp != POE_REC_NONE) start[t][(size_t)(rec[i].iz / tz) * ctx->ntx + rec[i].ix / ctx->tile_x + 1]++;
        for (int c = 0; c < ncell; ++c) start[t][c + 1] += start[t][c];
        sorted[t].resize((size_t)start[t][ncell]);
        std::vector<int> fill(start[t].begin(), start[t].end() - 1);
        for (int i = 0; i < nrec; ++i) {
            const poe_receiver &r = rec[i];
            if (r.comp == POE_REC_NONE) continue;
            sorted[t][fill[(size_t)(r.iz / tz) * ctx->ntx + r.ix / ctx->tile_x]++] = make_int4(r.ix, r.comp, i, r.iz);
        }
    }
    auto bad = [&](cudaError_t e, const char *what) {
        free_shot(s);
        return fail(ctx, e == cudaErrorMemoryAllocation ? POE_ENOMEM : POE_ECUDA,
                    std::string(what) + ": " + cudaGetErrorString(e));
    };
    cudaError_t e;
    const size_t fbytes = sizeof(float) * m.plane * NSF;
    const size_t xbytes = sizeof(float) * 3 * (size_t)(NZ + 1) * m.Wx;
    const size_t zbytes = sizeof(float) * 3 * (size_t)m.Hz * m.P;
    if ((e = cudaMalloc(&s.f[0], 2 * fbytes)) != cudaSuccess) return bad(e, "state");
    if ((e = cudaMemsetAsync(s.f[0], 0, 2 * fbytes, ctx->stream)) != cudaSuccess) return bad(e, "state");
    s.f[1] = s.f[0] + NSF * m.plane;
    {
        CUtensorMap tm[4];
        // the 4 velocity planes (SF_VX .. SF_WZ) and the 5 stress-state planes
        // (SF_SXZ .. SF_XI2) of a tile, one copy each, for either tile height
        for (int t = 0; t < 2; ++t) {
            const int tz = t ? PAL_TZ_SMALL : PAL_TZ;
            if (!encode_planes(&tm[2 * t], s.f[0], m, 2 * NSF, TMA_VW, tile_vh(tz), 4) ||
                !encode_planes(&tm[2 * t + 1], s.f[0], m, 2 * NSF, TMA_VW, tile_sh(tz), 5))
                return bad(cudaErrorInvalidValue, "TMA descriptor");
        }
        if ((e = cudaMalloc(&s.tm, sizeof(tm))) != cudaSuccess) return bad(e, "TMA descriptor");
        if ((e = cudaMemcpyAsync(s.tm, tm, sizeof(tm), cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess)
            return bad(e, "TMA descriptor");
    }
    for (int b = 0; b < 2; ++b) {
        if (xbytes) {
            if ((e = cudaMalloc(&s.mx[b], xbytes)) != cudaSuccess) return bad(e, "x strips");
            if ((e = cudaMemsetAsync(s.mx[b], 0, xbytes, ctx->stream)) != cudaSuccess) return bad(e, "x strips");
        }
        if (zbytes) {
            if ((e = cudaMalloc(&s.mz[b], zbytes)) != cudaSuccess) return bad(e, "z strips");
            if ((e = cudaMemsetAsync(s.mz[b], 0, zbytes, ctx->stream)) != cudaSuccess) return bad(e, "z strips");
        }
    }
    if (xbytes) {
        if ((e = cudaMalloc(&s.mxv, xbytes)) != cudaSuccess) return bad(e, "x strips");
        if ((e = cudaMemsetAsync(s.mxv, 0, xbytes, ctx->stream)) != cudaSuccess) return bad(e, "x strips");
    }
    if (zbytes) {
        if ((e = cudaMalloc(&s.mzv, zbytes)) != cudaSuccess) return bad(e, "z strips");
        if ((e = cudaMemsetAsync(s.mzv, 0, zbytes, ctx->stream)) != cudaSuccess) return bad(e, "z strips");
    }
    if ((e = cudaMalloc(&s.acc, sizeof(float) * 2)) != cudaSuccess) return bad(e, "acc");
    if ((e = cudaMemsetAsync(s.acc, 0, sizeof(float) * 2, ctx->stream)) != cudaSuccess) return bad(e, "acc");
    if ((e = cudaMalloc(&s.done, sizeof(int) * ctx->ncell_max)) != cudaSuccess) return bad(e, "tile flags");
    if ((e = cudaMemsetAsync(s.done, 0, sizeof(int) * ctx->ncell_max, ctx->stream)) != cudaSuccess)
        return bad(e, "tile flags");
    for (int t = 0; t < 2; ++t) {
        if ((e = cudaMalloc(&s.rec_start[t], sizeof(int) * start[t].size())) != cudaSuccess) return bad(e, "receivers");
        if ((e = cudaMemcpyAsync(s.rec_start[t], start[t].data(), sizeof(int) * start[t].size(),
                                 cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess)
            return bad(e, "receivers");
        if (!sorted[t].empty()) {
            if ((e = cudaMalloc(&s.rec_sorted[t], sizeof(int4) * sorted[t].size())) != cudaSuccess)
                return bad(e, "receivers");
            if ((e = cudaMemcpyAsync(s.rec_sorted[t], sorted[t].data(), sizeof(int4) * sorted[t].size(),
                                     cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess)
                return bad(e, "receivers");
        }
    }
    s.nrec = nrec;
    {
        Hash64 hr;
        hr.word((uint32_t)nrec);
        for (int i = 0; i < nrec; ++i) {
            hr.word((uint32_t)rec[i].ix);
            hr.word((uint32_t)rec[i].iz);
            hr.word((uint32_t)rec[i].comp);
        }
        s.rec_hash = hr.h;
    }
    if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return bad(e, "add shot");
    ctx->shots.push_back(s);
    ctx->shots_dirty = true;
    if (shot_id) *shot_id = (int32_t)ctx->shots.size() - 1;
    return POE_OK;
}

int poe_run(poe_ctx *ctx, int64_t nsteps)
{
    if (!ctx) return POE_EINVAL;
    if (nsteps < 0) return fail(ctx, POE_EINVAL, "nsteps < 0");
    if (ctx->shots.empty()) return fail(ctx, POE_ESTATE, "no shots");
    if (nsteps == 0) return POE_OK;
    CK(cudaSetDevice(ctx->device));
    int rc;
    for (ShotHost &s : ctx->shots) {
        if ((rc = ensure_trace(ctx, s, s.steps + nsteps)) != POE_OK) return rc;
        if ((rc = ensure_source(ctx, s, s.steps + nsteps)) != POE_OK) return rc;
    }
    if ((rc = sync_shots(ctx)) != POE_OK) return rc;
    int64_t left = nsteps;
    if (left >= ctx->graph_steps) {
        if (!ctx->graph && (rc = build_graph(ctx)) != POE_OK) return rc;
        for (; left >= ctx->graph_steps; left -= ctx->graph_steps) {
            CK(cudaGraphLaunch(ctx->graph, ctx->stream));
            ctx->launches += ctx->graph_kernels;
        }
    }
    if (left > 0 && (rc = run_direct(ctx, left)) != POE_OK) return rc;
    for (ShotHost &s : ctx->shots) s.steps += nsteps;
    return POE_OK;
}

int poe_sync(poe_ctx *ctx)
{
    if (!ctx) return POE_EINVAL;
    CK(cudaStreamSynchronize(ctx->stream));
    return device_status(ctx);
}

int poe_get_traces(poe_ctx *ctx, int32_t shot, float *host_out, int64_t capacity_floats)
{
    ShotHost *s = get_shot(ctx, shot);
    if (!s) return fail(ctx, POE_EINVAL, "shot id");
    const int64_t n = s->steps * s->nrec;
    if (n == 0) return POE_OK;
    if (!host_out || capacity_floats < n) return fail(ctx, POE_EINVAL, "trace buffer too small");
    CK(cudaMemcpyAsync(host_out, s->trace, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return device_status(ctx);
}

namespace {
// plane holding a field of the shot's current state (derived planes are
// computed into ctx->derived first)
int field_plane(poe_ctx *ctx, int32_t shot, int32_t field, const float **plane)
{
    ShotHost *s = &ctx->shots[shot];
    const ModelDev &m = ctx->m;
    const float *cur = s->f[s->steps & 1];
    static const int map[POE_NFIELDS] = {SF_VX, SF_VZ, SF_WX, SF_WZ, -1, -1, SF_SXZ, -1,
                                         SF_G11, SF_G22, SF_XI1, SF_XI2};
    if (map[field] >= 0) {
        *plane = cur + map[field] * m.plane;
        return POE_OK;
    }
    if (!ctx->derived) CK(cudaMalloc(&ctx->derived, sizeof(float) * 3 * m.plane));
    int rc;
    if ((rc = sync_shots(ctx)) != POE_OK) return rc;
    CKL(launch_derive(m, ctx->shots_dev, shot, s->steps, ctx->derived, ctx->stream));
    const int which = field == POE_F_SXX ? 0 : (field == POE_F_SZZ ? 1 : 2);
    *plane = ctx->derived + which * m.plane;
    return POE_OK;
}
}  // namespace

int poe_get_field(poe_ctx *ctx, int32_t shot, int32_t field, float *host_out)
{
    ShotHost *s = get_shot(ctx, shot);
    if (!s) return fail(ctx, POE_EINVAL, "shot id");
    if (field < 0 || field >= POE_NFIELDS || !host_out) return fail(ctx, POE_EINVAL, "field id");
    const ModelDev &m = ctx->m;
    const int nx = m.NX + 1, nz = m.NZ + 1;
    const float *plane = nullptr;
    int rc = field_plane(ctx, shot, field, &plane);
    if (rc != POE_OK) return rc;
    CK(cudaMemcpy2DAsync(host_out, sizeof(float) * nx, plane + (int64_t)ZH * m.P + XH, sizeof(float) * m.P,
                         sizeof(float) * nx, nz, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return device_status(ctx);
}

int poe_get_derived_noalloc(poe_ctx *ctx, int32_t shot, int32_t field, float *host_out)
{
    ShotHost *s = get_shot(ctx, shot);
    if (!s) return fail(ctx, POE_EINVAL, "shot id");
    if (!host_out) return fail(ctx, POE_EINVAL, "null output");
    if (field != POE_F_SXX && field != POE_F_SZZ && field != POE_F_P)
        return fail(ctx, POE_EINVAL, "only sigma_xx, sigma_zz and p are derived; read the others with poe_get_field");
    const ModelDev &m = ctx->m;
    if (m.plane > NOALLOC_SCRATCH_FLOATS)
        return fail(ctx, POE_EINVAL,
                    "padded plane of " + std::to_string(m.plane) + " floats exceeds the static scratch of " +
                        std::to_string(NOALLOC_SCRATCH_FLOATS) + " floats");
    CK(cudaSetDevice(ctx->device));
    const int which = field == POE_F_SXX ? 0 : (field == POE_F_SZZ ? 1 : 2);
    const int rc = derive_noalloc(m, s->f[s->steps & 1], s->acc, s->src_off, s->src_where, s->src_n, s->src_tab,
                                  s->steps, which, host_out, ctx->stream);
    if (rc != 0) return fail(ctx, POE_ECUDA, std::string("derived read-out: ") + cudaGetErrorString((cudaError_t)rc));
    return device_status(ctx);
}

int poe_wait_limit_check(int32_t device, int32_t polls, int32_t *gave_up)
{
    if (!gave_up || polls < 1 || polls > (1 << 24)) return POE_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return POE_ECUDA;
    int *buf = nullptr;   // [0]: error bits; [1..9]: tile flags
    int flag = 0;
    const int h[10] = {0, 0, 5, 5, 5, 5, 5, 5, 5, 5};
    cudaError_t e = cudaMalloc(&buf, sizeof(h));
    if (e == cudaSuccess) e = cudaMemcpy(buf, h, sizeof(h), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = (cudaError_t)launch_wait_limit(buf, buf + 1, polls, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(&flag, buf, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(buf);
    if (e != cudaSuccess) return POE_ECUDA;
    // both waits on conditions that never hold gave up, the one on set flags did not
    *gave_up = flag == 3 ? 1 : 0;
    return POE_OK;
}

int poe_set_field(poe_ctx *ctx, int32_t shot, int32_t field, const float *host_in)
{
    ShotHost *s = get_shot(ctx, shot);
    if (!s) return fail(ctx, POE_EINVAL, "shot id");
    if (field < 0 || field >= POE_NFIELDS || !host_in) return fail(ctx, POE_EINVAL, "field id");
    if (field == POE_F_SXX || field == POE_F_SZZ || field == POE_F_P)
        return fail(ctx, POE_EINVAL, "sigma_xx, sigma_zz and p are derived from g11 g22 xi1 xi2");
    static const int map[POE_NFIELDS] = {SF_VX, SF_VZ, SF_WX, SF_WZ, -1, -1, SF_SXZ, -1,
                                         SF_G11, SF_G22, SF_XI1, SF_XI2};
    const ModelDev &m = ctx->m;
    const int nx = m.NX + 1, nz = m.NZ + 1;
    float *plane = s->f[s->steps & 1] + map[field] * m.plane;
    CK(cudaMemcpy2DAsync(plane + (int64_t)ZH * m.P + XH, sizeof(float) * m.P, host_in, sizeof(float) * nx,
                         sizeof(float) * nx, nz, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return POE_OK;
}

int poe_steps_done(poe_ctx *ctx, int32_t shot, int64_t *steps)
{
    ShotHost *s = get_shot(ctx, shot);
    if (!s || !steps) return fail(ctx, POE_EINVAL, "shot id");
    *steps = s->steps;
    return POE_OK;
}

int poe_reset_shot(poe_ctx *ctx, int32_t shot)
{
    ShotHost *s = get_shot(ctx, shot);
    if (!s) return fail(ctx, POE_EINVAL, "shot id");
    const ModelDev &m = ctx->m;
    const size_t xbytes = sizeof(float) * 3 * (size_t)(m.NZ + 1) * m.Wx;
    const size_t zbytes = sizeof(float) * 3 * (size_t)m.Hz * m.P;
    CK(cudaMemsetAsync(s->f[0], 0, sizeof(float) * m.plane * NSF * 2, ctx->stream));
    for (int b = 0; b < 2; ++b) {
        if (s->mx[b]) CK(cudaMemsetAsync(s->mx[b], 0, xbytes, ctx->stream));
        if (s->mz[b]) CK(cudaMemsetAsync(s->mz[b], 0, zbytes, ctx->stream));
    }
    if (s->mxv) CK(cudaMemsetAsync(s->mxv, 0, xbytes, ctx->stream));
    if (s->mzv) CK(cudaMemsetAsync(s->mzv, 0, zbytes, ctx->stream));
    CK(cudaMemsetAsync(s->acc, 0, sizeof(float) * 2, ctx->stream));
    CK(cudaMemsetAsync(s->done, 0, sizeof(int) * ctx->ncell_max, ctx->stream));   // never ahead of the shot
    if (s->trace) CK(cudaMemsetAsync(s->trace, 0, sizeof(float) * s->trace_cap * s->nrec, ctx->stream));
    s->steps = 0;
    ctx->shots_dirty = true;
    return sync_shots(ctx);
}

// ---- full-state checkpoints of one shot
//
// Layout: CkHeader, then (all float32, device layout incl. padding) the 9
// integrated state planes of the current buffer, the x-strip and z-strip
// C-PML memory of the stress update (current buffer) and of the velocity
// update, the pressure-source accumulator (padded to 4 floats) and the
// traces recorded so far (steps x nrec).  The other buffer of each pair is
// not needed: step n reads buffer (n-1)&1 only.
namespace {
typedef poe_checkpoint_header CkHeader;
static_assert(sizeof(CkHeader) % 16 == 0, "header keeps the payload 16-byte aligned");
static_assert(sizeof(CkHeader) == 160, "checkpoint header layout");
constexpr char kCkMagic[8] = {'P', 'O', 'E', '2', 'D', 'C', 'K', '1'};

uint64_t ck_sum(const unsigned char *p, size_t n)
{
    uint64_t h = 0x9e3779b97f4a7c15ull;
    size_t i = 0;
    for (; i + 8 <= n; i += 8) {
        uint64_t w;
        std::memcpy(&w, p + i, 8);
        h = (h ^ w) * 0x100000001b3ull;
        h ^= h >> 29;
    }
    for (; i < n; ++i) h = (h ^ p[i]) * 0x100000001b3ull;
    return h;
}

// hash of the model's 8 coefficient planes over the grid, plane by plane,
// rows of x: the same value whether the context keeps the planes or a
// material palette (read back from the device once per context)
int coef_hash(poe_ctx *ctx, uint64_t *out)
{
    if (!ctx->coef_hashed) {
        const ModelDev &m = ctx->m;
        const int nx = m.NX + 1, nz = m.NZ + 1;
        Hash64 h;
        if (ctx->ids) {
            std::vector<uint8_t> ids((size_t)nx * nz);
            std::vector<float> tab((size_t)ctx->nmat * MT_W);
            CK(cudaMemcpy2DAsync(ids.data(), nx, ctx->ids + (size_t)ZH * m.P + XH, m.P, nx, nz,
                                 cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaMemcpyAsync(tab.data(), ctx->mtab, sizeof(float) * tab.size(), cudaMemcpyDeviceToHost,
                               ctx->stream));
            CK(cudaStreamSynchronize(ctx->stream));
            // the table column of each coefficient plane (poe2d_palette.h)
            static const int col[POE_NCOEF] = {MT_RHO, MT_RHOF, MT_RSM, MT_EOK, MT_LC, MT_MU, MT_AL, MT_M};
            for (int c = 0; c < POE_NCOEF; ++c)
                for (size_t j = 0; j < ids.size(); ++j) h.floats(&tab[(size_t)ids[j] * MT_W + col[c]], 1);
        } else {
            std::vector<float> plane((size_t)nx * nz);
            for (int c = 0; c < POE_NCOEF; ++c) {
                CK(cudaMemcpy2DAsync(plane.data(), sizeof(float) * nx, ctx->coef + c * m.plane + (int64_t)ZH * m.P + XH,
                                     sizeof(float) * m.P, sizeof(float) * nx, nz, cudaMemcpyDeviceToHost, ctx->stream));
                CK(cudaStreamSynchronize(ctx->stream));
                h.floats(plane.data(), plane.size());
            }
        }
        ctx->coef_hash = h.h;
        ctx->coef_hashed = true;
    }
    *out = ctx->coef_hash;
    return POE_OK;
}

struct CkParts {
    size_t f, x, z, acc, tr;
};

CkParts ck_parts(const poe_ctx *ctx, const ShotHost &s)
{
    const ModelDev &m = ctx->m;
    CkParts c;
    c.f = sizeof(float) * m.plane * NSF;
    c.x = s.mxv ? sizeof(float) * 3 * (size_t)(m.NZ + 1) * m.Wx : 0;
    c.z = s.mzv ? sizeof(float) * 3 * (size_t)m.Hz * m.P : 0;
    c.acc = 4 * sizeof(float);
    c.tr = sizeof(float) * (size_t)s.steps * s.nrec;
    return c;
}

size_t ck_payload(const CkParts &c) { return c.f + 2 * c.x + 2 * c.z + c.acc + c.tr; }

int ck_fill_header(poe_ctx *ctx, const ShotHost &s, CkHeader &h)
{
    std::memset(&h, 0, sizeof h);
    std::memcpy(h.magic, kCkMagic, 8);
    h.version = POE_CHECKPOINT_VERSION;
    h.header_bytes = sizeof(CkHeader);
    const ModelDev &m = ctx->m;
    h.NX = m.NX;
    h.NZ = m.NZ;
    h.P = m.P;
    h.R = m.R;
    h.Wx = m.Wx;
    h.Hz = m.Hz;
    h.plane = m.plane;
    h.steps = s.steps;
    h.nrec = s.nrec;
    h.src_kind = s.src_where == SRC_NONE ? -1 : s.src.kind;
    h.src_ix = s.src_where == SRC_NONE ? 0 : s.src.ix;
    h.src_iz = s.src_where == SRC_NONE ? 0 : s.src.iz;
    h.f0 = s.src_where == SRC_NONE ? 0.0f : s.src.f0;
    h.amplitude = s.src_where == SRC_NONE ? 0.0f : s.src.amplitude;
    h.t_cut = s.src_where == SRC_NONE ? 0.0 : s.src.t_cut;
    h.dx = ctx->g.dx;
    h.dz = ctx->g.dz;
    h.dt = ctx->g.dt;
    h.prof_hash = ctx->prof_hash;
    h.rec_hash = s.rec_hash;
    return coef_hash(ctx, &h.coef_hash);
}

bool same_bits(float a, float b) { return std::memcmp(&a, &b, 4) == 0; }
}  // namespace

int poe_checkpoint_info(const void *host_buf, int64_t size, poe_checkpoint_header *out)
{
    if (!host_buf || size < (int64_t)sizeof(CkHeader)) return POE_EINVAL;
    CkHeader h;
    std::memcpy(&h, host_buf, sizeof h);
    if (std::memcmp(h.magic, kCkMagic, 8) || h.version != POE_CHECKPOINT_VERSION ||
        h.header_bytes != sizeof(CkHeader) || h.payload_bytes < 0 ||
        size - (int64_t)sizeof(CkHeader) < h.payload_bytes)
        return POE_EINVAL;
    if (ck_sum(static_cast<const unsigned char *>(host_buf) + sizeof(CkHeader), (size_t)h.payload_bytes) !=
        h.checksum)
        return POE_EIO;
    if (out) *out = h;
    return POE_OK;
}

int poe_checkpoint_size(poe_ctx *ctx, int32_t shot, int64_t *bytes)
{
    ShotHost *s = get_shot(ctx, shot);
    if (!s || !bytes) return fail(ctx, POE_EINVAL, "shot id");
    *bytes = (int64_t)(sizeof(CkHeader) + ck_payload(ck_parts(ctx, *s)));
    return POE_OK;
}

int poe_checkpoint_save(poe_ctx *ctx, int32_t shot, void *host_buf, int64_t capacity)
{
    ShotHost *s = get_shot(ctx, shot);
    if (!s) return fail(ctx, POE_EINVAL, "shot id");
    const CkParts c = ck_parts(ctx, *s);
    const size_t need = sizeof(CkHeader) + ck_payload(c);
    if (!host_buf || capacity < (int64_t)need) return fail(ctx, POE_EINVAL, "checkpoint buffer too small");
    CK(cudaSetDevice(ctx->device));
    const int b = (int)(s->steps & 1);
    unsigned char *p = static_cast<unsigned char *>(host_buf) + sizeof(CkHeader);
    auto get = [&](const void *src, size_t n) -> int {
        if (n) CK(cudaMemcpyAsync(p, src, n, cudaMemcpyDeviceToHost, ctx->stream));
        p += n;
        return POE_OK;
    };
    int rc;
    if ((rc = get(s->f[b], c.f)) || (rc = get(s->mx[b], c.x)) || (rc = get(s->mxv, c.x)) ||
        (rc = get(s->mz[b], c.z)) || (rc = get(s->mzv, c.z)))
        return rc;
    std::memset(p, 0, c.acc);
    if ((rc = get(s->acc + b, sizeof(float)))) return rc;
    p += c.acc - sizeof(float);
    if ((rc = get(s->trace, c.tr))) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    if ((rc = device_status(ctx)) != POE_OK) return rc;
    CkHeader h;
    if ((rc = ck_fill_header(ctx, *s, h)) != POE_OK) return rc;
    h.payload_bytes = (int64_t)ck_payload(c);
    h.checksum = ck_sum(static_cast<unsigned char *>(host_buf) + sizeof(CkHeader), ck_payload(c));
    std::memcpy(host_buf, &h, sizeof h);
    return POE_OK;
}

int poe_checkpoint_load(poe_ctx *ctx, int32_t shot, const void *host_buf, int64_t size)
{
    ShotHost *s = get_shot(ctx, shot);
    if (!s) return fail(ctx, POE_EINVAL, "shot id");
    if (!host_buf || size < (int64_t)sizeof(CkHeader)) return fail(ctx, POE_EINVAL, "checkpoint too short");
    CkHeader h, want;
    std::memcpy(&h, host_buf, sizeof h);
    if (std::memcmp(h.magic, kCkMagic, 8) || h.version != POE_CHECKPOINT_VERSION || h.header_bytes != sizeof(CkHeader))
        return fail(ctx, POE_EINVAL, "not a poe2d checkpoint of version " + std::to_string(POE_CHECKPOINT_VERSION));
    int rc;
    if ((rc = ck_fill_header(ctx, *s, want)) != POE_OK) return rc;
    if (h.NX != want.NX || h.NZ != want.NZ || h.P != want.P || h.R != want.R || h.Wx != want.Wx ||
        h.Hz != want.Hz || h.plane != want.plane)
        return fail(ctx, POE_EINVAL, "checkpoint of another grid or C-PML layout");
    if (!same_bits(h.dx, want.dx) || !same_bits(h.dz, want.dz) || !same_bits(h.dt, want.dt))
        return fail(ctx, POE_EINVAL, "checkpoint of another grid spacing or time step");
    if (h.prof_hash != want.prof_hash) return fail(ctx, POE_EINVAL, "checkpoint of other C-PML profiles");
    if (h.coef_hash != want.coef_hash) return fail(ctx, POE_EINVAL, "checkpoint of another model (coefficients)");
    if (h.nrec != want.nrec || h.rec_hash != want.rec_hash || h.src_kind != want.src_kind ||
        h.src_ix != want.src_ix || h.src_iz != want.src_iz || h.f0 != want.f0 || h.amplitude != want.amplitude ||
        h.t_cut != want.t_cut)
        return fail(ctx, POE_EINVAL, "checkpoint of another shot (source or receivers differ)");
    if (h.steps < 0) return fail(ctx, POE_EINVAL, "checkpoint step count");
    const int64_t keep = s->steps;
    s->steps = h.steps;
    const CkParts c = ck_parts(ctx, *s);
    s->steps = keep;
    if (h.payload_bytes != (int64_t)ck_payload(c) || size < (int64_t)(sizeof(CkHeader) + ck_payload(c)))
        return fail(ctx, POE_EINVAL, "checkpoint size");
    const unsigned char *p = static_cast<const unsigned char *>(host_buf) + sizeof(CkHeader);
    if (ck_sum(p, ck_payload(c)) != h.checksum) return fail(ctx, POE_EIO, "checkpoint checksum mismatch");
    if ((rc = poe_reset_shot(ctx, shot)) != POE_OK) return rc;   // both buffers and traces zero, clock 0
    if ((rc = ensure_trace(ctx, *s, h.steps)) != POE_OK) return rc;
    const int b = (int)(h.steps & 1);
    auto put = [&](void *dst, size_t n) -> int {
        if (n) CK(cudaMemcpyAsync(dst, p, n, cudaMemcpyHostToDevice, ctx->stream));
        p += n;
        return POE_OK;
    };
    if ((rc = put(s->f[b], c.f)) || (rc = put(s->mx[b], c.x)) || (rc = put(s->mxv, c.x)) ||
        (rc = put(s->mz[b], c.z)) || (rc = put(s->mzv, c.z)) || (rc = put(s->acc + b, sizeof(float))))
        return rc;
    p += c.acc - sizeof(float);
    if ((rc = put(s->trace, c.tr))) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    s->steps = h.steps;
    ctx->shots_dirty = true;
    return sync_shots(ctx);
}

int poe_tune(poe_ctx *ctx, int32_t order, int32_t graph_steps)
{
    if (!ctx) return POE_EINVAL;
    if (order < POE_ORDER_ROWS || order > POE_ORDER_BALANCED || graph_steps < 1 || graph_steps > 4096)
        return fail(ctx, POE_EINVAL, "tuning: order or graph_steps out of range");
    if (order != ctx->order) ctx->shots_dirty = true;   // rebuilds the work list (and the graph)
    if (graph_steps != ctx->graph_steps) drop_graph(ctx);
    ctx->order = order;
    ctx->graph_steps = graph_steps;
    return POE_OK;
}

int poe_tune_span(poe_ctx *ctx, int32_t span)
{
    if (!ctx) return POE_EINVAL;
    if (span != POE_SPAN_NEVER && span != POE_SPAN_ALWAYS && span != POE_SPAN_AUTO)
        return fail(ctx, POE_EINVAL, "tuning: span must be POE_SPAN_NEVER, POE_SPAN_ALWAYS or POE_SPAN_AUTO");
    if (span != ctx->span) drop_graph(ctx);
    ctx->span = span;
    return POE_OK;
}

int poe_tune_tile(poe_ctx *ctx, int32_t tile_z)
{
    if (!ctx) return POE_EINVAL;
    if (tile_z != PAL_TZ && tile_z != PAL_TZ_SMALL)
        return fail(ctx, POE_EINVAL, "tuning: tile_z must be 32 or 16");
    if (tile_z == ctx->tile_z) return POE_OK;
    if (tile_z == PAL_TZ_SMALL && ctx->exact)
        return fail(ctx, POE_EINVAL, "tuning: 16-row tiles are built for FAST stencils only");
    if (ctx->batch) return fail(ctx, POE_ESTATE, "tuning: the context belongs to a batch (32-row tiles)");
    CK(cudaStreamSynchronize(ctx->stream));   // no launch still reads the old work list
    drop_graph(ctx);
    set_tile(ctx, tile_z);
    // the flags are indexed by tile: start the new tiling from zero (never ahead of a shot)
    for (ShotHost &sh : ctx->shots) CK(cudaMemsetAsync(sh.done, 0, sizeof(int) * ctx->ncell_max, ctx->stream));
    return sync_shots(ctx);
}

int poe_tuning(const poe_ctx *ctx, int32_t *order, int32_t *graph_steps, int32_t *span, int32_t *tile_z)
{
    if (!ctx) return POE_EINVAL;
    if (order) *order = ctx->order;
    if (graph_steps) *graph_steps = ctx->graph_steps;
    if (span) *span = ctx->span;
    if (tile_z) *tile_z = ctx->tile_z;
    return POE_OK;
}

int poe_autotune(poe_ctx *ctx, int32_t trial_steps, int32_t *order_out, int32_t *graph_steps_out, float *ms_out)
{
    if (!ctx || trial_steps < 1) return POE_EINVAL;
    if (ctx->shots.empty()) return fail(ctx, POE_ESTATE, "autotune: no shots");
    for (const ShotHost &s : ctx->shots)
        if (s.steps != 0) return fail(ctx, POE_ESTATE, "autotune: every shot must be at step 0 (it is reset after)");
    CK(cudaSetDevice(ctx->device));
    static const int32_t kSteps[2] = {16, 64};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    int best = -1, rc = POE_OK;
    float best_ms = 0.0f;
    // 16-row tiles: FAST contexts outside a batch
    const bool small_ok = !ctx->exact && !ctx->batch;
    // candidate c: tile height {32, 16}[c / 16], order (c / 4) % 4, graph length
    // kSteps[(c / 2) % 2], span c % 2
    for (int c = 0; c < POE_AUTOTUNE_CANDIDATES && rc == POE_OK; ++c) {
        const int tz = c / 16 ? PAL_TZ_SMALL : PAL_TZ, order = (c / 4) % 4, gs = kSteps[(c / 2) % 2], span = c % 2;
        if (tz == PAL_TZ_SMALL && !small_ok) {
            if (ms_out) ms_out[c] = -1.0f;    // not a candidate for this context
            continue;
        }
        if ((rc = poe_tune_tile(ctx, tz)) != POE_OK || (rc = poe_tune(ctx, order, gs)) != POE_OK ||
            (rc = poe_tune_span(ctx, span)) != POE_OK)
            break;
        if ((rc = poe_run(ctx, gs)) != POE_OK) break;        // capture the graph, first touch
        cudaEventRecord(e0, ctx->stream);
        if ((rc = poe_run(ctx, trial_steps)) != POE_OK) break;
        cudaEventRecord(e1, ctx->stream);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            rc = fail(ctx, POE_ECUDA, "autotune: event");
            break;
        }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms_out) ms_out[c] = ms;
        if (best < 0 || ms < best_ms) {
            best = c;
            best_ms = ms;
        }
        if ((rc = device_status(ctx)) != POE_OK) break;
        for (int i = 0; i < (int)ctx->shots.size() && rc == POE_OK; ++i) rc = poe_reset_shot(ctx, i);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != POE_OK) return rc;
    if ((rc = poe_tune_tile(ctx, best / 16 ? PAL_TZ_SMALL : PAL_TZ)) != POE_OK) return rc;
    if ((rc = poe_tune(ctx, (best / 4) % 4, kSteps[(best / 2) % 2])) != POE_OK) return rc;
    rc = poe_tune_span(ctx, best % 2);
    if (order_out) *order_out = (best / 4) % 4;
    if (graph_steps_out) *graph_steps_out = kSteps[(best / 2) % 2];
    return rc;
}

int poe_check_finite(poe_ctx *ctx, int32_t shot, float threshold, float *max_abs_out)
{
    ShotHost *s = get_shot(ctx, shot);
    if (!s) return fail(ctx, POE_EINVAL, "shot id");
    const ModelDev &m = ctx->m;
    std::vector<float> h((size_t)m.plane * NSF);
    CK(cudaMemcpyAsync(h.data(), s->f[s->steps & 1], sizeof(float) * h.size(), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    float mx = 0.0f;
    bool bad = false;
    for (float v : h) {
        if (!std::isfinite(v)) bad = true;
        else mx = std::max(mx, std::fabs(v));
    }
    if (max_abs_out) *max_abs_out = bad ? INFINITY : mx;
    if (bad || (threshold > 0.0f && mx > threshold))
        return fail(ctx, POE_ENONFINITE, "field not finite or above threshold");
    return POE_OK;
}

int poe_kernel_launches(const poe_ctx *ctx, int64_t *count)
{
    if (!ctx || !count) return POE_EINVAL;
    *count = ctx->launches;
    return POE_OK;
}

const char *poe_last_error(const poe_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

void poe_destroy(poe_ctx *ctx)
{
    if (!ctx) return;
    if (ctx->batch) batch_forget(ctx->batch, ctx);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    drop_graph(ctx);
    for (ShotHost &s : ctx->shots) free_shot(s);
    cudaFree(ctx->shots_dev);
    cudaFree(ctx->steps_dev);
    cudaFree(ctx->items_dev);
    cudaFree(ctx->coef);
    cudaFree(ctx->px);
    cudaFree(ctx->pz);
    cudaFree(ctx->derived);
    cudaFree(ctx->err_dev);
    cudaFree(ctx->queue_dev);
    cudaFree(ctx->ids);
    cudaFree(ctx->mtab);
    cudaFree(ctx->tm_model);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

}  // extern "C"

// ---------------------------------------------------------------- batches
//
// A batch concatenates the work lists of its contexts: item (model, shot, x0,
// z0) with model indexing the batch's ModelDev array and shot its StreamShot
// array.  Contexts are ordered by steps requested (most first), so the items of
// the contexts still running are always a prefix of the list: a run is a few
// segments, each launching over a shorter prefix, and no kernel tests whether
// its model is finished.

struct poe_batch {
    std::vector<poe_ctx *> ctxs;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int device = 0;
    bool exact = true, kone = true, few = true;
    bool coef = false;          // the models read their coefficient planes per cell
    int span = POE_SPAN_AUTO;   // step-spanning launches (POE_SPAN_*)
    ModelDev *models_dev = nullptr;
    StreamShot *shots_dev = nullptr;
    int4 *items_dev = nullptr;
    int *queue_dev = nullptr;   // the step kernel's work queue (2 ints, zero between launches)
    int models_cap = 0, shots_cap = 0, items_cap = 0;
    std::vector<std::array<int, 2>> graph_keys;   // (items, shots) prefix of each graph
    std::vector<cudaGraphExec_t> graphs;
    std::vector<int64_t> graph_kernels;            // kernels one walk of each graph launches
    cudaEvent_t done = nullptr;
    int64_t launches = 0;
    bool orphaned = false;      // a member context was destroyed: the batch no longer runs
    std::string err;
};

namespace {

int bfail(poe_batch *b, int code, const std::string &msg)
{
    if (b) b->err = msg;
    return code;
}

#define BK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return bfail(b, e_ == cudaErrorMemoryAllocation ? POE_ENOMEM : POE_ECUDA,    \
                         std::string(#call) + ": " + cudaGetErrorString(e_));            \
    } while (0)

void batch_forget(poe_batch *b, poe_ctx *ctx)
{
    b->ctxs.erase(std::remove(b->ctxs.begin(), b->ctxs.end(), ctx), b->ctxs.end());
    b->orphaned = true;
    ctx->batch = nullptr;
}

void drop_batch_graphs(poe_batch *b)
{
    for (cudaGraphExec_t g : b->graphs) cudaGraphExecDestroy(g);
    b->graphs.clear();
    b->graph_keys.clear();
    b->graph_kernels.clear();
}

template <class T>
int grow(poe_batch *b, T **p, int &cap, int need)
{
    if (need <= cap) return POE_OK;
    drop_batch_graphs(b);   // graphs hold the old pointers
    const int c = std::max(need, 2 * cap);
    cudaFree(*p);
    *p = nullptr;
    cap = 0;
    BK(cudaMalloc(p, sizeof(T) * c));
    cap = c;
    return POE_OK;
}

// the batch's launches for nsteps steps over the first nitems items (one
// step-spanning launch, or one per step); returns the launches or -1
int64_t batch_issue(poe_batch *b, int nitems, int64_t nsteps)
{
    const bool span = nsteps > 1 && (b->span == POE_SPAN_ALWAYS ||
                                     (b->span == POE_SPAN_AUTO && nitems <= kSpanTilesPerSM * device_sms(b->device)));
    const int64_t nl = span ? 1 : nsteps;
    for (int64_t k = 0; k < nl; ++k) {
        const int r = launch_batch_step(b->models_dev, b->shots_dev, b->items_dev, nitems, (int)k,
                                        span ? (int)nsteps : 1, b->exact, b->few, b->coef, b->kone, b->queue_dev,
                                        b->stream);
        if (r) return bfail(b, POE_ECUDA, std::string("kernel launch: ") + cudaGetErrorString((cudaError_t)r)), -1;
    }
    return nl;
}

int batch_steps(poe_batch *b, int nitems, int nshots, int64_t nsteps)
{
    const int64_t l = batch_issue(b, nitems, nsteps);
    if (l < 0) return POE_ECUDA;
    const int r = launch_advance_shots(b->shots_dev, nshots, nsteps, b->stream);
    if (r) return bfail(b, POE_ECUDA, std::string("kernel launch: ") + cudaGetErrorString((cudaError_t)r));
    b->launches += l + 1;
    return POE_OK;
}

// the graph of kGraphSteps steps over the first nitems items, captured on
// first use; *kernels = the kernels one walk of it launches
cudaGraphExec_t batch_graph(poe_batch *b, int nitems, int nshots, int64_t *kernels)
{
    for (size_t i = 0; i < b->graph_keys.size(); ++i)
        if (b->graph_keys[i][0] == nitems && b->graph_keys[i][1] == nshots) {
            *kernels = b->graph_kernels[i];
            return b->graphs[i];
        }
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return nullptr;
    const int64_t l = batch_issue(b, nitems, kGraphSteps);
    int rc = l < 0 ? 1 : 0;
    if (rc == 0) rc = launch_advance_shots(b->shots_dev, nshots, kGraphSteps, b->stream);
    const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (rc != 0 || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return nullptr;
    }
    cudaGraphExec_t x = nullptr;
    const cudaError_t ei = cudaGraphInstantiate(&x, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) return nullptr;
    b->graph_keys.push_back({nitems, nshots});
    b->graphs.push_back(x);
    b->graph_kernels.push_back(l + 1);
    *kernels = l + 1;
    return x;
}

int batch_segment(poe_batch *b, int nitems, int nshots, int64_t nsteps)
{
    int64_t left = nsteps;
    if (left >= kGraphSteps) {
        int64_t kernels = 0;
        cudaGraphExec_t g = batch_graph(b, nitems, nshots, &kernels);
        if (!g) return bfail(b, POE_ECUDA, "batch graph capture failed");
        for (; left >= kGraphSteps; left -= kGraphSteps) {
            BK(cudaGraphLaunch(g, b->stream));
            b->launches += kernels;
        }
    }
    return left > 0 ? batch_steps(b, nitems, nshots, left) : POE_OK;
}

}  // namespace

extern "C" {

int poe_batch_create(poe_ctx *const *ctxs, int32_t n, void *stream, poe_batch **out)
{
    if (!out) return POE_EINVAL;
    *out = nullptr;
    if (!ctxs || n <= 0) return POE_EINVAL;
    for (int i = 0; i < n; ++i) {
        if (!ctxs[i]) return POE_EINVAL;
        if ((ctxs[i]->ids == nullptr) != (ctxs[0]->ids == nullptr))
            return fail(ctxs[i], POE_EINVAL, "batch: palette models and per-cell coefficient models in one batch");
        if (ctxs[i]->device != ctxs[0]->device) return fail(ctxs[i], POE_EINVAL, "batch: contexts on other devices");
        if (ctxs[i]->exact != ctxs[0]->exact) return fail(ctxs[i], POE_EINVAL, "batch: mixed stencil modes");
        if (ctxs[i]->tile_z != PAL_TZ)
            return fail(ctxs[i], POE_EINVAL, "batch: a context tuned to 16-row tiles (batches run 32-row tiles)");
        for (int j = 0; j < i; ++j)
            if (ctxs[j] == ctxs[i]) return fail(ctxs[i], POE_EINVAL, "batch: context listed twice");
        if (ctxs[i]->batch) return fail(ctxs[i], POE_ESTATE, "batch: context already belongs to a batch");
    }
    poe_batch *b = new poe_batch;
    b->ctxs.assign(ctxs, ctxs + n);
    b->device = ctxs[0]->device;
    b->exact = ctxs[0]->exact;
    b->coef = ctxs[0]->ids == nullptr;
    b->span = ctxs[0]->span;
    for (poe_ctx *c : b->ctxs) b->kone = b->kone && c->kone;   // K = 1 divides are exact: KONE=false is safe
    for (poe_ctx *c : b->ctxs) b->few = b->few && c->m.qx.few_bits && c->m.qz.few_bits;
    if (cudaSetDevice(b->device) != cudaSuccess) {
        delete b;
        return POE_ECUDA;
    }
    if (stream) {
        b->stream = (cudaStream_t)stream;
    } else if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess) {
        b->own_stream = true;
    } else {
        delete b;
        return POE_ECUDA;
    }
    if (cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) != cudaSuccess ||
        cudaMalloc(&b->queue_dev, 2 * sizeof(int)) != cudaSuccess ||
        cudaMemsetAsync(b->queue_dev, 0, 2 * sizeof(int), b->stream) != cudaSuccess) {
        poe_batch_destroy(b);
        return POE_ECUDA;
    }
    for (poe_ctx *c : b->ctxs) c->batch = b;
    *out = b;
    return POE_OK;
}

int poe_batch_run(poe_batch *b, const int64_t *nsteps)
{
    if (!b) return POE_EINVAL;
    if (b->orphaned) return bfail(b, POE_ESTATE, "a context of this batch was destroyed");
    if (!nsteps) return bfail(b, POE_EINVAL, "nsteps");
    const int n = (int)b->ctxs.size();
    for (int i = 0; i < n; ++i) {
        if (nsteps[i] < 0) return bfail(b, POE_EINVAL, "nsteps < 0");
        if (nsteps[i] > 0 && b->ctxs[i]->shots.empty()) return bfail(b, POE_ESTATE, "a context has no shots");
    }
    BK(cudaSetDevice(b->device));
    BK(cudaStreamSynchronize(b->stream));   // the previous run still reads the work list
    std::vector<int> order;
    for (int i = 0; i < n; ++i) {
        if (nsteps[i] == 0) continue;
        poe_ctx *ctx = b->ctxs[i];
        int rc;
        for (ShotHost &s : ctx->shots) {
            if ((rc = ensure_trace(ctx, s, s.steps + nsteps[i])) != POE_OK) return bfail(b, rc, ctx->err);
            if ((rc = ensure_source(ctx, s, s.steps + nsteps[i])) != POE_OK) return bfail(b, rc, ctx->err);
        }
        if ((rc = sync_shots(ctx)) != POE_OK) return bfail(b, rc, ctx->err);
        BK(cudaStreamSynchronize(ctx->stream));   // earlier work on the context's own stream
        order.push_back(i);
    }
    if (order.empty()) return POE_OK;
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return nsteps[a] > nsteps[c]; });

    // concatenated work list; item_end[p] / shot_end[p]: prefix sizes through context order[p]
    std::vector<ModelDev> hm;
    std::vector<StreamShot> hs;
    std::vector<int4> hi;
    std::vector<int> item_end, shot_end;
    for (int p = 0; p < (int)order.size(); ++p) {
        const poe_ctx *ctx = b->ctxs[order[p]];
        const int shot0 = (int)hs.size();
        hm.push_back(ctx->m);
        hs.insert(hs.end(), ctx->shots_host.begin(), ctx->shots_host.end());
        for (int4 it : ctx->items) hi.push_back(make_int4(p, shot0 + it.y, it.z, it.w));
        item_end.push_back((int)hi.size());
        shot_end.push_back((int)hs.size());
    }
    int rc;
    if ((rc = grow(b, &b->models_dev, b->models_cap, (int)hm.size())) != POE_OK) return rc;
    if ((rc = grow(b, &b->shots_dev, b->shots_cap, (int)hs.size())) != POE_OK) return rc;
    if ((rc = grow(b, &b->items_dev, b->items_cap, (int)hi.size())) != POE_OK) return rc;
    BK(cudaMemcpyAsync(b->models_dev, hm.data(), sizeof(ModelDev) * hm.size(), cudaMemcpyHostToDevice, b->stream));
    BK(cudaMemcpyAsync(b->shots_dev, hs.data(), sizeof(StreamShot) * hs.size(), cudaMemcpyHostToDevice, b->stream));
    BK(cudaMemcpyAsync(b->items_dev, hi.data(), sizeof(int4) * hi.size(), cudaMemcpyHostToDevice, b->stream));
    BK(cudaStreamSynchronize(b->stream));   // host vectors go out of scope

    int64_t done = 0;
    for (int p = (int)order.size() - 1; p >= 0; --p) {   // segment: contexts order[0..p] still running
        const int64_t until = nsteps[order[p]];
        if (until > done) {
            if ((rc = batch_segment(b, item_end[p], shot_end[p], until - done)) != POE_OK) return rc;
            done = until;
        }
    }
    BK(cudaEventRecord(b->done, b->stream));
    for (int i : order) {
        poe_ctx *ctx = b->ctxs[i];
        BK(cudaStreamWaitEvent(ctx->stream, b->done, 0));
        for (ShotHost &s : ctx->shots) s.steps += nsteps[i];
    }
    return POE_OK;
}

int poe_batch_tune_span(poe_batch *b, int32_t span)
{
    if (!b) return POE_EINVAL;
    if (span != POE_SPAN_NEVER && span != POE_SPAN_ALWAYS && span != POE_SPAN_AUTO)
        return bfail(b, POE_EINVAL, "tuning: span must be POE_SPAN_NEVER, POE_SPAN_ALWAYS or POE_SPAN_AUTO");
    if (span != b->span) {
        BK(cudaStreamSynchronize(b->stream));   // a graph still running holds the old launches
        drop_batch_graphs(b);
    }
    b->span = span;
    return POE_OK;
}

int poe_batch_sync(poe_batch *b)
{
    if (!b) return POE_EINVAL;
    BK(cudaStreamSynchronize(b->stream));
    for (poe_ctx *ctx : b->ctxs) {
        const int rc = device_status(ctx);
        if (rc != POE_OK) {
            // a launch that gave up may have left the batch's work queue mid-way
            BK(cudaMemsetAsync(b->queue_dev, 0, 2 * sizeof(int), b->stream));
            BK(cudaStreamSynchronize(b->stream));
            return bfail(b, rc, ctx->err);
        }
    }
    return POE_OK;
}

int poe_batch_launches(const poe_batch *b, int64_t *count)
{
    if (!b || !count) return POE_EINVAL;
    *count = b->launches;
    return POE_OK;
}

const char *poe_batch_last_error(const poe_batch *b) { return b ? b->err.c_str() : "null batch"; }

void poe_batch_destroy(poe_batch *b)
{
    if (!b) return;
    for (poe_ctx *c : b->ctxs)   // destroyed members already left the list
        if (c->batch == b) c->batch = nullptr;
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_batch_graphs(b);
    cudaFree(b->models_dev);
    cudaFree(b->shots_dev);
    cudaFree(b->items_dev);
    cudaFree(b->queue_dev);
    if (b->done) cudaEventDestroy(b->done);
    if (b->own_stream) cudaStreamDestroy(b->stream);
    delete b;
}

}  // extern "C"
