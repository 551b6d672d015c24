// sg_net.cpp -- the surrogate network's runtime behind poe2d_surrogate.h:
// layer table, parameter and activation buffers, forward, backward and Adam
// as sequences of launches of the tcgen05 GEMM (sg_gemm.cu) and the layer
// kernels (sg_ops.cu) on one stream.
//
// Every layer is a GEMM over an im2col matrix (channels last):
//   forward   out[M, Cout] = col[M, Kp] . W[Cout, Kp]^T + b  (ReLU)
//             (the time convolutions read their input in place instead:
//             sg::gemm_conv1d, one GEMM per phase of the upsampled axis)
//   backward  dZ = dOut * (out > 0)
//             dW[Cout, Kp] = dZ^T . col         (GEMM of dZ^T and col^T, K = M)
//             db = column sums of dZ
//             dcol[M, Kp] = dZ . W              (GEMM of dZ and W^T, K = Cout)
//             dX = col2im(dcol)
// Kp is the layer's reduction length rounded up to 64 (zero columns).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/poe2d_surrogate.h"
#include "sg_internal.h"
#include "sg_ops.h"

namespace {

enum Kind { CONV2D, FC, CONV1D };

struct Layer {
    Kind kind;
    int cin, cout, k, kp;      // k: real reduction length, kp: padded
    int h, w;                  // conv2d: input height / width
    int t, up;                 // conv1d: input length, upsampling
    bool relu;
    int64_t rows_per_item;     // output rows per batch item
    int64_t w_off, b_off;      // in the flat parameter arrays
    __nv_bfloat16 *col = nullptr;   // GEMM A operand [B*rows, kp] (FC: the input itself)
    __nv_bfloat16 *out = nullptr;   // [B*rows, cout] (last layer: FP32 output elsewhere)
};

constexpr int kCat = 4096 + 64;       // flattened encoder output + scalars, padded

int rup(int v, int m) { return (v + m - 1) / m * m; }

struct Rng {   // splitmix64 + Box-Muller: He-normal initial weights
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    double uni() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
    double normal()
    {
        const double u = uni(), v = uni();
        return std::sqrt(-2.0 * std::log(u)) * std::cos(6.283185307179586 * v);
    }
};

}  // namespace

struct poe_sg {
    int bmax = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::vector<Layer> L;
    int64_t nparam = 0;          // flat length (weights incl. padding columns + biases)
    float *w32 = nullptr, *g32 = nullptr, *m32 = nullptr, *v32 = nullptr;
    __nv_bfloat16 *w16 = nullptr;
    float *out = nullptr;        // [bmax*1024, 384]
    __nv_bfloat16 *cat = nullptr, *dout = nullptr;
    __nv_bfloat16 *s_dz = nullptr, *s_dzt = nullptr, *s_colt = nullptr, *s_wt = nullptr, *s_dcol = nullptr;
    __nv_bfloat16 *s_dx[2] = {nullptr, nullptr};
    float *ws = nullptr;
    int64_t ws_floats = 0;
    float *partial = nullptr, *loss_dev = nullptr, *colpart = nullptr;
    int *err = nullptr;
    int adam_t = 0;
    int64_t launches = 0;
    std::vector<void *> allocs;
    std::string errmsg;
};

namespace {

int fail(poe_sg *n, int code, const std::string &m)
{
    if (n) n->errmsg = m;
    return code;
}

#define SK(call)                                                                                    \
    do {                                                                                            \
        const int r_ = (int)(call);                                                                 \
        if (r_ != 0)                                                                                \
            return fail(net, r_ == (int)cudaErrorMemoryAllocation ? 6 : 5,                          \
                        std::string(#call) + ": " + cudaGetErrorString((cudaError_t)r_));           \
        ++net->launches;                                                                            \
    } while (0)

template <class T>
int alloc(poe_sg *net, T **p, int64_t n)
{
    void *q = nullptr;
    const cudaError_t e = cudaMalloc(&q, sizeof(T) * (size_t)std::max<int64_t>(n, 1));
    if (e != cudaSuccess) return fail(net, 6, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    net->allocs.push_back(q);
    *p = static_cast<T *>(q);
    return 0;
}

void build_layers(poe_sg *net)
{
    auto conv2d = [&](int cin, int cout, int h) {
        Layer l{};
        l.kind = CONV2D;
        l.cin = cin;
        l.cout = cout;
        l.k = 9 * cin;
        l.kp = rup(l.k, 64);
        l.h = l.w = h;
        l.relu = true;
        l.rows_per_item = (int64_t)(h / 2) * (h / 2);
        net->L.push_back(l);
    };
    auto fc = [&](int cin, int kp, int cout) {
        Layer l{};
        l.kind = FC;
        l.cin = cin;
        l.cout = cout;
        l.k = cin;
        l.kp = kp;
        l.relu = true;
        l.rows_per_item = 1;
        net->L.push_back(l);
    };
    auto conv1d = [&](int cin, int cout, int t, int up, bool relu) {
        Layer l{};
        l.kind = CONV1D;
        l.cin = cin;
        l.cout = cout;
        l.k = 3 * cin;
        l.kp = rup(l.k, 64);
        l.t = t;
        l.up = up;
        l.relu = relu;
        l.rows_per_item = (int64_t)t * up;
        net->L.push_back(l);
    };
    conv2d(2, 64, 64);
    conv2d(64, 128, 32);
    conv2d(128, 128, 16);
    conv2d(128, 256, 8);
    fc(4096 + POE_SG_SCALARS, kCat, 256);
    fc(256, 256, 2048);
    conv1d(128, 128, 16, 2, true);
    conv1d(128, 128, 32, 2, true);
    conv1d(128, 128, 64, 2, true);
    conv1d(128, 64, 128, 2, true);
    conv1d(64, 64, 256, 2, true);
    conv1d(64, 64, 512, 2, true);
    conv1d(64, POE_SG_CHANNELS, 1024, 1, false);
    int64_t off = 0;
    for (Layer &l : net->L) {
        l.w_off = off;
        off += (int64_t)l.cout * l.kp;
        l.b_off = off;
        off += rup(l.cout, 8);
    }
    net->nparam = off;
}

int64_t real_count(const poe_sg *net)
{
    int64_t n = 0;
    for (const Layer &l : net->L) n += (int64_t)l.cout * l.k + l.cout;
    return n;
}

int gemm_call(poe_sg *net, const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, int M, int N, int K,
              const sg::Epilogue &e)
{
    sg::Gemm g{A, lda, B, ldb, M, N, K};
    SK(sg::gemm(g, e, net->ws, net->ws_floats, net->err, net->stream));
    return 0;
}

int forward(poe_sg *net, const __nv_bfloat16 *maps, const float *scalars, int B, float *out)
{
    const cudaStream_t st = net->stream;
    const __nv_bfloat16 *x = maps;
    for (size_t i = 0; i < net->L.size(); ++i) {
        Layer &l = net->L[i];
        const int64_t M = (int64_t)B * l.rows_per_item;
        const __nv_bfloat16 *A = l.col;
        if (l.kind == CONV1D) {
            // the time convolutions read x in place, one GEMM per output phase of
            // the upsampled axis (no im2col matrix; backward builds it)
            sg::Epilogue e;
            e.bias = net->w32 + l.b_off;
            e.relu = l.relu;
            e.ldc = l.cout;
            if (i + 1 == net->L.size()) e.out_f32 = out;
            else e.out_bf16 = l.out;
            for (int p = 0; p < l.up; ++p)
                SK(sg::gemm_conv1d(x, B, l.t, l.cin, l.up, p, net->w16 + l.w_off, l.cout, e, net->err, st));
            x = l.out;
            continue;
        }
        if (l.kind == CONV2D) {
            SK(sg::im2col2d(x, B, l.h, l.w, l.cin, l.col, l.kp, st));
        } else if (i == 4) {   // first FC: flattened encoder output | scalars
            SK(sg::concat(x, 4096, scalars, POE_SG_SCALARS, B, net->cat, kCat, st));
            A = net->cat;
        } else {
            A = x;
        }
        sg::Epilogue e;
        e.bias = net->w32 + l.b_off;
        e.relu = l.relu;
        e.ldc = l.cout;
        if (i + 1 == net->L.size()) e.out_f32 = out;
        else e.out_bf16 = l.out;
        int rc = gemm_call(net, A, l.kp, net->w16 + l.w_off, l.kp, (int)M, l.cout, l.kp, e);
        if (rc) return rc;
        x = l.out;
    }
    return 0;
}

int backward(poe_sg *net, int B)
{
    const cudaStream_t st = net->stream;
    // dY of the current layer's output (bf16, pitch ldy)
    const __nv_bfloat16 *dy = net->dout;
    int ldy = POE_SG_CHANNELS;
    int flip = 0;
    for (int i = (int)net->L.size() - 1; i >= 0; --i) {
        Layer &l = net->L[i];
        const int64_t M = (int64_t)B * l.rows_per_item;
        const __nv_bfloat16 *dz = dy;
        if (l.relu) {
            SK(sg::relu_bwd(dy, ldy, l.out, (i == 3 ? B : M), (i == 3 ? 4096 : l.cout), net->s_dz, st));
            dz = net->s_dz;
        }
        // bias gradient
        SK(sg::colsum(dz, M, l.cout, l.cout, net->g32 + l.b_off, net->colpart, st));
        // a time convolution's im2col matrix (forward reads its input in place)
        if (l.kind == CONV1D) SK(sg::im2col1d(net->L[i - 1].out, B, l.t, l.cin, l.up, l.col, l.kp, st));
        // weight gradient: dZ^T [cout x M] . A^T [kp x M]
        const __nv_bfloat16 *A = l.kind == FC ? (i == 4 ? net->cat : net->L[i - 1].out) : l.col;
        SK(sg::transpose(dz, M, l.cout, l.cout, net->s_dzt, M, st));
        SK(sg::transpose(A, M, l.kp, l.kp, net->s_colt, M, st));
        sg::Epilogue ew;
        ew.out_f32 = net->g32 + l.w_off;
        ew.ldc = l.kp;
        int rc = gemm_call(net, net->s_dzt, (int)M, net->s_colt, (int)M, l.cout, l.kp, (int)M, ew);
        if (rc) return rc;
        if (i == 0) break;
        // input gradient: dcol = dZ [M x cout] . (W^T)^T, W^T [kp x cout]
        SK(sg::transpose(net->w16 + l.w_off, l.cout, l.kp, l.kp, net->s_wt, l.cout, st));
        sg::Epilogue ex;
        __nv_bfloat16 *dx = net->s_dx[flip];
        flip ^= 1;
        ex.ldc = l.kp;
        ex.out_bf16 = l.kind == FC ? dx : net->s_dcol;
        rc = gemm_call(net, dz, l.cout, net->s_wt, l.cout, (int)M, l.kp, l.cout, ex);
        if (rc) return rc;
        // dX in the previous layer's output layout: dense rows of its cout,
        // except after an FC layer, whose dcol rows have pitch kp (the first
        // FC's columns past 4096, the scalars, are not propagated)
        if (l.kind == CONV2D) {
            SK(sg::col2im2d(net->s_dcol, l.kp, B, l.h, l.w, l.cin, dx, st));
            ldy = net->L[i - 1].cout;
        } else if (l.kind == CONV1D) {
            SK(sg::col2im1d(net->s_dcol, l.kp, B, l.t, l.cin, l.up, dx, st));
            ldy = net->L[i - 1].cout;
        } else {
            ldy = l.kp;
        }
        dy = dx;
    }
    return 0;
}

int check_err(poe_sg *net)
{
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, net->err, sizeof(int), cudaMemcpyDeviceToHost, net->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(net->stream);
    if (e != cudaSuccess) return fail(net, 5, std::string("sync: ") + cudaGetErrorString(e));
    if (h) {
        cudaMemsetAsync(net->err, 0, sizeof(int), net->stream);
        return fail(net, 4, "a GEMM's bounded wait gave up");
    }
    return 0;
}

}  // namespace

extern "C" {

int poe_sg_create(int32_t max_batch, uint64_t seed, void *stream, poe_sg **out)
{
    if (!out || max_batch < 1) return 1;
    *out = nullptr;
    poe_sg *net = new poe_sg;
    net->bmax = max_batch;
    if (stream) {
        net->stream = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&net->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete net;
            return 5;
        }
        net->own_stream = true;
    }
    build_layers(net);
    const int B = max_batch;
    int rc = 0;
    int64_t max_mk = 0, max_act = 0, max_ck = 0, max_wt = 0;
    for (Layer &l : net->L) {
        const int64_t M = (int64_t)B * l.rows_per_item;
        if (!rc && l.kind != FC) rc = alloc(net, &l.col, M * l.kp);
        if (!rc && &l != &net->L.back()) rc = alloc(net, &l.out, M * l.cout);
        max_mk = std::max(max_mk, M * std::max(l.kp, l.cout));
        max_act = std::max(max_act, M * std::max(l.cout, l.kp));
        max_ck = std::max(max_ck, (int64_t)l.cout * l.kp);
        max_wt = std::max(max_wt, (int64_t)l.cout * l.kp);
    }
    const int64_t nout = (int64_t)B * POE_SG_SAMPLES * POE_SG_CHANNELS;
    if (!rc) rc = alloc(net, &net->w32, net->nparam);
    if (!rc) rc = alloc(net, &net->g32, net->nparam);
    if (!rc) rc = alloc(net, &net->m32, net->nparam);
    if (!rc) rc = alloc(net, &net->v32, net->nparam);
    if (!rc) rc = alloc(net, &net->w16, net->nparam);
    if (!rc) rc = alloc(net, &net->out, nout);
    if (!rc) rc = alloc(net, &net->dout, nout);
    if (!rc) rc = alloc(net, &net->cat, (int64_t)B * kCat);
    if (!rc) rc = alloc(net, &net->s_dz, max_act);
    if (!rc) rc = alloc(net, &net->s_dzt, max_act);
    if (!rc) rc = alloc(net, &net->s_colt, max_mk);
    if (!rc) rc = alloc(net, &net->s_dcol, max_mk);
    if (!rc) rc = alloc(net, &net->s_wt, max_wt);
    if (!rc) rc = alloc(net, &net->s_dx[0], max_act);
    if (!rc) rc = alloc(net, &net->s_dx[1], max_act);
    net->ws_floats = (int64_t)sg::kMaxSplits * max_ck;
    if (!rc) rc = alloc(net, &net->ws, net->ws_floats);
    if (!rc) rc = alloc(net, &net->partial, sg::kMseBlocks);
    if (!rc) rc = alloc(net, &net->loss_dev, 1);
    if (!rc) rc = alloc(net, &net->colpart, ((int64_t)B * POE_SG_SAMPLES / sg::kColChunkRows + 1) * 4160);
    if (!rc) rc = alloc(net, &net->err, 1);
    if (rc) {
        poe_sg_destroy(net);
        return rc;
    }
    // He-normal weights over the real reduction length, zero biases and padding
    std::vector<float> h((size_t)net->nparam, 0.0f);
    Rng r{seed ^ 0x5eed5eed5eedull};
    for (const Layer &l : net->L) {
        const double sd = std::sqrt(2.0 / l.k) * (l.relu ? 1.0 : 0.5);
        for (int o = 0; o < l.cout; ++o)
            for (int c = 0; c < l.k; ++c) h[(size_t)(l.w_off + (int64_t)o * l.kp + c)] = (float)(sd * r.normal());
    }
    rc = poe_sg_set_params(net, nullptr, 0);   // zero state
    cudaError_t e = cudaMemcpy(net->w32, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(net->err, 0, sizeof(int));
    if (e != cudaSuccess || sg::to_bf16(net->w32, net->nparam, net->w16, net->stream) != 0 ||
        cudaStreamSynchronize(net->stream) != cudaSuccess) {
        poe_sg_destroy(net);
        return 5;
    }
    *out = net;
    return 0;
}

int poe_sg_param_count(const poe_sg *net, int64_t *count)
{
    if (!net || !count) return 1;
    *count = real_count(net);
    return 0;
}

// host <-> device in the compact layout (per layer: W [cout][k], then b [cout])
static int params_io(poe_sg *net, float *host, const float *in, int64_t n, float *dev, bool to_dev)
{
    if (n != real_count(net)) return fail(net, 1, "parameter array length");
    std::vector<float> full((size_t)net->nparam, 0.0f);
    if (!to_dev && cudaMemcpy(full.data(), dev, sizeof(float) * full.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail(net, 5, "parameter copy");
    int64_t q = 0;
    for (const Layer &l : net->L) {
        for (int o = 0; o < l.cout; ++o)
            for (int c = 0; c < l.k; ++c, ++q) {
                float &f = full[(size_t)(l.w_off + (int64_t)o * l.kp + c)];
                if (to_dev) f = in[q];
                else host[q] = f;
            }
        for (int o = 0; o < l.cout; ++o, ++q) {
            float &f = full[(size_t)(l.b_off + o)];
            if (to_dev) f = in[q];
            else host[q] = f;
        }
    }
    if (to_dev && cudaMemcpy(dev, full.data(), sizeof(float) * full.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(net, 5, "parameter copy");
    return 0;
}

int poe_sg_get_state(poe_sg *net, float *m, float *v, float *w16_f32, int64_t n, int32_t *step)
{
    if (!net) return 1;
    cudaStreamSynchronize(net->stream);
    int rc = 0;
    if (m && (rc = params_io(net, m, nullptr, n, net->m32, false))) return rc;
    if (v && (rc = params_io(net, v, nullptr, n, net->v32, false))) return rc;
    if (w16_f32) {
        if (n != real_count(net)) return fail(net, 1, "parameter array length");
        // the bf16 copy widened to FP32 (exact), then the compact layout
        std::vector<uint16_t> h16((size_t)net->nparam);
        if (cudaMemcpy(h16.data(), net->w16, sizeof(uint16_t) * h16.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
            return fail(net, 5, "parameter copy");
        std::vector<float> wide(h16.size());
        for (size_t i = 0; i < h16.size(); ++i) {
            const uint32_t bits = (uint32_t)h16[i] << 16;
            std::memcpy(&wide[i], &bits, 4);
        }
        float *tmp = nullptr;
        if (cudaMalloc(&tmp, sizeof(float) * wide.size()) != cudaSuccess) return fail(net, 6, "state copy");
        rc = cudaMemcpy(tmp, wide.data(), sizeof(float) * wide.size(), cudaMemcpyHostToDevice) == cudaSuccess
                 ? params_io(net, w16_f32, nullptr, n, tmp, false)
                 : fail(net, 5, "state copy");
        cudaFree(tmp);
        if (rc) return rc;
    }
    if (step) *step = net->adam_t;
    return 0;
}

int poe_sg_get_params(poe_sg *net, float *host, int64_t n)
{
    if (!net || !host) return 1;
    cudaStreamSynchronize(net->stream);
    return params_io(net, host, nullptr, n, net->w32, false);
}

int poe_sg_get_grads(poe_sg *net, float *host, int64_t n)
{
    if (!net || !host) return 1;
    cudaStreamSynchronize(net->stream);
    return params_io(net, host, nullptr, n, net->g32, false);
}

int poe_sg_set_params(poe_sg *net, const float *host, int64_t n)
{
    if (!net) return 1;
    cudaStreamSynchronize(net->stream);
    if (host) {
        const int rc = params_io(net, nullptr, host, n, net->w32, true);
        if (rc) return rc;
        if (sg::to_bf16(net->w32, net->nparam, net->w16, net->stream) != 0) return fail(net, 5, "to_bf16");
    }
    if (cudaMemsetAsync(net->m32, 0, sizeof(float) * net->nparam, net->stream) != cudaSuccess ||
        cudaMemsetAsync(net->v32, 0, sizeof(float) * net->nparam, net->stream) != cudaSuccess ||
        cudaMemsetAsync(net->g32, 0, sizeof(float) * net->nparam, net->stream) != cudaSuccess)
        return fail(net, 5, "memset");
    net->adam_t = 0;
    return cudaStreamSynchronize(net->stream) == cudaSuccess ? 0 : fail(net, 5, "sync");
}

int poe_sg_forward(poe_sg *net, const void *maps, const float *scalars, int32_t B, float *out)
{
    if (!net || !maps || !scalars || B < 1 || B > net->bmax) return net ? fail(net, 1, "batch") : 1;
    if (((uintptr_t)out & 15) != 0)   // the output layer writes it with TMA stores
        return fail(net, 1, "out must be 16-byte aligned");
    int rc = forward(net, static_cast<const __nv_bfloat16 *>(maps), scalars, B, out ? out : net->out);
    if (rc) return rc;
    return check_err(net);
}

int poe_sg_loss_grad(poe_sg *net, const void *maps, const float *scalars, const void *targets, int32_t B,
                     float *loss_out)
{
    if (!net || !maps || !scalars || !targets || B < 8 || B > net->bmax || B % 8)
        return net ? fail(net, 1, "training batch: a multiple of 8 up to max_batch") : 1;
    int rc = forward(net, static_cast<const __nv_bfloat16 *>(maps), scalars, B, net->out);
    if (rc) return rc;
    const int64_t n = (int64_t)B * POE_SG_SAMPLES * POE_SG_CHANNELS;
    SK(sg::mse(net->out, static_cast<const __nv_bfloat16 *>(targets), n, 2.0f / (float)n, net->dout, net->partial,
               net->loss_dev, net->stream));
    if ((rc = backward(net, B))) return rc;
    float s = 0.0f;
    if (cudaMemcpyAsync(&s, net->loss_dev, sizeof(float), cudaMemcpyDeviceToHost, net->stream) != cudaSuccess)
        return fail(net, 5, "loss copy");
    if ((rc = check_err(net))) return rc;
    if (loss_out) *loss_out = s / (float)n;
    return 0;
}

int poe_sg_adam(poe_sg *net, float lr)
{
    if (!net) return 1;
    const float b1 = 0.9f, b2 = 0.999f;
    net->adam_t += 1;
    const double c1 = 1.0 - std::pow((double)b1, net->adam_t), c2 = 1.0 - std::pow((double)b2, net->adam_t);
    // w -= lr * (m / c1) / (sqrt(v / c2) + eps)  ==  w -= lr_t m / (sqrt(v) + eps sqrt(c2))
    const float lr_t = (float)(lr * std::sqrt(c2) / c1);
    const float eps_t = (float)(1e-8 * std::sqrt(c2));
    SK(sg::adam(net->w32, net->g32, net->m32, net->v32, net->nparam, lr_t, b1, b2, eps_t, net->w16, net->stream));
    return 0;
}

int poe_sg_train_step(poe_sg *net, const void *maps, const float *scalars, const void *targets, int32_t B, float lr,
                      float *loss_out)
{
    int rc = poe_sg_loss_grad(net, maps, scalars, targets, B, loss_out);
    return rc ? rc : poe_sg_adam(net, lr);
}

int poe_sg_launches(const poe_sg *net, int64_t *count)
{
    if (!net || !count) return 1;
    *count = net->launches;
    return 0;
}

const char *poe_sg_last_error(const poe_sg *net) { return net ? net->errmsg.c_str() : "null network"; }

void poe_sg_destroy(poe_sg *net)
{
    if (!net) return;
    if (net->stream) cudaStreamSynchronize(net->stream);
    for (void *p : net->allocs) cudaFree(p);
    if (net->own_stream) cudaStreamDestroy(net->stream);
    delete net;
}

}  // extern "C"
