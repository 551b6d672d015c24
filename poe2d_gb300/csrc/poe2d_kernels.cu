// poe2d_kernels.cu -- sm_103a kernels of the poroelastic C-PML time step.
//
// One time step (reference order cu:1628-1634):
//   k_stress    stress1 + source + stress2 + stress3 fused per cell
//               (cu:49-112, 202-229, 231-244)
//   k_record    receivers, between the stress and velocity updates (cu:114-201)
//   k_velocity  vx_kernel + vz_kernel fused per cell (cu:279-386)
// Shots are the z dimension of every grid, so one launch advances all of a
// model's shots.  The step number comes from each shot's device counter plus
// the launch's offset k, so a captured CUDA graph replays unchanged.
//
// Built with -fmad=false: every a*b+c below is two IEEE operations, as in the
// reference; the only fused multiply-adds are the explicit fmaf() calls in
// poe2d_math.cuh.
#include <cuda_runtime.h>

#include "poe2d_internal.h"

namespace poe {

constexpr int BX = 32, BY = 8;

template <bool EXACT>
__device__ __forceinline__ float D4(float a, float b, float c, float d, const Div24 &q)
{
    return EXACT ? d4_exact(a, b, c, d, q) : d4_fast(a, b, c, d, q);
}

template <bool KONE>
__device__ __forceinline__ float KDIV(float v, float K)
{
    return KONE ? v : v / K;   // K == 1 exactly everywhere when KONE: v / 1 == v
}

// ---------------------------------------------------------------- stress
template <bool EXACT, bool KONE>
__global__ void __launch_bounds__(BX *BY) k_stress(const ModelDev m, const ShotDev *__restrict__ shots, int k)
{
    const int x = blockIdx.x * BX + threadIdx.x;
    const int z = blockIdx.y * BY + threadIdx.y;
    if (x > m.NX || z > m.NZ) return;
    const ShotDev &S = shots[blockIdx.z];
    const int64_t n = *S.step + k + 1;
    const int NX = m.NX, NZ = m.NZ;
    const int64_t P = m.P, PL = m.plane;
    const int64_t o = (int64_t)(z + ZH) * P + (x + XH);
    float *F = S.f;
    const float *vx = F + F_VX * PL, *vz = F + F_VZ * PL, *wx = F + F_WX * PL, *wz = F + F_WZ * PL;
    const float *C = m.coef;
    const float dt = m.dt;

    const bool g1 = x >= 1 && x <= NX - 1 && z >= 2 && z <= NZ - 2;   // stress1 (cu:60-62)
    const bool g2 = x >= 2 && x <= NX - 1 && z >= 1 && z <= NZ - 2;   // stress2 (cu:212-214)
    const bool g3 = x >= 1 && x <= NX - 2 && z >= 2 && z <= NZ - 1;   // stress3 (cu:237-239)
    const int xc = xcol(m, x), zr = zrow(m, z);
    const int64_t nzx = (int64_t)(NZ + 1) * m.Wx, hzp = (int64_t)m.Hz * P;
    const int64_t ix = (int64_t)z * m.Wx + xc, iz = (int64_t)zr * P + (x + XH);

    float g11 = F[F_G11 * PL + o], g22 = F[F_G22 * PL + o];
    float pv = F[F_P * PL + o];
    if (g1) {
        const float *pxh_a = m.px + PAH * P, *pxh_b = m.px + PBH * P, *pxh_k = m.px + PKH * P;
        const float *pz_a = m.pz + PA * m.R, *pz_b = m.pz + PB * m.R, *pz_k = m.pz + PK * m.R;
        const int xi = x + XH, zi = z + ZH;
        float vdx = D4<EXACT>(vx[o + 1], vx[o], vx[o + 2], vx[o - 1], m.qx);
        float vdz = D4<EXACT>(vz[o], vz[o - P], vz[o + P], vz[o - 2 * P], m.qz);
        float wdx = D4<EXACT>(wx[o + 1], wx[o], wx[o + 2], wx[o - 1], m.qx);
        float wdz = D4<EXACT>(wz[o], wz[o - P], wz[o + P], wz[o - 2 * P], m.qz);
        float m1 = 0.0f, m2 = 0.0f, m3 = 0.0f, m4 = 0.0f;
        if (xc >= 0) {
            float *M1 = S.mx + MX_SXX * nzx + ix, *M3 = S.mx + MX_S2 * nzx + ix;
            m1 = pxh_b[xi] * *M1 + pxh_a[xi] * vdx;   *M1 = m1;
            m3 = pxh_b[xi] * *M3 + pxh_a[xi] * wdx;   *M3 = m3;
        }
        if (zr >= 0) {
            float *M2 = S.mz + MZ_SXX * hzp + iz, *M4 = S.mz + MZ_S2 * hzp + iz;
            m2 = pz_b[zi] * *M2 + pz_a[zi] * vdz;     *M2 = m2;
            m4 = pz_b[zi] * *M4 + pz_a[zi] * wdz;     *M4 = m4;
        }
        g11 = g11 + dt * (KDIV<KONE>(vdx, pxh_k[xi]) + m1);
        g22 = g22 + dt * (KDIV<KONE>(vdz, pz_k[zi]) + m2);
        float xi1 = F[F_XI1 * PL + o], xi2 = F[F_XI2 * PL + o];
        xi1 = xi1 - (KDIV<KONE>(wdx, pxh_k[xi]) + m3) * dt;
        xi2 = xi2 - (KDIV<KONE>(wdz, pz_k[zi]) + m4) * dt;
        const float al = C[C_AL * PL + o], M = C[C_M * PL + o];
        pv = -al * M * (g11 + g22) + M * (xi1 + xi2);
        F[F_G11 * PL + o] = g11;
        F[F_G22 * PL + o] = g22;
        F[F_XI1 * PL + o] = xi1;
        F[F_XI2 * PL + o] = xi2;
    }
    const bool src = (o == S.src_off) && S.src_where == SRC_P && n <= S.src_n;
    if (src) pv = pv + S.src_tab[n - 1];                 // cu:107-109
    if (g1 || src) F[F_P * PL + o] = pv;

    if (g2) {
        const int xi = x + XH, zi = z + ZH;
        const float c33 = C[C_MU * PL + o + P];            // rmu[top] (cu:218)
        float vdx = D4<EXACT>(vz[o], vz[o - 1], vz[o + 1], vz[o - 2], m.qx);
        float vdz = D4<EXACT>(vx[o + P], vx[o], vx[o + 2 * P], vx[o - P], m.qz);
        float m1 = 0.0f, m2 = 0.0f;
        if (xc >= 0) {
            float *M1 = S.mx + MX_SXZ * nzx + ix;
            m1 = m.px[PB * P + xi] * *M1 + m.px[PA * P + xi] * vdx;
            *M1 = m1;
        }
        if (zr >= 0) {
            float *M2 = S.mz + MZ_SXZ * hzp + iz;
            m2 = m.pz[PBH * m.R + zi] * *M2 + m.pz[PAH * m.R + zi] * vdz;
            *M2 = m2;
        }
        float Ssum = KDIV<KONE>(vdx, m.px[PK * P + xi]) + m1 + KDIV<KONE>(vdz, m.pz[PK * m.R + zi]) + m2;
        float s = F[F_SXZ * PL + o];
        F[F_SXZ * PL + o] = EXACT ? sxz_exact(s, c33, Ssum, dt) : sxz_fast(s, c33, Ssum, dt);
    }
    if (g3) {
        float sxx, szz;
        const float l = C[C_LC * PL + o], mu = C[C_MU * PL + o], al = C[C_AL * PL + o];
        if (EXACT) sxx_szz_exact(l, mu, g11, g22, al, pv, sxx, szz);
        else sxx_szz_fast(l, mu, g11, g22, al, pv, sxx, szz);
        F[F_SXX * PL + o] = sxx;
        F[F_SZZ * PL + o] = szz;
    }
}

// ---------------------------------------------------------------- receivers
__global__ void k_record(const ModelDev m, const ShotDev *__restrict__ shots, int k)
{
    const ShotDev &S = shots[blockIdx.y];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= S.nrec) return;
    const int64_t n = *S.step + k + 1;
    if (n > S.trace_cap) return;
    const int2 rc = S.rec[r];
    float v = 0.0f;
    if (rc.y >= 0) {
        const int plane = rc.y == 0 ? F_VX : (rc.y == 1 ? F_VZ : F_P);
        v = S.f[plane * m.plane + rc.x];
    }
    S.trace[(n - 1) * S.nrec + r] = v;
}

// ---------------------------------------------------------------- velocity
template <bool EXACT, bool KONE>
__global__ void __launch_bounds__(BX *BY) k_velocity(const ModelDev m, const ShotDev *__restrict__ shots, int k)
{
    const int x = blockIdx.x * BX + threadIdx.x;
    const int z = blockIdx.y * BY + threadIdx.y;
    if (x > m.NX || z > m.NZ) return;
    const ShotDev &S = shots[blockIdx.z];
    const int64_t n = *S.step + k + 1;
    const int NX = m.NX, NZ = m.NZ;
    const int64_t P = m.P, PL = m.plane;
    const int64_t o = (int64_t)(z + ZH) * P + (x + XH);
    float *F = S.f;
    const float *sxx = F + F_SXX * PL, *szz = F + F_SZZ * PL, *sxz = F + F_SXZ * PL, *p = F + F_P * PL;
    const float *C = m.coef;
    const float dt = m.dt;
    const int xc = xcol(m, x), zr = zrow(m, z);
    const int64_t nzx = (int64_t)(NZ + 1) * m.Wx, hzp = (int64_t)m.Hz * P;
    const int64_t ix = (int64_t)z * m.Wx + xc, iz = (int64_t)zr * P + (x + XH);
    const int xi = x + XH, zi = z + ZH;

    // vx, wx (cu:289-312)
    if (x >= 2 && x <= NX - 1 && z >= 2 && z <= NZ - 1) {
        const float rho = C[C_RHO * PL + o], rsm = C[C_RSM * PL + o];
        const float rhof = C[C_RHOF * PL + o], eok = C[C_EOK * PL + o];
        const float co = (rho * rsm - rhof * rhof) / dt;
        const float c1 = co + rho * eok * 0.5f;
        const float c2 = co - rho * eok * 0.5f;
        float d1 = D4<EXACT>(sxx[o], sxx[o - 1], sxx[o + 1], sxx[o - 2], m.qx);
        float d2 = D4<EXACT>(p[o], p[o - 1], p[o + 1], p[o - 2], m.qx);
        float d3 = D4<EXACT>(sxz[o], sxz[o - P], sxz[o + P], sxz[o - 2 * P], m.qz);
        float m1 = 0.0f, m2 = 0.0f, m3 = 0.0f;
        if (xc >= 0) {
            const float b = m.px[PB * P + xi], a = m.px[PA * P + xi];
            float *M1 = S.mx + MX_VX1 * nzx + ix, *M2 = S.mx + MX_VX2 * nzx + ix;
            m1 = b * *M1 + a * d1;  *M1 = m1;
            m2 = b * *M2 + a * d2;  *M2 = m2;
        }
        if (zr >= 0) {
            float *M3 = S.mz + MZ_VX * hzp + iz;
            m3 = m.pz[PB * m.R + zi] * *M3 + m.pz[PA * m.R + zi] * d3;
            *M3 = m3;
        }
        const float Kx = m.px[PK * P + xi], Kz = m.pz[PK * m.R + zi];
        const float A = KDIV<KONE>(d1, Kx) + m1 + KDIV<KONE>(d3, Kz) + m3;
        const float B = KDIV<KONE>(d2, Kx) + m2;
        const float w0 = F[F_WX * PL + o];
        const float w1 = (c2 * w0 + (-rhof * A - rho * B)) / c1;
        const float vt = (w0 + w1) * 0.5f;
        F[F_WX * PL + o] = w1;
        F[F_VX * PL + o] = F[F_VX * PL + o] + (rsm * A + rhof * B + rhof * eok * vt) / co;
    }
    // vz, wz with material at top (cu:326-354)
    if (x >= 1 && x <= NX - 2 && z >= 1 && z <= NZ - 2) {
        const int64_t t = o + P;
        const float rho = C[C_RHO * PL + t], rsm = C[C_RSM * PL + t];
        const float rhof = C[C_RHOF * PL + t], eok = C[C_EOK * PL + t];
        const float co = (rho * rsm - rhof * rhof) / dt;
        const float c1 = co + rho * eok * 0.5f;
        const float c2 = co - rho * eok * 0.5f;
        float d1 = D4<EXACT>(sxz[o + 1], sxz[o], sxz[o + 2], sxz[o - 1], m.qx);
        float d2 = D4<EXACT>(szz[o + P], szz[o], szz[o + 2 * P], szz[o - P], m.qz);
        float d3 = D4<EXACT>(p[o + P], p[o], p[o + 2 * P], p[o - P], m.qz);
        float m1 = 0.0f, m2 = 0.0f, m3 = 0.0f;
        if (xc >= 0) {
            float *M1 = S.mx + MX_VZ * nzx + ix;
            m1 = m.px[PBH * P + xi] * *M1 + m.px[PAH * P + xi] * d1;
            *M1 = m1;
        }
        if (zr >= 0) {
            const float b = m.pz[PBH * m.R + zi], a = m.pz[PAH * m.R + zi];
            float *M2 = S.mz + MZ_VZ1 * hzp + iz, *M3 = S.mz + MZ_VZ2 * hzp + iz;
            m2 = b * *M2 + a * d2;  *M2 = m2;
            m3 = b * *M3 + a * d3;  *M3 = m3;
        }
        const float Kxh = m.px[PKH * P + xi], Kzh = m.pz[PKH * m.R + zi];
        float A = KDIV<KONE>(d1, Kxh) + m1 + KDIV<KONE>(d2, Kzh) + m2;
        const float B = KDIV<KONE>(d3, Kzh) + m3;
        if (o == S.src_off && S.src_where == SRC_FZ && n <= S.src_n) A = A + S.src_tab[n - 1];
        const float w0 = F[F_WZ * PL + o];
        const float w1 = (c2 * w0 + (-rhof * A - rho * B)) / c1;
        const float vt = (w0 + w1) * 0.5f;
        F[F_WZ * PL + o] = w1;
        F[F_VZ * PL + o] = F[F_VZ * PL + o] + (rsm * A + rhof * B + rhof * eok * vt) / co;
    }
}

__global__ void k_advance(int64_t *steps, int nshots, int64_t by)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nshots) steps[i] += by;
}

__global__ void k_zero(float *f, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        f[i] = 0.0f;
}

// ---------------------------------------------------------------- launchers
template <bool EXACT, bool KONE>
static int step_impl(const ModelDev &m, const ShotDev *shots, int nshots, int k, int max_rec, cudaStream_t st)
{
    dim3 blk(BX, BY);
    dim3 grd((m.NX + 1 + BX - 1) / BX, (m.NZ + 1 + BY - 1) / BY, nshots);
    k_stress<EXACT, KONE><<<grd, blk, 0, st>>>(m, shots, k);
    if (max_rec > 0) k_record<<<dim3((max_rec + 127) / 128, nshots), 128, 0, st>>>(m, shots, k);
    k_velocity<EXACT, KONE><<<grd, blk, 0, st>>>(m, shots, k);
    return (int)cudaGetLastError();
}

int launch_step(const ModelDev &m, const ShotDev *shots_dev, int nshots, int max_rec, int k,
                bool exact, bool kone, void *stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    if (exact) return kone ? step_impl<true, true>(m, shots_dev, nshots, k, max_rec, st)
                           : step_impl<true, false>(m, shots_dev, nshots, k, max_rec, st);
    return kone ? step_impl<false, true>(m, shots_dev, nshots, k, max_rec, st)
                : step_impl<false, false>(m, shots_dev, nshots, k, max_rec, st);
}

int launch_advance(int64_t *steps_dev, int nshots, int64_t by, void *stream)
{
    k_advance<<<(nshots + 127) / 128, 128, 0, (cudaStream_t)stream>>>(steps_dev, nshots, by);
    return (int)cudaGetLastError();
}

int launch_zero(float *f, int64_t n, void *stream)
{
    if (n <= 0) return 0;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_zero<<<blocks, 256, 0, (cudaStream_t)stream>>>(f, n);
    return (int)cudaGetLastError();
}

}  // namespace poe
