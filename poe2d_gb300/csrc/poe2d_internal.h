// poe2d_internal.h -- device data layout shared by the kernels and the host
// library (not part of the C ABI).
//
// HBM layout of one model (one grid, shared by all its shots):
//   * every full-grid plane has pitch P floats (a multiple of 32, i.e. 128 B
//     rows) and R = nz + 2*ZH rows; cell (x, z) sits at (z+ZH)*P + (x+XH).
//     The XH columns left of x = 0, the columns right of x = NX and the ZH
//     rows above/below the grid are zero forever, so every 4-point stencil
//     read stays inside the allocation with no bounds test.  The reference's
//     one out-of-row read (stress1 at x = NX-1 reads x+2, which with pitch
//     NX+1 wraps to column 0 of the next row, cu:56) reads a zero here as it
//     does there: column 0 is never written by any kernel.
//   * coefficients: 8 planes (rho, rhof, m, eta/kappa, lambda_c, mu, alpha, M).
//   * profiles: 6 x-profiles of length P (index x+XH) and 6 z-profiles of
//     length R (index z+ZH).
// Per shot:
//   * 12 state planes (vx vz wx wz sxx szz sxz p g11 g22 xi1 xi2);
//   * C-PML memory only on the absorbing strips: the 6 x-direction variables
//     on columns x < xL or x >= xR (nz x Wx each), the 6 z-direction ones on
//     rows z < zT or z >= zB (Hz x P each).  Outside the strips the
//     reference's a = 0 and b = 1, so its memory variables stay exactly zero
//     (cu:1090-1095, 1152-1158): they are not stored.
#pragma once
#include <stdint.h>

#include "poe2d_math.cuh"

namespace poe {

constexpr int XH = 4;  // halo columns left of x = 0
constexpr int ZH = 4;  // halo rows above z = 0 and below z = NZ

enum { NSTATE = 12 };
enum { F_VX = 0, F_VZ, F_WX, F_WZ, F_SXX, F_SZZ, F_SXZ, F_P, F_G11, F_G22, F_XI1, F_XI2 };
enum { C_RHO = 0, C_RHOF, C_RSM, C_EOK, C_LC, C_MU, C_AL, C_M };
enum { PA = 0, PB, PK, PAH, PBH, PKH };
// memory variables: x-direction (stored on x strips) and z-direction
enum { MX_SXX = 0, MX_S2, MX_SXZ, MX_VX1, MX_VX2, MX_VZ };   // b/a: xh xh x x x xh
enum { MZ_SXX = 0, MZ_S2, MZ_SXZ, MZ_VX, MZ_VZ1, MZ_VZ2 };   // b/a: z z zh z zh zh
enum { SRC_NONE = -1, SRC_P = 0, SRC_FZ = 1 };

struct ModelDev {
    int NX, NZ;        // last indices
    int P, R;          // plane pitch (floats) and rows
    int64_t plane;     // P * R
    float dt;
    Div24 qx, qz;      // 1/(24 dx), 1/(24 dz)
    const float *coef; // 8 planes
    const float *px;   // 6 * P
    const float *pz;   // 6 * R
    int xL, xR, Wx;    // x strips: x < xL or x >= xR; Wx = xL + (NX+1 - xR)
    int zT, zB, Hz;    // z strips: z < zT or z >= zB; Hz = zT + (NZ+1 - zB)
};

struct ShotDev {
    float *f;              // NSTATE planes
    float *mx;             // 6 * (NZ+1) * Wx
    float *mz;             // 6 * Hz * P
    const int64_t *step;   // steps done (device counter)
    int64_t src_off;       // plane offset of the source cell, or -1
    int src_where;         // SRC_P / SRC_FZ / SRC_NONE
    int64_t src_n;         // active steps
    const float *src_tab;
    const int2 *rec;       // (plane offset, comp) ; comp < 0: inert
    int nrec;
    float *trace;          // [cap][nrec]
    int64_t trace_cap;
};

// x-strip column of x, or -1
__host__ __device__ __forceinline__ int xcol(const ModelDev &m, int x)
{
    return x < m.xL ? x : (x >= m.xR ? m.xL + (x - m.xR) : -1);
}
// z-strip row of z, or -1
__host__ __device__ __forceinline__ int zrow(const ModelDev &m, int z)
{
    return z < m.zT ? z : (z >= m.zB ? m.zT + (z - m.zB) : -1);
}

// kernel launchers (poe2d_kernels.cu); return cudaError_t as int
// one time step of every shot: stress, record, velocity (k: offset added to
// each shot's step counter)
int launch_step(const ModelDev &m, const ShotDev *shots_dev, int nshots, int max_rec, int k,
                bool exact, bool kone, void *stream);
// steps[i] += by for every shot
int launch_advance(int64_t *steps_dev, int nshots, int64_t by, void *stream);
// f[0..n) = 0
int launch_zero(float *f, int64_t n, void *stream);

}  // namespace poe
