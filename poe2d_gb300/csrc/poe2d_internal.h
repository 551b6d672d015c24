// poe2d_internal.h -- device data layout shared by the kernels and the host
// library (not part of the C ABI).
//
// HBM layout of one model (one grid, shared by all its shots):
//   * every full-grid plane has pitch P floats (a multiple of 32, i.e. 128 B
//     rows) and R rows; cell (x, z) sits at (z+ZH)*P + (x+XH).  P and R
//     cover every tile of the grid plus its 4-cell halo (P >= 64 ntx + 8,
//     R = 32 ntz + 8), and everything outside the grid is zero forever, so
//     tile loads and 4-point stencils need no bounds test.  The reference's
//     one out-of-row read (stress1 at x = NX-1 reads x+2, which with pitch
//     NX+1 wraps to column 0 of the next row, cu:56) reads a zero here as it
//     does there: column 0 is never written by any kernel.
//   * coefficients: 8 planes (rho, rhof, m, eta/kappa, lambda_c, mu, alpha, M).
//   * profiles: 6 x-profiles of length P (index x+XH) and 6 z-profiles of
//     length R (index z+ZH).
// Per shot:
//   * 9 integrated state planes (vx vz wx wz sxz g11 g22 xi1 xi2), twice
//     (step n reads one set and writes the other); sigma_xx, sigma_zz and
//     sigma2 = p are pointwise functions of these and are not stored;
//   * C-PML memory only on the absorbing strips: x-direction variables on
//     columns x < xL or x >= xR (nz x Wx each), z-direction ones on rows
//     z < zT or z >= zB (Hz x P each).  Outside the strips the reference's
//     a = 0 and b = 1, so its memory variables stay exactly zero
//     (cu:1090-1095, 1152-1158): they are not stored.
#pragma once
#include <stdint.h>

#include "poe2d_math.cuh"
#include "poe2d_palette.h"

namespace poe {

constexpr int XH = 4;  // halo columns left of x = 0
constexpr int ZH = 4;  // halo rows above z = 0 and below z = NZ

enum { C_RHO = 0, C_RHOF, C_RSM, C_EOK, C_LC, C_MU, C_AL, C_M };
enum { PA = 0, PB, PK, PAH, PBH, PKH };
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
    int *err;          // device flag: a bounded wait in a kernel gave up
    // palette mode: one byte per cell selects a row of a small material table
    const uint8_t *ids;      // padded plane of material ids (pitch P bytes, R rows), or null
    const float *mtab;       // nmat rows of MT_W floats
    int nmat;
    int ntx, ntz;            // tiles across x and z of the step kernel (receiver lists, tile flags)
    // TMA descriptors (device memory) of the id plane (palette models only) and
    // of the 6 x-profile and 6 z-profile rows, boxed for the step kernel's tiles
    const void *tm_ids, *tm_px, *tm_pz;
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

// ---- fused tile step (poe2d_tile.cu) ----
// the padded planes also round the grid up to 64 x 32 cells (a layout choice
// kept from an earlier tile shape; the step kernel's tiles are PAL_TX x PAL_TZ)
constexpr int TILE_X = 64;
constexpr int TILE_Z = 32;

// integrated state planes per buffer (sigma_xx, sigma_zz, p are derived)
enum { SF_VX = 0, SF_VZ, SF_WX, SF_WZ, SF_SXZ, SF_G11, SF_G22, SF_XI1, SF_XI2, NSF };
// stress C-PML memory (double-buffered) and velocity C-PML memory (in place)
enum { MXS_SXX = 0, MXS_S2, MXS_SXZ };   // x strips, profiles xh xh x
enum { MZS_SXX = 0, MZS_S2, MZS_SXZ };   // z strips, profiles z z zh
enum { MXV_VX1 = 0, MXV_VX2, MXV_VZ };   // x strips, profiles x x xh
enum { MZV_VX = 0, MZV_VZ1, MZV_VZ2 };   // z strips, profiles z zh zh

struct StreamShot {
    float *f[2];           // NSF planes each; step n reads f[(n-1)&1], writes f[n&1]
    float *mx[2], *mz[2];  // 3 stress memory arrays each (nz x Wx / Hz x P)
    float *mxv, *mzv;      // 3 velocity memory arrays each
    float *acc;            // [2]: sigma2 at a source cell outside stress1's range
    const int64_t *step;   // steps done (device counter)
    int64_t src_off;       // plane offset of the source cell, or -1
    int src_where;         // SRC_P / SRC_FZ / SRC_NONE
    int64_t src_n;         // active steps of the source table
    const float *src_tab;
    const int *rec_start;  // CSR over tiles: ntiles + 1 entries
    const int4 *rec_sorted;// (x, comp, slot, z), grouped by tile
    int nrec;
    float *trace;          // [cap][nrec]
    int64_t trace_cap;
    const void *tm_v;      // TMA descriptors over both state buffers (palette mode)
    const void *tm_s;
    int *done;             // per tile (tz ntx + tx): a step it has completed (step-spanning launches);
                           // never ahead of the shot (zeroed on reset and restore), the first step of a
                           // launch waits for none, later steps only for flags published in the launch
};

// nk steps (k .. k+nk-1 of the graph or run, n = *step + k + 1 ...) of a model's
// shots over the work list items[0..nitems) of (0, shot, x0, z0).  nk = 1:
// one launch per step.  nk > 1: one step-spanning launch, in which a tile of
// step n > its first starts once its 3 x 3 neighbourhood has completed step
// n-1 (the shots' done flags).  queue: 2 device ints, zero before the first
// launch; each launch's CTAs take its items from it and set it back to zero.
// tile_z: the tiles' height (PAL_TZ, or PAL_TZ_SMALL with FAST stencils)
int launch_tile_step(const ModelDev &m, const StreamShot *shots_dev, int nshots, const int4 *items, int nitems, int k,
                     int nk, bool exact, bool kone, int tile_z, int *queue, void *stream);
// one step over several models: items (model, shot, x0, z0) index models_dev and shots_dev;
// exact_few: every model's spacings have a 24 h of few bits; coef: the models read
// their 8 coefficient planes per cell (all of them), else each has a material palette
int launch_batch_step(const ModelDev *models_dev, const StreamShot *shots_dev, const int4 *items, int nitems, int k,
                      int nk, bool exact, bool exact_few, bool coef, bool kone, int *queue, void *stream);
// the step kernel of one stencil mode (poe2d_tile_fast.cu, poe2d_tile_exact.cu,
// poe2d_tile_exact_any.cu): models null for a single model m, else a batch
int tile_step_fast(const ModelDev &m, const ModelDev *models, const StreamShot *shots, const int4 *items, int nitems,
                   int k, int nk, bool kone, bool coef, int *queue, void *stream);
int tile_step_exact(const ModelDev &m, const ModelDev *models, const StreamShot *shots, const int4 *items, int nitems,
                    int k, int nk, bool kone, bool coef, int *queue, void *stream);
int tile_step_exact_any(const ModelDev &m, const ModelDev *models, const StreamShot *shots, const int4 *items,
                        int nitems, int k, int nk, bool kone, bool coef, int *queue, void *stream);
// the FAST single-model variants on 60 x PAL_TZ_SMALL tiles (poe2d_tile_fast16.cu)
int tile_step_fast16(const ModelDev &m, const StreamShot *shots, const int4 *items, int nitems, int k, int nk,
                     bool kone, bool coef, int *queue, void *stream);
// *shots[i].step += by for i < nshots
int launch_advance_shots(const StreamShot *shots_dev, int nshots, int64_t by, void *stream);
// the step kernel's bounded waits against conditions that never hold: an
// mbarrier no thread arrives at (bit 0 of *err when it gives up), a tile flag
// nothing sets (bit 1), and flags that are set (bit 2 if that wait gives up);
// flags: 9 device ints, flags[0] = 0, flags[1..8] = 5
int launch_wait_limit(int *err, const int *flags, int polls, void *stream);
// step kernel tile: 60 x TZ cells worked by 64 x 4 threads per warp pair
// (stress on 64 columns = tile + 2-cell halo each side); TZ = 32 for every
// variant, PAL_TZ_SMALL = 16 for the FAST single-model ones.  TMA boxes of
// 68 x TZ+8 (velocity) and 68 x TZ+4 (stress state) floats
constexpr int PAL_TX = 60, PAL_TZ = 32, PAL_TZ_SMALL = 16;
constexpr int TMA_VW = PAL_TX + 8;
constexpr int tile_vh(int tz) { return tz + 8; }
constexpr int tile_sh(int tz) { return tz + 4; }
// material-id box: rows z0-2 .. z0+TZ+2, 80 bytes from x0+XH-4 rounded down to
// 16 bytes (a TMA box starts on a 16-byte column), covering x0-4 .. x0+63
constexpr int PAL_IDS_W = 80;
constexpr int tile_ids_h(int tz) { return tz + 5; }
int launch_derive(const ModelDev &m, const StreamShot *shots_dev, int shot, int64_t n, float *out, void *stream);
// allocation-free read-out of one derived field (sigma_xx 0, sigma_zz 1, p 2)
// through the library's static scratch plane; returns a cudaError_t
constexpr int64_t NOALLOC_SCRATCH_FLOATS = (int64_t)8 << 20;
int derive_noalloc(const ModelDev &m, const float *F, const float *acc, int64_t src_off, int src_where,
                   int64_t src_n, const float *src_tab, int64_t n, int which, float *host_out, void *stream);
// steps[i] += by for every shot
int launch_advance(int64_t *steps_dev, int nshots, int64_t by, void *stream);

}  // namespace poe
