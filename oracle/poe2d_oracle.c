/*
 * poe2d_oracle.c -- CPU oracle for the 2-D poroelastic C-PML time loop.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA product path, never the
 * thing measured or shipped.  Restates, in plain C:
 *   - the C-PML profile builder          cu:985-1159
 *   - the medium-ID table lookup         cu:646-661
 *   - the Biot coefficient derivation    cu:682-713
 *   - the source wavelet and its clock   cu:90-111
 *   - the six-launch time step           cu:1628-1634 (kernels cu:49-386)
 * where cu = seismic_CPML_2D_poroelastic_withCUDA.cu of thejatmik/poe2d.
 *
 * Must be compiled with -ffp-contract=off: the reference arithmetic is
 * specified as separate IEEE operations (C semantics), and GCC contracts
 * a*b+c into FMA by default on aarch64.
 */
#include "poe2d_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)

/* PI as the reference defines it: a float literal (cu:41) */
#define ORC_PI_F 3.1415926535897932f

struct orc_state {
    int mode, NX, NZ;
    float dx, dz, dt;
    int64_t ncell;
    void *f[ORC_NFIELDS];
    void *coef, *px, *pz;
    int src_ix, src_iz, src_where;
    float *src_table;
    int64_t src_n;
    int nrec;
    int32_t *rec;
    int64_t step;
    int nthreads;
};

/* ------------------------------------------------------------------------ */
/* C-PML profiles (cu:985-1159).  Types follow the reference: float variables,
 * double literals promote the expressions they appear in, and the <cmath>
 * float overloads (powf, expf, logf, fabsf) are what C++ picks for float
 * arguments.  Low side: left origin at thickness + 3 dx (cu:1042), top
 * origin at thickness with alpha raised by extra * alpha_max (cu:1102, 1116,
 * 1126).  High side: (N-2) delta - thickness (cu:1043, 1101). */
static void pml_one(float absc, float thickness, float d0, float k_max, float npower,
                    float alpha_max, double extra, float *d, float *K, float *alpha)
{
    float nrm = absc / thickness;
    *d = d0 * powf(nrm, npower);
    *K = (float)(1.0 + ((double)k_max - 1.0) * (double)powf(nrm, npower));
    if (extra != 0.0)
        *alpha = (float)((double)alpha_max * (1.0 - (double)nrm) + extra * (double)alpha_max);
    else
        *alpha = (float)((double)alpha_max * (1.0 - (double)nrm));
}

static void pml_axis(int n1, float delta, float dt, float thickness, float d0, float k_max,
                     float npower, float alpha_max, float origin_lo, float origin_hi,
                     double extra_lo, float *out /* 6*n1 */)
{
    float *a = out + ORC_PA * n1, *b = out + ORC_PB * n1, *K = out + ORC_PK * n1;
    float *ah = out + ORC_PAH * n1, *bh = out + ORC_PBH * n1, *Kh = out + ORC_PKH * n1;
    for (int i = 0; i < n1; ++i) {
        float d = 0.0f, dh = 0.0f, al = 0.0f, alh = 0.0f;   /* cu:1013-1038 */
        K[i] = 1.0f; Kh[i] = 1.0f; a[i] = 0.0f; ah[i] = 0.0f; b[i] = 0.0f; bh[i] = 0.0f;
        float val = delta * (float)i;
        float absc;
        absc = origin_lo - val;
        if (absc >= 0.0f) pml_one(absc, thickness, d0, k_max, npower, alpha_max, extra_lo, &d, &K[i], &al);
        absc = (float)((double)origin_lo - ((double)val + (double)delta / 2.0));
        if (absc >= 0.0f) pml_one(absc, thickness, d0, k_max, npower, alpha_max, extra_lo, &dh, &Kh[i], &alh);
        absc = val - origin_hi;
        if (absc >= 0.0f) pml_one(absc, thickness, d0, k_max, npower, alpha_max, 0.0, &d, &K[i], &al);
        absc = (float)(((double)val + (double)delta / 2.0) - (double)origin_hi);
        if (absc >= 0.0f) pml_one(absc, thickness, d0, k_max, npower, alpha_max, 0.0, &dh, &Kh[i], &alh);
        if (al < 0.0f) al = 0.0f;
        if (alh < 0.0f) alh = 0.0f;
        b[i] = expf(-(d / K[i] + al) * dt);
        bh[i] = expf(-(dh / Kh[i] + alh) * dt);
        if (fabsf(d) > 1.e-6)
            a[i] = (float)((double)d * ((double)b[i] - 1.0) / (double)(K[i] * (d + K[i] * al)));
        if (fabsf(dh) > 1.e-6)
            ah[i] = (float)((double)dh * ((double)bh[i] - 1.0) / (double)(Kh[i] * (dh + Kh[i] * alh)));
    }
}

void orc_pml_profiles(int NX, int NZ, float dx, float dz, float dt, int npoints,
                      float rcoef, float npower, float k_max, float alpha_max,
                      double alpha_top_extra, float cp_max, float *prof_x, float *prof_z)
{
    float thx = (float)npoints * dx;                        /* cu:988-989 */
    float thz = (float)npoints * dz;
    float d0x = (float)(-((double)npower + 1.0) * (double)cp_max * (double)logf(rcoef) / (2.0 * (double)thx));
    float d0z = (float)(-((double)npower + 1.0) * (double)cp_max * (double)logf(rcoef) / (2.0 * (double)thz));
    float xl = thx + (float)3 * dx;                          /* cu:1042 */
    float xr = (float)(NX - 2) * dx - thx;                   /* cu:1043 */
    float zb = (float)(NZ - 2) * dz - thz;                   /* cu:1101 */
    float zt = thz;                                          /* cu:1102 */
    pml_axis(NX + 1, dx, dt, thx, d0x, k_max, npower, alpha_max, xl, xr, 0.0, prof_x);
    pml_axis(NZ + 1, dz, dt, thz, d0z, k_max, npower, alpha_max, zt, zb, alpha_top_extra, prof_z);
}

/* ------------------------------------------------------------------------ */
/* Medium-ID lookup (cu:646-661) + Biot coefficients (cu:682-713).
 * fluid_table rows: kf, eta, kappa, phi, a (tortuosity), rhof.
 * Returns the number of cells whose ID matched no table row (the reference
 * leaves those cells' fluid arrays uninitialised). */
int orc_coeffs_from_medium(int64_t ncell, const float *medium, const float *cp,
                           const float *cs, const float *rho_sat,
                           const float *fluid_table, int ntab, float *coef)
{
    int bad = 0;
    float *rho = coef + ORC_C_RHO * ncell, *rhof = coef + ORC_C_RHOF * ncell;
    float *rsm = coef + ORC_C_RSM * ncell, *eok = coef + ORC_C_EOK * ncell;
    float *lc = coef + ORC_C_LAMBDAC * ncell, *mu = coef + ORC_C_MU * ncell;
    float *alpha = coef + ORC_C_ALPHA * ncell, *M = coef + ORC_C_RBM * ncell;
    for (int64_t j = 0; j < ncell; ++j) {
        int hit = -1;
        for (int i = 0; i < ntab; ++i)
            if (medium[j] == (float)i) hit = i;
        if (hit < 0) {
            ++bad;
            for (int c = 0; c < ORC_NCOEF; ++c) coef[c * ncell + j] = 0.0f;
            continue;
        }
        const float *row = fluid_table + 6 * hit;
        float Kf = row[0], eta = row[1], kappa = row[2], phi = row[3], a = row[4], crhof = row[5];
        float crho = rho_sat[j];
        float crmu = cs[j] * cs[j] * crho;
        float Ksat = (float)((double)rho_sat[j] * ((double)(cp[j] * cp[j]) - (4.0 / 3.0) * (double)(cs[j] * cs[j])));
        float vgede = (float)((3.0 * (double)Ksat - 2.0 * (double)crmu) / (2.0 * (3.0 * (double)Ksat + (double)crmu)));
        float Kb = (float)(((2.0 * (double)vgede / (1.0 - 2.0 * (double)vgede)) + (2.0 / 3.0)) * (double)crmu);
        float Ks = (float)((double)Kb / (1.0 - (double)phi));
        float crsm = a * crhof / phi;
        float ceok = eta / kappa;
        float calpha = (float)(1.0 - (double)(Kb / Ks));
        float crbM = (float)(1.0 / (double)(phi / Kf + (calpha - phi) / Ks));
        if ((eta == 0.0f) || (kappa == 0.0f)) ceok = 0.0f;
        float crlambdao = (float)((double)Kb - (2.0 / 3.0) * (double)crmu);
        float crlambdac = crlambdao + calpha * calpha * crbM;
        rho[j] = crho; rhof[j] = crhof; rsm[j] = crsm; eok[j] = ceok;
        lc[j] = crlambdac; mu[j] = crmu; alpha[j] = calpha; M[j] = crbM;
    }
    return bad;
}

/* ------------------------------------------------------------------------ */
/* Source tables.  Step n (1-based) uses t = i_gpu * dt with i_gpu = n - 1,
 * both float (cu:94, 110); the table stops at the first step with
 * t >= t_cut (cu:107).  kind 0: the reference's first derivative of a
 * Gaussian, factor 1e10, a = pi^2 f0^2, t0 = 1/f0 (cu:93-97), evaluated as
 * the host compiler evaluates that line (double pow/exp).  kind 1: Ricker
 * wavelet, t0 = 1.2/f0, as a vertical body force amplitude/(dx dz)
 * (no reference counterpart; the commented variants at cu:252, 363 use the
 * same 1.2/f0 delay).  t_cut <= 0 means no cut-off.  Returns the number of
 * active steps (the table length). */
int64_t orc_source_table(int kind, float f0, float amplitude, double t_cut, float dt,
                         float dx, float dz, int64_t nsteps, float *table)
{
    const float a = ORC_PI_F * ORC_PI_F * f0 * f0;
    int64_t n;
    for (n = 0; n < nsteps; ++n) {
        float t = (float)n * dt;
        if (t_cut > 0.0 && !((double)t < t_cut)) break;
        if (kind == 0) {
            float t0 = (float)(1.0 / (double)f0);
            float tt = t - t0;
            table[n] = (float)(1.0e10 * 2.0 * (double)a * (double)tt *
                               exp((double)(-a) * pow((double)tt, 2.0)));
        } else {
            float t0 = (float)(1.2 / (double)f0);
            float tt = t - t0;
            double e = exp((double)(-a) * pow((double)tt, 2.0));
            double r = (1.0 - 2.0 * (double)a * pow((double)tt, 2.0)) * e;
            table[n] = (float)((double)amplitude * r / ((double)dx * (double)dz));
        }
    }
    return n;
}

/* ------------------------------------------------------------------------ */
/* time-step instantiations */

/* REFMIXED: FP32 storage; the reference's double literals make these
 * sub-expressions FP64 (cu:64-65, 226, 241-242, 294-295, 309). */
#define SFX refmixed
#define REAL float
#define D4(a, b, c, d, h) \
    ((float)(((27.0 * (double)(a) - 27.0 * (double)(b)) - (double)(c) + (double)(d)) / (double)(h) / 24.0))
#define SXZ(s, c, S, dt) ((float)((double)(s) + (double)(c) / 1.0 * (double)(S) * (double)(dt)))
#define SXX(l, m, g1, g2, al, p) \
    ((float)(((double)(l) + 2.0 * (double)(m)) * (double)(g1) + (double)((l) * (g2)) - (double)((al) * (p))))
#define SZZ(l, m, g1, g2, al, p) \
    ((float)((double)((l) * (g1)) + ((double)(l) + 2.0 * (double)(m)) * (double)(g2) - (double)((al) * (p))))
#define HADD(co, x) ((float)((double)(co) + (double)(x) * 0.50))
#define HSUB(co, x) ((float)((double)(co) - (double)(x) * 0.50))
#define HALF(x) ((float)((double)(x) * 0.50))
#include "oracle_step.inc"
#undef SFX
#undef REAL
#undef D4
#undef SXZ
#undef SXX
#undef SZZ
#undef HADD
#undef HSUB
#undef HALF

/* F32 / F64: the same statements with every literal in the storage type. */
#define SFX f32
#define REAL float
#define D4(a, b, c, d, h) ((27.0f * (a) - 27.0f * (b) - (c) + (d)) / (h) / 24.0f)
#define SXZ(s, c, S, dt) ((s) + (c) * (S) * (dt))
#define SXX(l, m, g1, g2, al, p) (((l) + 2.0f * (m)) * (g1) + (l) * (g2) - (al) * (p))
#define SZZ(l, m, g1, g2, al, p) ((l) * (g1) + ((l) + 2.0f * (m)) * (g2) - (al) * (p))
#define HADD(co, x) ((co) + (x) * 0.5f)
#define HSUB(co, x) ((co) - (x) * 0.5f)
#define HALF(x) ((x) * 0.5f)
#include "oracle_step.inc"
#undef SFX
#undef REAL
#undef D4
#undef SXZ
#undef SXX
#undef SZZ
#undef HADD
#undef HSUB
#undef HALF

#define SFX f64
#define REAL double
#define D4(a, b, c, d, h) ((27.0 * (a) - 27.0 * (b) - (c) + (d)) / (double)(h) / 24.0)
#define SXZ(s, c, S, dt) ((s) + (c) * (S) * (dt))
#define SXX(l, m, g1, g2, al, p) (((l) + 2.0 * (m)) * (g1) + (l) * (g2) - (al) * (p))
#define SZZ(l, m, g1, g2, al, p) ((l) * (g1) + ((l) + 2.0 * (m)) * (g2) - (al) * (p))
#define HADD(co, x) ((co) + (x) * 0.5)
#define HSUB(co, x) ((co) - (x) * 0.5)
#define HALF(x) ((x) * 0.5)
#include "oracle_step.inc"

/* ------------------------------------------------------------------------ */
static size_t real_size(int mode) { return mode == ORC_F64 ? sizeof(double) : sizeof(float); }

static void *copy_promote(int mode, const float *src, int64_t n)
{
    if (mode == ORC_F64) {
        double *d = (double *)malloc(sizeof(double) * (size_t)n);
        for (int64_t i = 0; i < n; ++i) d[i] = (double)src[i];
        return d;
    }
    float *f = (float *)malloc(sizeof(float) * (size_t)n);
    memcpy(f, src, sizeof(float) * (size_t)n);
    return f;
}

orc_state *orc_new(int mode, int NX, int NZ, float dx, float dz, float dt,
                   const float *coef, const float *prof_x, const float *prof_z)
{
    orc_state *s = (orc_state *)calloc(1, sizeof(orc_state));
    s->mode = mode; s->NX = NX; s->NZ = NZ; s->dx = dx; s->dz = dz; s->dt = dt;
    s->ncell = (int64_t)(NX + 1) * (NZ + 1);
    for (int f = 0; f < ORC_NFIELDS; ++f) s->f[f] = calloc((size_t)s->ncell, real_size(mode));
    s->coef = copy_promote(mode, coef, ORC_NCOEF * s->ncell);
    s->px = copy_promote(mode, prof_x, ORC_NPROF * (int64_t)(NX + 1));
    s->pz = copy_promote(mode, prof_z, ORC_NPROF * (int64_t)(NZ + 1));
    s->src_ix = -1;
    s->nthreads = 1;
    return s;
}

void orc_free(orc_state *s)
{
    if (!s) return;
    for (int f = 0; f < ORC_NFIELDS; ++f) free(s->f[f]);
    free(s->coef); free(s->px); free(s->pz); free(s->src_table); free(s->rec);
    free(s);
}

void orc_set_source(orc_state *s, int ix, int iz, int where, const float *table, int64_t ntable)
{
    free(s->src_table);
    s->src_table = NULL;
    s->src_ix = ix; s->src_iz = iz; s->src_where = where; s->src_n = ntable;
    if (ntable > 0) {
        s->src_table = (float *)malloc(sizeof(float) * (size_t)ntable);
        memcpy(s->src_table, table, sizeof(float) * (size_t)ntable);
    }
}

void orc_set_receivers(orc_state *s, int nrec, const int32_t *rec)
{
    free(s->rec);
    s->rec = NULL;
    s->nrec = nrec;
    if (nrec > 0) {
        s->rec = (int32_t *)malloc(sizeof(int32_t) * 3 * (size_t)nrec);
        memcpy(s->rec, rec, sizeof(int32_t) * 3 * (size_t)nrec);
    }
}

void orc_set_threads(orc_state *s, int nthreads) { s->nthreads = nthreads > 0 ? nthreads : 1; }

int64_t orc_run(orc_state *s, int64_t nsteps, float *traces)
{
    for (int64_t k = 0; k < nsteps; ++k) {
        float *row = traces ? traces + k * s->nrec : NULL;
        if (s->mode == ORC_REFMIXED) orc_step_refmixed(s, row);
        else if (s->mode == ORC_F32) orc_step_f32(s, row);
        else orc_step_f64(s, row);
    }
    return s->step;
}

void orc_get_field(const orc_state *s, int field, float *out)
{
    if (s->mode == ORC_F64) {
        const double *d = (const double *)s->f[field];
        for (int64_t i = 0; i < s->ncell; ++i) out[i] = (float)d[i];
    } else {
        memcpy(out, s->f[field], sizeof(float) * (size_t)s->ncell);
    }
}

void orc_get_field64(const orc_state *s, int field, double *out)
{
    if (s->mode == ORC_F64) {
        memcpy(out, s->f[field], sizeof(double) * (size_t)s->ncell);
    } else {
        const float *f = (const float *)s->f[field];
        for (int64_t i = 0; i < s->ncell; ++i) out[i] = (double)f[i];
    }
}

void orc_set_field(orc_state *s, int field, const float *in)
{
    if (s->mode == ORC_F64) {
        double *d = (double *)s->f[field];
        for (int64_t i = 0; i < s->ncell; ++i) d[i] = (double)in[i];
    } else {
        memcpy(s->f[field], in, sizeof(float) * (size_t)s->ncell);
    }
}

int64_t orc_steps_done(const orc_state *s) { return s->step; }
