/*
 * poe2d_oracle.h -- CPU oracle for the 2-D poroelastic C-PML time loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * algorithm (thejatmik/poe2d, seismic_CPML_2D_poroelastic_withCUDA.cu) used
 * as the checker for the CUDA product path.  Only tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline / reference arm may load it.  The product path
 * (poe2d_gb300) never links, imports or calls it.
 *
 * Parity pin: the restatement is compared bit-for-bit against the reference's
 * own kernels and set-up code compiled for the host from the reference
 * sources (oracle/build_ref.sh -> oracle/_ref/libpoe2d_ref.so) and against the
 * golden fixtures that harness produced (tests/golden/).
 *
 * Grid convention (cu:486-487, cu:58, cu:685): (NX+1) x (NZ+1) cells, x
 * fastest, row pitch NX+1.  Field, coefficient and profile ids below.
 */
#ifndef POE2D_ORACLE_H
#define POE2D_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* precision modes */
enum {
    ORC_REFMIXED = 0, /* FP32 storage, FP64 stencil temporaries (the reference's double literals) */
    ORC_F32 = 1,      /* everything FP32 */
    ORC_F64 = 2       /* everything FP64 (drift yardstick) */
};

/* field ids (same numbering as the product's C-ABI) */
enum {
    ORC_VX = 0, ORC_VZ, ORC_WX, ORC_WZ, ORC_SXX, ORC_SZZ, ORC_SXZ, ORC_P,
    ORC_G11, ORC_G22, ORC_XI1, ORC_XI2,
    /* C-PML memory variables (cu:67-68, 79-80, 223-224, 303-305, 346-348) */
    ORC_M_DX_SXX, ORC_M_DZ_SXX, ORC_M_DX_S2, ORC_M_DZ_S2, ORC_M_DX_SXZ, ORC_M_DZ_SXZ,
    ORC_M_DX_VX1, ORC_M_DX_VX2, ORC_M_DZ_VX, ORC_M_DX_VZ, ORC_M_DZ_VZ1, ORC_M_DZ_VZ2,
    ORC_NFIELDS
};

/* coefficient planes: rho, rhof, m (rsm), eta/kappa, lambda_c, mu, alpha, M */
enum { ORC_C_RHO = 0, ORC_C_RHOF, ORC_C_RSM, ORC_C_EOK, ORC_C_LAMBDAC, ORC_C_MU, ORC_C_ALPHA, ORC_C_RBM, ORC_NCOEF };

/* profile rows: x -> a_x, b_x, K_x, a_x_half, b_x_half, K_x_half ; z likewise */
enum { ORC_PA = 0, ORC_PB, ORC_PK, ORC_PAH, ORC_PBH, ORC_PKH, ORC_NPROF };

/* where a source table is added */
enum { ORC_SRC_P = 0, ORC_SRC_FZ = 1 };

typedef struct orc_state orc_state;

/* set-up restatements */
void orc_pml_profiles(int NX, int NZ, float dx, float dz, float dt, int npoints,
                      float rcoef, float npower, float k_max, float alpha_max,
                      double alpha_top_extra, float cp_max,
                      float *prof_x /* 6*(NX+1) */, float *prof_z /* 6*(NZ+1) */);
int orc_coeffs_from_medium(int64_t ncell, const float *medium, const float *cp,
                           const float *cs, const float *rho_sat,
                           const float *fluid_table /* ntab x 6: kf eta kappa phi a rhof */,
                           int ntab, float *coef /* 8*ncell */);
int64_t orc_source_table(int kind, float f0, float amplitude, double t_cut, float dt,
                         float dx, float dz, int64_t nsteps, float *table);

/* time loop */
orc_state *orc_new(int mode, int NX, int NZ, float dx, float dz, float dt,
                   const float *coef, const float *prof_x, const float *prof_z);
void orc_free(orc_state *s);
void orc_set_source(orc_state *s, int ix, int iz, int where, const float *table, int64_t ntable);
void orc_set_receivers(orc_state *s, int nrec, const int32_t *rec /* nrec x (ix, iz, comp) */);
void orc_set_threads(orc_state *s, int nthreads);
int64_t orc_run(orc_state *s, int64_t nsteps, float *traces /* nsteps x nrec, may be NULL */);
void orc_get_field(const orc_state *s, int field, float *out);
void orc_get_field64(const orc_state *s, int field, double *out);
void orc_set_field(orc_state *s, int field, const float *in);
int64_t orc_steps_done(const orc_state *s);

#ifdef __cplusplus
}
#endif
#endif
