/*
 * poe2d.h -- C ABI of the GB300 solver for the 2-D poroelastic (Biot)
 * 4th-order staggered-grid velocity-stress time loop with C-PML.
 *
 * Drop-in boundary for the hot loop of thejatmik/poe2d
 * (seismic_CPML_2D_poroelastic_withCUDA.cu, abbreviated cu:).  The reference
 * has no plugin interface: its loop sits inside main() between set-up
 * (cu:470-1592) and output (cu:1737-1905).  Each entry point below replaces
 * the part of main() cited beside it, with plain pointers and sizes, status
 * codes instead of exit(), and no CUDA or torch types in the signatures.
 *
 * Conventions
 *   Grid: (NX+1) x (NZ+1) cells, x fastest, row pitch NX+1 (cu:58, 685);
 *         every host array below uses that layout.
 *   Ownership: the caller owns every host buffer; the library owns device
 *         memory, freed by poe_destroy.
 *   Errors: every call returns a poe_status; poe_last_error() has the text.
 *   Threading: one context per host thread; calls on a context are issued
 *         on its stream (the caller's, or the default stream).
 */
#ifndef POE2D_H
#define POE2D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference exits through HANDLE_ERROR/book.h or
 *      returns 0 on a Courant failure, cu:1203, cu:1212) ---- */
typedef enum poe_status {
    POE_OK = 0,
    POE_EINVAL = 1,     /* bad argument or size */
    POE_ECFL = 2,       /* Courant condition violated (cu:1197-1212) */
    POE_ENONFINITE = 3, /* field not finite or above 1e25 (cu:797) */
    POE_ETIMEOUT = 4,   /* a bounded device wait gave up */
    POE_ECUDA = 5,      /* CUDA runtime error */
    POE_ENOMEM = 6,     /* allocation failed */
    POE_EIO = 7,        /* file read/write failed */
    POE_ESTATE = 8      /* call not valid in the context's current state */
} poe_status;

/* coefficient planes, in this order, in every coef array (cu:1436-1451) */
enum {
    POE_C_RHO = 0,     /* rho (saturated density)            cu:687 */
    POE_C_RHOF = 1,    /* rho_f                              cu:658 */
    POE_C_RSM = 2,     /* m = a rho_f / phi                  cu:697 */
    POE_C_EOK = 3,     /* eta / kappa                        cu:698, 701-704 */
    POE_C_LAMBDAC = 4, /* lambda_c                           cu:708 */
    POE_C_MU = 5,      /* mu                                 cu:688 */
    POE_C_ALPHA = 6,   /* Biot alpha                         cu:699 */
    POE_C_RBM = 7,     /* Biot M                             cu:700 */
    POE_NCOEF = 8
};

/* profile rows: prof_x is 6 x (NX+1), prof_z is 6 x (NZ+1) (cu:886-906) */
enum { POE_PA = 0, POE_PB = 1, POE_PK = 2, POE_PA_HALF = 3, POE_PB_HALF = 4, POE_PK_HALF = 5 };

/* fields readable with poe_get_field (the first 12 are full grids) */
enum {
    POE_F_VX = 0, POE_F_VZ = 1, POE_F_WX = 2, POE_F_WZ = 3,     /* vx vz vxf vzf */
    POE_F_SXX = 4, POE_F_SZZ = 5, POE_F_SXZ = 6, POE_F_P = 7,   /* sigma xx zz xz, sigma2 */
    POE_F_G11 = 8, POE_F_G22 = 9, POE_F_XI1 = 10, POE_F_XI2 = 11,
    POE_NFIELDS = 12
};

/* receiver components (POE_REC_NONE: an inert slot that records 0) */
enum { POE_REC_NONE = -1, POE_REC_VX = 0, POE_REC_VZ = 1, POE_REC_P = 2 };

/* source kinds */
enum {
    POE_SRC_REF_DGAUSS_P = 0, /* the reference: 1e10 * 2a(t-t0) exp(-a(t-t0)^2), a = pi^2 f0^2,
                                 t0 = 1/f0, added to sigma2 while t < t_cut (cu:90-111) */
    POE_SRC_RICKER_FZ = 1     /* Ricker, t0 = 1.2/f0, vertical body force amplitude/(dx dz)
                                 on the bulk equation of the vz update (no reference counterpart) */
};

typedef struct poe_grid {
    int32_t NX, NZ;  /* last cell index per axis (cu:486-487) */
    float dx, dz;    /* DELTAX, DELTAZ (cu:494-495) */
    float dt;        /* DELTAT (cu:504) */
} poe_grid;

typedef struct poe_pml_params {
    int32_t npoints;        /* NPOINTS_PML (cu:510) */
    float rcoef;            /* Rcoef, 1e-3 (cu:992) */
    float npower;           /* NPOWER, 2 (cu:840) */
    float k_max;            /* K_MAX_PML, 1 (cu:843) */
    float alpha_max;        /* ALPHA_MAX_PML = 2 pi (f0/2) (cu:845) */
    double alpha_top_extra; /* 0.10: top strip alpha += 0.10 alpha_max (cu:1116, 1126) */
    float cp_max;           /* max P velocity for d0 (cu:716, 1001) */
} poe_pml_params;

typedef struct poe_source {
    int32_t ix, iz;    /* ISOURCE, JSOURCE (cu:757-758) */
    int32_t kind;      /* POE_SRC_* */
    float f0;          /* input2.txt (cu:830) */
    float amplitude;   /* POE_SRC_RICKER_FZ force amplitude (N/m); unused by the reference kind */
    double t_cut;      /* source active while t < t_cut; 0.4 in the reference (cu:107); <= 0: always */
} poe_source;

typedef struct poe_receiver {
    int32_t ix, iz, comp; /* comp: POE_REC_VX / POE_REC_VZ / POE_REC_P */
} poe_receiver;

/* one uniform Biot material, for poe_coeffs_biot */
typedef struct poe_biot_material {
    float rho_s, phi, k_s, k_frame, mu_frame;       /* solid grain density, porosity, moduli */
    float rho_f, k_f, eta, kappa, tortuosity;       /* fluid and transport */
} poe_biot_material;

typedef struct poe_ctx poe_ctx;

/* ---------------------------------------------------------------- set-up */

/* C-PML damping profiles.  Replaces cu:985-1159 (d0 cu:1001-1002, origins
 * cu:1042-1043 and 1101-1102, b and a cu:1090-1095, 1152-1158). */
int poe_pml_build(const poe_grid *grid, const poe_pml_params *pml,
                  float *prof_x /* 6*(NX+1) */, float *prof_z /* 6*(NZ+1) */);

/* Reference defaults for poe_pml_params given f0 and max cp (cu:510, 840-845, 992). */
void poe_pml_defaults(poe_pml_params *pml, int32_t npoints, float f0, float cp_max);

/* Medium-ID lookup and Biot coefficients from cp, cs and saturated density.
 * Replaces cu:646-661 (ID -> fluid row) and cu:682-713.  fluid_table rows
 * are (K_f, eta, kappa, phi, tortuosity, rho_f), ntab rows, IDs 0..ntab-1
 * (the reference's 4-row tables are cu:565-575).  A cell whose ID matches
 * no row is an error (POE_EINVAL), where the reference reads uninitialised
 * memory. */
int poe_coeffs_from_medium(const poe_grid *grid, const float *medium, const float *cp,
                           const float *cs, const float *rho_sat,
                           const float *fluid_table, int32_t ntab, float *coef /* 8*ncell */);

/* Biot coefficients from direct material parameters, one material per ID:
 * coef of cell j from mats[ids[j]].  Same formulas as cu:697-708 with
 * K_b = K_frame and K_s given (the reference's cp/cs path forces
 * K_s = K_b/(1-phi), i.e. alpha = phi).  vp_max_out (may be NULL) receives
 * the largest fast-P velocity of the high-frequency Biot dispersion relation,
 * for the Courant check and d0. */
int poe_coeffs_biot(int64_t ncell, const poe_biot_material *mats, int32_t nmat,
                    const uint8_t *ids, float *coef, float *vp_max_out);

/* The material palette poe_create builds when a model's 8 coefficient planes
 * take at most POE_MAX_MATERIALS distinct tuples (patchy models): a one-byte
 * id per cell and one row of POE_MROW floats per material.  A row holds the 8
 * coefficients (POE_C_* order), then what the velocity update derives from
 * them per cell, with the reference's float operations (cu:293-295, 311):
 * co = (rho m - rho_f^2) / dt, c1 = co + rho (eta/kappa) 0.5,
 * c2 = co - rho (eta/kappa) 0.5, rho_f (eta/kappa); then 1/co and 1/c1,
 * correctly rounded.  ids: ncell bytes; rows: POE_MAX_MATERIALS * POE_MROW
 * floats.  *nmat = 0 when the model has more tuples, or a material whose co
 * or c1 is not a normal float: poe_create then keeps the 8 coefficient planes
 * and reads them per cell. */
enum { POE_MAX_MATERIALS = 64, POE_MROW = 14 };
enum { POE_M_CO = 8, POE_M_C1 = 9, POE_M_C2 = 10, POE_M_RHOF_EOK = 11, POE_M_RCO = 12, POE_M_RC1 = 13 };
int poe_material_palette(const float *coef, int64_t ncell, float dt, uint8_t *ids, float *rows,
                         int32_t *nmat);

/* Courant checks of cu:1197-1212 (max cp dt/dx <= 1/sqrt(2) and
 * <= (6/7)/sqrt(2)).  Returns POE_OK or POE_ECFL. */
int poe_check_courant(const poe_grid *grid, float cp_max);

/* Source table as the loop adds it: entry n-1 is the value for step n
 * (t = (n-1) dt as a float, cu:94, 110).  Writes at most nsteps entries and
 * returns the count of active steps in *n_active (cut-off at t_cut). */
int poe_source_table(const poe_grid *grid, const poe_source *src, int64_t nsteps,
                     float *table, int64_t *n_active);

/* ---------------------------------------------------------------- context */

/* Create a solver context on the current CUDA device: uploads the 8
 * coefficient planes and the profiles (replaces the cudaMalloc/cudaMemcpy
 * block cu:1215-1592).  stream: a cudaStream_t, or NULL for the legacy
 * default stream.  flags: POE_CTX_* below. */
enum {
    POE_CTX_FAST_STENCIL = 1, /* plain FP32 stencils instead of rounding them as the reference's
                                 FP64 expressions do (faster, ~1e-6 relative drift) */
    POE_CTX_NO_PALETTE = 2    /* keep the 8 coefficient planes even when the model has few
                                 distinct materials (default: a 1-byte material id per cell) */
};
int poe_create(const poe_grid *grid, const float *coef, const float *prof_x,
               const float *prof_z, void *stream, uint32_t flags, poe_ctx **out);

/* Add a shot (its own wavefields and C-PML memory) with a source and an
 * explicit receiver list.  Replaces the fixed geometry of save1_kernel
 * (cu:114-201); poe_ref_receivers() builds that geometry as a list. */
int poe_add_shot(poe_ctx *ctx, const poe_source *src, const poe_receiver *rec,
                 int32_t nrec, int32_t *shot_id);

/* Advance every shot of the context by nsteps time steps (the chunk loop of
 * cu:1620-1636).  Receivers are recorded each step before the velocity
 * update, as save1_kernel does (cu:1629). */
int poe_run(poe_ctx *ctx, int64_t nsteps);

/* Wait for the context's stream. */
int poe_sync(poe_ctx *ctx);

/* Traces of a shot: [steps_done][nrec] floats, row = step - 1 (cu:129-200). */
int poe_get_traces(poe_ctx *ctx, int32_t shot, float *host_out, int64_t capacity_floats);

/* One full field of a shot, (NX+1)*(NZ+1) floats, x fastest (cu:1642-1645). */
int poe_get_field(poe_ctx *ctx, int32_t shot, int32_t field, float *host_out);

/* sigma_xx, sigma_zz or p (POE_F_SXX / POE_F_SZZ / POE_F_P) of a shot, like
 * poe_get_field, but allocating nothing: no reference counterpart.  For callers
 * that cannot allocate device memory (a fixed memory budget, a pool shared with
 * other work, or code between allocation-free phases): poe_get_field builds
 * these fields in a device buffer it allocates on first use, this entry point
 * builds them in a static 32 MiB plane that every GPU loading the library
 * holds until the process exits.  Limit: padded planes of at most 8 Mi floats
 * (grids up to about 2850 x 2850); larger ones return POE_EINVAL.  The first
 * call on a device looks up that plane's device address, so make it before any
 * stream capture.  All calls share the plane: calls that overlap on the GPU
 * (several contexts or threads at once) race, so serialise them.  Every cell
 * read back is written by the same call, nothing needs clearing. */
int poe_get_derived_noalloc(poe_ctx *ctx, int32_t shot, int32_t field, float *host_out);

/* The kernels' bounded waits, checked: no reference counterpart.  Every wait
 * of a kernel on an mbarrier (a tile's copies landing, a buffer's release)
 * or on other tiles' flags (a step-spanning launch) polls a bounded number of
 * times; a wait that gives up flags the context's error (POE_ETIMEOUT from the
 * next call that checks it) and the kernel ends, so a lost arrival or flag
 * cannot hang the GPU.  This runs the step kernel's wait code on device
 * `device` against a barrier no thread arrives at and against a tile flag
 * nothing sets, for at most `polls` polls each (1 .. 2^24), and the flag wait
 * once more against flags that are set: *gave_up = 1 when the first two
 * ended at their limit and the third passed (the expected answer), and the
 * device stays usable afterwards. */
int poe_wait_limit_check(int32_t device, int32_t polls, int32_t *gave_up);

/* Overwrite one full field of a shot (checkpoint restore; no reference counterpart). */
int poe_set_field(poe_ctx *ctx, int32_t shot, int32_t field, const float *host_in);

/* Full-state checkpoint of one shot: no reference counterpart (the
 * reference's vz/vx snapshots, cu:1653-1727, cannot restart a run).  The
 * image holds a header (poe_checkpoint_header below: grid, C-PML layout,
 * spacings, time step, hashes of the profiles, coefficients and receiver
 * list, source, step clock, checksum), every integrated field, the C-PML
 * memory variables, the pressure-source accumulator and the traces recorded
 * so far, in host byte order.  poe_checkpoint_load restores it into a shot
 * of a context built with the same grid, spacings, time step, profiles,
 * coefficients and shot definition (POE_EINVAL otherwise, POE_EIO on a
 * checksum mismatch); running on from there gives the same fields and
 * traces, bit for bit, as the uninterrupted run.  The first save or load on
 * a context reads its coefficients back from the device once, to hash them. */
int poe_checkpoint_size(poe_ctx *ctx, int32_t shot, int64_t *bytes);
int poe_checkpoint_save(poe_ctx *ctx, int32_t shot, void *host_buf, int64_t capacity);
int poe_checkpoint_load(poe_ctx *ctx, int32_t shot, const void *host_buf, int64_t size);

/* The header that starts every checkpoint image (host byte order).  The
 * payload follows it: the 9 integrated state planes of the current buffer
 * (device layout: pitch P, R rows), the stress and the velocity C-PML memory
 * on the x strips (3 x (NZ+1) x Wx floats each) and the z strips
 * (3 x Hz x P each), the pressure-source accumulator padded to 4 floats and
 * the traces recorded so far (steps x nrec floats).  poe_checkpoint_load
 * accepts an image only into a shot whose context has the same grid, C-PML
 * layout, spacings and time step (bit for bit), the same C-PML profiles
 * (prof_hash), the same coefficients cell by cell (coef_hash: the 8 planes,
 * whether the context keeps them or a material palette), the same source and
 * the same receiver list (rec_hash). */
enum { POE_CHECKPOINT_VERSION = 2 };
typedef struct poe_checkpoint_header {
    char magic[8];                  /* "POE2DCK1" */
    uint32_t version;               /* POE_CHECKPOINT_VERSION */
    uint32_t header_bytes;          /* sizeof(poe_checkpoint_header) */
    int32_t NX, NZ, P, R, Wx, Hz;   /* grid and device layout (plane pitch, rows, strip widths) */
    int64_t plane, steps;           /* floats per plane; steps done */
    int32_t nrec, src_kind, src_ix, src_iz;   /* src_kind -1: no source */
    float f0, amplitude;
    double t_cut;
    float dx, dz, dt;
    int32_t reserved0;
    uint64_t prof_hash, coef_hash, rec_hash;
    int64_t payload_bytes;
    uint64_t checksum;              /* of the payload */
    uint64_t reserved[2];
} poe_checkpoint_header;

/* Read and check the header of a checkpoint image on the host (no device
 * needed): POE_EINVAL when the buffer is not a version-2 image or is shorter
 * than its header and payload, POE_EIO when the payload's checksum differs.
 * out (may be NULL) receives the header. */
int poe_checkpoint_info(const void *host_buf, int64_t size, poe_checkpoint_header *out);

/* Tuning (no reference counterpart).  The step kernel walks a list of
 * (shot, tile) items, one CTA per SM, each CTA taking the next item from a
 * shared counter; the order of that list decides which tiles run side by
 * side (halo reuse in L2), and poe_run replays a captured CUDA graph of
 * graph_steps steps.  Results do not depend on either. */
enum {
    POE_ORDER_ROWS = 0,       /* per shot, tile rows; the default with FAST stencils */
    POE_ORDER_COLUMNS = 1,    /* per shot, tile columns */
    POE_ORDER_TILE_MAJOR = 2, /* the same tile of every shot side by side */
    POE_ORDER_BALANCED = 3    /* rows, with the edge tiles (C-PML strips, grid edges, the source:
                                 about twice an interior tile's work) spread evenly through the
                                 list, so that edge and interior tiles are in flight together;
                                 the default with EXACT stencils */
};
int poe_tune(poe_ctx *ctx, int32_t order, int32_t graph_steps);

/* Step-spanning launches (no reference counterpart).  POE_SPAN_ALWAYS runs
 * the graph_steps steps of each captured graph as ONE persistent launch, in
 * which a tile of step n starts as soon as its 3 x 3 neighbourhood of tiles
 * has completed step n-1 (per-tile flags in device memory, bounded waits), so
 * the steps overlap instead of each ending on its slowest CTA;
 * POE_SPAN_NEVER launches the step kernel once per step; POE_SPAN_AUTO (the
 * default) spans when a step holds at most 96 tiles per SM (one 2001 x 2001
 * shot: 14; 16 shots of 1001 x 1001: 57), where the step tail it removes
 * outweighs its per-tile costs.
 * Results do not depend on it. */
enum { POE_SPAN_NEVER = 0, POE_SPAN_ALWAYS = 1, POE_SPAN_AUTO = 2 };
int poe_tune_span(poe_ctx *ctx, int32_t span);

/* The step kernel's tile height (no reference counterpart): 60 x 32 tiles
 * (the default; every kernel variant) or 60 x 16 (FAST stencils, a context
 * outside any batch: twice the tiles per step, for grids too small to keep
 * every SM busy).  Results do not depend on it.  POE_EINVAL for another
 * height or 16 with EXACT stencils, POE_ESTATE for a context in a batch. */
int poe_tune_tile(poe_ctx *ctx, int32_t tile_z);

/* The context's current tuning; any pointer may be NULL. */
int poe_tuning(const poe_ctx *ctx, int32_t *order, int32_t *graph_steps, int32_t *span, int32_t *tile_z);

/* Time every (tile height, order, graph_steps in {16, 64}, span NEVER or
 * ALWAYS) candidate on this context for trial_steps steps, keep the fastest
 * and report it; ms_out (may be NULL) receives the POE_AUTOTUNE_CANDIDATES
 * timings, candidate c = tile height {32, 16}[c / 16], order (c / 4) % 4,
 * graph_steps {16, 64}[(c / 2) % 2], span c % 2 (-1 for a 16-row candidate
 * the context cannot take: EXACT stencils or a batch member).  Every shot
 * must be at step 0; the shots are reset to step 0 afterwards; poe_tune_tile,
 * poe_tune and poe_tune_span then hold the winner. */
enum { POE_AUTOTUNE_CANDIDATES = 32 };
int poe_autotune(poe_ctx *ctx, int32_t trial_steps, int32_t *order_out, int32_t *graph_steps_out, float *ms_out);

/* Steps completed by a shot. */
int poe_steps_done(poe_ctx *ctx, int32_t shot, int64_t *steps);

/* Zero a shot's state and step clock (zero_kernel, cu:387-422, cu:1736). */
int poe_reset_shot(poe_ctx *ctx, int32_t shot);

/* Check a shot's fields: POE_ENONFINITE if any velocity or stress is NaN,
 * Inf or of magnitude above threshold (the reference's unused
 * STABILITY_THRESHOLD = 1e25, cu:797).  max_abs_out may be NULL. */
int poe_check_finite(poe_ctx *ctx, int32_t shot, float threshold, float *max_abs_out);

/* Device kernels launched by this context since creation. */
int poe_kernel_launches(const poe_ctx *ctx, int64_t *count);

const char *poe_last_error(const poe_ctx *ctx);
const char *poe_status_string(int status);
void poe_destroy(poe_ctx *ctx);

/* ---------------------------------------------------------------- batches */

/* A batch advances the shots of several contexts (models of any sizes) in one
 * persistent launch per time step: no reference counterpart (the reference
 * runs one shot of one model per process, cu:1596-1736).  Every context must
 * be on the same device and use the same stencil mode, and either all use the
 * material palette (few distinct materials) or none does (per-cell
 * coefficient planes: many materials or POE_CTX_NO_PALETTE).  The contexts
 * stay owned by the caller.  A context belongs to at most one batch at a time
 * (POE_ESTATE for a context of a live batch); destroy the batch before its
 * contexts: a batch one of whose contexts was destroyed refuses
 * poe_batch_run with POE_ESTATE.  stream: a cudaStream_t or NULL for a
 * private stream. */
typedef struct poe_batch poe_batch;
int poe_batch_create(poe_ctx *const *ctxs, int32_t n, void *stream, poe_batch **out);

/* Advance every shot of context i by nsteps[i] steps (nsteps[i] may differ and
 * may be 0).  Results equal poe_run(ctxs[i], nsteps[i]) bit for bit.  Work
 * after the batch on a context's own stream (poe_get_traces, poe_run) is
 * ordered after it. */
int poe_batch_run(poe_batch *b, const int64_t *nsteps);

/* Step-spanning launches for the batch (poe_tune_span; a new batch takes its
 * first context's setting). */
int poe_batch_tune_span(poe_batch *b, int32_t span);

/* Wait for the batch; POE_ETIMEOUT if a kernel's bounded wait gave up. */
int poe_batch_sync(poe_batch *b);

/* Device kernels launched by this batch since creation. */
int poe_batch_launches(const poe_batch *b, int64_t *count);
const char *poe_batch_last_error(const poe_batch *b);
void poe_batch_destroy(poe_batch *b);

/* ---------------------------------------------------------------- reference geometry */

/* The receiver set save1_kernel records (cu:114-201), as an explicit list:
 *   panj vz then panj vx on the VSP line x = ISOURCE, y = k L2 - 1, L2 = (NZ+1)/panj;
 *   panj2 vz then panj2 vx on the line y = 10, x = k L - 1, L = (NX+1)/panj2;
 *   vz at x = (NX+1)/2 - 1 for y = 50, a0_pos, a1_pos, JSOURCE.
 * Always fills 2 panj + 2 panj2 + 4 slots in that order and returns the count
 * (or -1 if capacity is too small); a slot whose cell lies outside the grid
 * gets comp = POE_REC_NONE and records 0, as the reference never writes it. */
int32_t poe_ref_receivers(const poe_grid *grid, int32_t isource, int32_t jsource,
                          int32_t panj, int32_t panj2, int32_t a0_pos, int32_t a1_pos,
                          poe_receiver *out, int32_t capacity);

#ifdef __cplusplus
}
#endif
#endif /* POE2D_H */
