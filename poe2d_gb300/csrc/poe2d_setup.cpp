// poe2d_setup.cpp -- host-side set-up of the solver: C-PML profiles, Biot
// coefficients, Courant check, source tables, reference receiver geometry.
//
// Floating-point types follow the reference expression by expression so the
// arrays are bit-identical to what its main() computes (float variables,
// FP64 wherever a double literal appears, the <cmath> float overloads for
// float arguments).  Compiled with -ffp-contract=off.
#include <array>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/poe2d.h"
#include "poe2d_palette.h"

namespace {

// PI as the reference's float literal (cu:41)
constexpr float kPiF = 3.1415926535897932f;

struct PmlPoint {
    float d, K, alpha;
};

// damping at one abscissa inside a strip (cu:1053-1056, 1112-1116)
PmlPoint pml_point(float absc, float thickness, float d0, float k_max, float npower, float amax,
                   double extra)
{
    PmlPoint r;
    const float nrm = absc / thickness;
    r.d = d0 * std::pow(nrm, npower);
    r.K = (float)(1.0 + ((double)k_max - 1.0) * (double)std::pow(nrm, npower));
    double al = (double)amax * (1.0 - (double)nrm);
    if (extra != 0.0) al = al + extra * (double)amax;
    r.alpha = (float)al;
    return r;
}

// one axis: low strip [0, origin_lo] (left or top), high strip from origin_hi
void pml_axis(int n1, float delta, float dt, float thickness, float d0, float k_max, float npower,
              float amax, float origin_lo, float origin_hi, double extra_lo, float *out)
{
    float *a = out + POE_PA * n1, *b = out + POE_PB * n1, *K = out + POE_PK * n1;
    float *ah = out + POE_PA_HALF * n1, *bh = out + POE_PB_HALF * n1, *Kh = out + POE_PK_HALF * n1;
    for (int i = 0; i < n1; ++i) {
        PmlPoint g{0.0f, 1.0f, 0.0f}, h{0.0f, 1.0f, 0.0f};
        const float val = delta * (float)i;
        const double half = (double)val + (double)delta / 2.0;
        float absc = origin_lo - val;
        if (absc >= 0.0f) g = pml_point(absc, thickness, d0, k_max, npower, amax, extra_lo);
        absc = (float)((double)origin_lo - half);
        if (absc >= 0.0f) h = pml_point(absc, thickness, d0, k_max, npower, amax, extra_lo);
        absc = val - origin_hi;
        if (absc >= 0.0f) g = pml_point(absc, thickness, d0, k_max, npower, amax, 0.0);
        absc = (float)(half - (double)origin_hi);
        if (absc >= 0.0f) h = pml_point(absc, thickness, d0, k_max, npower, amax, 0.0);
        if (g.alpha < 0.0f) g.alpha = 0.0f;
        if (h.alpha < 0.0f) h.alpha = 0.0f;
        K[i] = g.K;
        Kh[i] = h.K;
        b[i] = std::exp(-(g.d / g.K + g.alpha) * dt);
        bh[i] = std::exp(-(h.d / h.K + h.alpha) * dt);
        a[i] = 0.0f;
        ah[i] = 0.0f;
        if (std::fabs(g.d) > 1.e-6)
            a[i] = (float)((double)g.d * ((double)b[i] - 1.0) / (double)(g.K * (g.d + g.K * g.alpha)));
        if (std::fabs(h.d) > 1.e-6)
            ah[i] = (float)((double)h.d * ((double)bh[i] - 1.0) / (double)(h.K * (h.d + h.K * h.alpha)));
    }
}

bool grid_ok(const poe_grid *g)
{
    return g && g->NX >= 4 && g->NZ >= 4 && g->dx > 0.0f && g->dz > 0.0f && g->dt > 0.0f &&
           (int64_t)(g->NX + 1) * (g->NZ + 1) < (int64_t)1 << 40;
}

}  // namespace

namespace poe {

bool build_palette(const float *coef, int64_t ncell, float dt, std::vector<uint8_t> &ids, std::vector<float> &tab)
{
    std::vector<std::array<uint32_t, POE_NCOEF>> keys;
    ids.resize((size_t)ncell);
    int last = -1;
    for (int64_t j = 0; j < ncell; ++j) {
        std::array<uint32_t, POE_NCOEF> key;
        for (int c = 0; c < POE_NCOEF; ++c) std::memcpy(&key[c], coef + c * ncell + j, 4);
        int id = -1;
        if (last >= 0 && keys[last] == key) id = last;
        for (int i = 0; id < 0 && i < (int)keys.size(); ++i)
            if (keys[i] == key) id = i;
        if (id < 0) {
            if ((int)keys.size() >= MAX_PALETTE) return false;
            keys.push_back(key);
            id = (int)keys.size() - 1;
        }
        ids[(size_t)j] = (uint8_t)id;
        last = id;
    }
    tab.assign(keys.size() * MT_W, 0.0f);
    for (size_t i = 0; i < keys.size(); ++i) {
        float *t = tab.data() + i * MT_W;
        for (int c = 0; c < POE_NCOEF; ++c) std::memcpy(&t[c], &keys[i][c], 4);
        const float rho = t[POE_C_RHO], rhof = t[POE_C_RHOF], rsm = t[POE_C_RSM], eok = t[POE_C_EOK];
        const float co = (rho * rsm - rhof * rhof) / dt;
        float row[MT_W] = {0};
        row[MT_LC] = t[POE_C_LAMBDAC];
        row[MT_MU] = t[POE_C_MU];
        row[MT_AL] = t[POE_C_ALPHA];
        row[MT_M] = t[POE_C_RBM];
        row[MT_RHO] = rho;
        row[MT_RHOF] = rhof;
        row[MT_RSM] = rsm;
        row[MT_EOK] = eok;
        row[MT_RHOF_EOK] = rhof * eok;
        row[MT_CO] = co;
        row[MT_C1] = co + rho * eok * 0.5f;
        row[MT_C2] = co - rho * eok * 0.5f;
        row[MT_RCO] = (float)(1.0 / (double)co);
        row[MT_RC1] = (float)(1.0 / (double)row[MT_C1]);
        std::memcpy(t, row, sizeof(row));
        if (!std::isfinite(row[MT_RCO]) || !std::isfinite(row[MT_RC1]) || !std::isnormal(co) ||
            !std::isnormal(row[MT_C1]))
            return false;   // degenerate material: keep the plane path and IEEE division
    }
    return true;
}

}  // namespace poe

extern "C" {

void poe_pml_defaults(poe_pml_params *pml, int32_t npoints, float f0, float cp_max)
{
    pml->npoints = npoints;
    pml->rcoef = 0.001e0f;                              // cu:992
    pml->npower = 2.e0f;                                // cu:840
    pml->k_max = 1.e0f;                                 // cu:843
    pml->alpha_max = (float)(2.e0 * (double)kPiF * ((double)f0 / 2.e0));  // cu:845
    pml->alpha_top_extra = 0.10;                        // cu:1116
    pml->cp_max = cp_max;
}

int poe_pml_build(const poe_grid *grid, const poe_pml_params *pml, float *prof_x, float *prof_z)
{
    if (!grid_ok(grid) || !pml || !prof_x || !prof_z || pml->npoints < 1 || pml->npower < 1.0f ||
        !(pml->rcoef > 0.0f) || !(pml->cp_max > 0.0f))
        return POE_EINVAL;
    const int NX = grid->NX, NZ = grid->NZ;
    const float thx = (float)pml->npoints * grid->dx;  // cu:988-989
    const float thz = (float)pml->npoints * grid->dz;
    const double lr = (double)std::log(pml->rcoef);
    const float d0x = (float)(-((double)pml->npower + 1.0) * (double)pml->cp_max * lr / (2.0 * (double)thx));
    const float d0z = (float)(-((double)pml->npower + 1.0) * (double)pml->cp_max * lr / (2.0 * (double)thz));
    pml_axis(NX + 1, grid->dx, grid->dt, thx, d0x, pml->k_max, pml->npower, pml->alpha_max,
             thx + (float)3 * grid->dx, (float)(NX - 2) * grid->dx - thx, 0.0, prof_x);
    pml_axis(NZ + 1, grid->dz, grid->dt, thz, d0z, pml->k_max, pml->npower, pml->alpha_max, thz,
             (float)(NZ - 2) * grid->dz - thz, pml->alpha_top_extra, prof_z);
    return POE_OK;
}

int poe_coeffs_from_medium(const poe_grid *grid, const float *medium, const float *cp, const float *cs,
                           const float *rho_sat, const float *fluid_table, int32_t ntab, float *coef)
{
    if (!grid_ok(grid) || !medium || !cp || !cs || !rho_sat || !fluid_table || ntab < 1 || !coef)
        return POE_EINVAL;
    const int64_t n = (int64_t)(grid->NX + 1) * (grid->NZ + 1);
    for (int64_t j = 0; j < n; ++j) {
        int id = -1;
        for (int i = 0; i < ntab; ++i)
            if (medium[j] == (float)i) id = i;          // cu:650 (float == int)
        if (id < 0) return POE_EINVAL;
        const float *row = fluid_table + 6 * id;
        const float Kf = row[0], eta = row[1], kappa = row[2], phi = row[3], a = row[4], rhof = row[5];
        const float rho = rho_sat[j];                    // cu:687
        const float mu = cs[j] * cs[j] * rho;            // cu:688
        const float ksat = (float)((double)rho_sat[j] *
                                   ((double)(cp[j] * cp[j]) - (4.0 / 3.0) * (double)(cs[j] * cs[j])));
        const float nu = (float)((3.0 * (double)ksat - 2.0 * (double)mu) /
                                 (2.0 * (3.0 * (double)ksat + (double)mu)));
        const float kb = (float)(((2.0 * (double)nu / (1.0 - 2.0 * (double)nu)) + (2.0 / 3.0)) * (double)mu);
        const float ks = (float)((double)kb / (1.0 - (double)phi));
        const float rsm = a * rhof / phi;
        float eok = eta / kappa;
        const float alpha = (float)(1.0 - (double)(kb / ks));
        const float M = (float)(1.0 / (double)(phi / Kf + (alpha - phi) / ks));
        if (eta == 0.0f || kappa == 0.0f) eok = 0.0f;
        const float lambdao = (float)((double)kb - (2.0 / 3.0) * (double)mu);
        const float lambdac = lambdao + alpha * alpha * M;
        coef[POE_C_RHO * n + j] = rho;
        coef[POE_C_RHOF * n + j] = rhof;
        coef[POE_C_RSM * n + j] = rsm;
        coef[POE_C_EOK * n + j] = eok;
        coef[POE_C_LAMBDAC * n + j] = lambdac;
        coef[POE_C_MU * n + j] = mu;
        coef[POE_C_ALPHA * n + j] = alpha;
        coef[POE_C_RBM * n + j] = M;
    }
    return POE_OK;
}

// Direct Biot parameters.  rho = (1-phi) rho_s + phi rho_f, m = a rho_f/phi,
// alpha = 1 - K_b/K_s, M = 1/(phi/K_f + (alpha-phi)/K_s),
// lambda_c = K_b - 2/3 mu + alpha^2 M (the formulas of cu:697-708), each
// evaluated in FP64 and rounded once.  The fast P velocity is the larger root
// of the inviscid Biot dispersion relation
//   (rho m - rho_f^2) v^4 - (H m + rho M - 2 C rho_f) v^2 + (H M - C^2) = 0,
// H = lambda_c + 2 mu, C = alpha M.
int poe_coeffs_biot(int64_t ncell, const poe_biot_material *mats, int32_t nmat, const uint8_t *ids,
                    float *coef, float *vp_max_out)
{
    if (ncell < 1 || !mats || nmat < 1 || nmat > 256 || !ids || !coef) return POE_EINVAL;
    std::vector<float> tab((size_t)nmat * POE_NCOEF);
    double vmax = 0.0;
    for (int i = 0; i < nmat; ++i) {
        const poe_biot_material &q = mats[i];
        if (!(q.phi > 0.0f && q.phi < 1.0f) || !(q.k_s > 0.0f) || !(q.k_f > 0.0f) || !(q.rho_f > 0.0f) ||
            !(q.k_frame > 0.0f) || q.k_frame >= q.k_s || !(q.mu_frame >= 0.0f) || !(q.tortuosity >= 1.0f))
            return POE_EINVAL;
        const double phi = q.phi, ks = q.k_s, kb = q.k_frame, mu = q.mu_frame, kf = q.k_f;
        const double rho = (1.0 - phi) * q.rho_s + phi * q.rho_f;
        const double m = (double)q.tortuosity * q.rho_f / phi;
        const double eok = (q.eta == 0.0f || q.kappa == 0.0f) ? 0.0 : (double)q.eta / (double)q.kappa;
        const double alpha = 1.0 - kb / ks;
        const double M = 1.0 / (phi / kf + (alpha - phi) / ks);
        const double lc = kb - 2.0 / 3.0 * mu + alpha * alpha * M;
        float *t = tab.data() + (size_t)i * POE_NCOEF;
        t[POE_C_RHO] = (float)rho;
        t[POE_C_RHOF] = q.rho_f;
        t[POE_C_RSM] = (float)m;
        t[POE_C_EOK] = (float)eok;
        t[POE_C_LAMBDAC] = (float)lc;
        t[POE_C_MU] = q.mu_frame;
        t[POE_C_ALPHA] = (float)alpha;
        t[POE_C_RBM] = (float)M;
        const double H = lc + 2.0 * mu, Cc = alpha * M, rf = q.rho_f;
        const double A2 = rho * m - rf * rf, B2 = H * m + rho * M - 2.0 * Cc * rf, C2 = H * M - Cc * Cc;
        const double disc = std::sqrt(std::fmax(B2 * B2 - 4.0 * A2 * C2, 0.0));
        const double v2 = (B2 + disc) / (2.0 * A2);
        if (v2 > 0.0) vmax = std::fmax(vmax, std::sqrt(v2));
    }
    for (int64_t j = 0; j < ncell; ++j) {
        const int id = ids[j];
        if (id >= nmat) return POE_EINVAL;
        for (int c = 0; c < POE_NCOEF; ++c) coef[c * ncell + j] = tab[(size_t)id * POE_NCOEF + c];
    }
    if (vp_max_out) *vp_max_out = (float)vmax;
    return POE_OK;
}

int poe_check_courant(const poe_grid *grid, float cp_max)
{
    if (!grid_ok(grid)) return POE_EINVAL;
    const float c = cp_max * grid->dt / grid->dx;   // cu:1197
    if ((double)c > 1.0 / std::sqrt(2.0)) return POE_ECFL;           // cu:1202
    if ((double)c > 6.0 / 7.0 / std::sqrt(2.0)) return POE_ECFL;     // cu:1211
    return POE_OK;
}

int poe_source_table(const poe_grid *grid, const poe_source *src, int64_t nsteps, float *table,
                     int64_t *n_active)
{
    if (!grid_ok(grid) || !src || nsteps < 0 || (nsteps > 0 && !table) || !(src->f0 > 0.0f) ||
        (src->kind != POE_SRC_REF_DGAUSS_P && src->kind != POE_SRC_RICKER_FZ))
        return POE_EINVAL;
    const float f0 = src->f0, dt = grid->dt;
    const float a = kPiF * kPiF * f0 * f0;                       // cu:93
    int64_t n = 0;
    for (; n < nsteps; ++n) {
        const float t = (float)n * dt;                           // i_gpu * DDELTAT (cu:94)
        if (src->t_cut > 0.0 && !((double)t < src->t_cut)) break;  // cu:107
        if (src->kind == POE_SRC_REF_DGAUSS_P) {
            const float t0 = (float)(1.0 / (double)f0);          // cu:95
            const float tt = t - t0;
            table[n] = (float)(1.0e10 * 2.0 * (double)a * (double)tt *
                               std::exp((double)(-a) * std::pow((double)tt, 2.0)));  // cu:97
        } else {
            const float t0 = (float)(1.2 / (double)f0);
            const float tt = t - t0;
            const double e = std::exp((double)(-a) * std::pow((double)tt, 2.0));
            const double r = (1.0 - 2.0 * (double)a * std::pow((double)tt, 2.0)) * e;
            table[n] = (float)((double)src->amplitude * r / ((double)grid->dx * (double)grid->dz));
        }
    }
    if (n_active) *n_active = n;
    return POE_OK;
}

int32_t poe_ref_receivers(const poe_grid *grid, int32_t isource, int32_t jsource, int32_t panj,
                          int32_t panj2, int32_t a0_pos, int32_t a1_pos, poe_receiver *out,
                          int32_t capacity)
{
    if (!grid_ok(grid) || panj < 1 || panj2 < 1) return -1;
    const int32_t total = 2 * panj + 2 * panj2 + 4;
    if (!out || capacity < total) return -1;
    const int NX = grid->NX, NZ = grid->NZ;
    const int L2 = (NZ + 1) / panj, L = (NX + 1) / panj2;   // cu:120, 143
    int32_t w = 0;
    auto put = [&](int ix, int iz, int comp) {
        const bool in = ix >= 0 && ix <= NX && iz >= 0 && iz <= NZ;
        out[w++] = poe_receiver{ix, iz, in ? comp : POE_REC_NONE};
    };
    for (int c : {POE_REC_VZ, POE_REC_VX})                  // seismo, deismo (cu:137-138)
        for (int k = 1; k <= panj; ++k) put(isource, L2 > 0 ? k * L2 - 1 : -1, c);
    for (int c : {POE_REC_VZ, POE_REC_VX})                  // seismo1, deismo1 (cu:159-160)
        for (int k = 1; k <= panj2; ++k) put(L > 0 ? k * L - 1 : -1, 10, c);
    const int xc = (NX + 1) / 2 - 1;                        // cu:181-200
    for (int y : {50, a0_pos, a1_pos, jsource}) put(xc, y, POE_REC_VZ);
    return w;
}

static_assert(POE_MAX_MATERIALS == poe::MAX_PALETTE, "the public palette bound is the kernels' one");

int poe_material_palette(const float *coef, int64_t ncell, float dt, uint8_t *ids, float *rows, int32_t *nmat)
{
    if (!coef || ncell < 1 || !ids || !rows || !nmat || !(dt > 0.0f)) return POE_EINVAL;
    *nmat = 0;
    std::vector<uint8_t> id;
    std::vector<float> tab;
    if (!poe::build_palette(coef, ncell, dt, id, tab)) return POE_OK;
    // the kernels' row layout (poe::MT_*) to the public one (POE_C_*, then POE_M_*)
    static const int from[POE_MROW] = {poe::MT_RHO, poe::MT_RHOF, poe::MT_RSM, poe::MT_EOK, poe::MT_LC,
                                       poe::MT_MU,  poe::MT_AL,   poe::MT_M,   poe::MT_CO,  poe::MT_C1,
                                       poe::MT_C2,  poe::MT_RHOF_EOK, poe::MT_RCO, poe::MT_RC1};
    const int n = (int)(tab.size() / poe::MT_W);
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < POE_MROW; ++k) rows[(size_t)i * POE_MROW + k] = tab[(size_t)i * poe::MT_W + from[k]];
    std::memcpy(ids, id.data(), (size_t)ncell);
    *nmat = n;
    return POE_OK;
}

const char *poe_status_string(int status)
{
    switch (status) {
    case POE_OK: return "ok";
    case POE_EINVAL: return "invalid argument";
    case POE_ECFL: return "Courant condition violated";
    case POE_ENONFINITE: return "non-finite or diverging field";
    case POE_ETIMEOUT: return "device wait timed out";
    case POE_ECUDA: return "CUDA error";
    case POE_ENOMEM: return "out of memory";
    case POE_EIO: return "I/O error";
    case POE_ESTATE: return "invalid state";
    default: return "unknown status";
    }
}

}  // extern "C"
