// poe2d_palette.h -- the material palette of a model: the table-row layout the
// step kernel reads and the host builder (not part of the C ABI;
// poe_material_palette in include/poe2d.h is its public form).
#pragma once
#include <stdint.h>

#include <vector>

namespace poe {

// material-table row: coefficients and the quantities the reference derives
// from them per cell, rounded as it rounds them, grouped for 16-byte loads:
//   [lambda_c mu alpha M] [c2 rhof rho c1] [1/c1 m rhof*eta/kappa co] [1/co eta/kappa - -]
enum {
    MT_LC = 0, MT_MU, MT_AL, MT_M,
    MT_C2, MT_RHOF, MT_RHO, MT_C1,
    MT_RC1, MT_RSM, MT_RHOF_EOK, MT_CO,
    MT_RCO, MT_EOK, MT_W = 16
};
constexpr int MAX_PALETTE = 64;

// One id per cell (ncell bytes) and one table row of MT_W floats per distinct
// tuple of the 8 coefficient planes (coef: 8 planes of ncell floats, POE_C_*
// order), holding the coefficients and the quantities the reference derives
// from them per cell with its own float rounding (cu:293-295, 311) plus
// correctly rounded 1/co and 1/c1.  False if there are more than MAX_PALETTE
// tuples or a material whose co or c1 is not a normal float (such a model
// keeps its 8 planes and IEEE division).
bool build_palette(const float *coef, int64_t ncell, float dt, std::vector<uint8_t> &ids, std::vector<float> &tab);

}  // namespace poe
