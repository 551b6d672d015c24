// poe2d_tile_exact_any.cu -- the step kernel's variants for the reference's FP64 rounding at any spacing.
// One translation unit per stencil mode, so the variants compile in parallel.
#include "poe2d_tile.cuh"

namespace poe {

int tile_step_exact_any(const ModelDev &m, const ModelDev *models, const StreamShot *shots, const int4 *items,
                        int nitems, int k, int nk, bool kone, bool coef, int *queue, void *stream)
{
    return tile_launch_mode<SM_EXACT_ANY, PAL_TZ>(m, models, shots, items, nitems, k, nk, kone, coef, queue, (cudaStream_t)stream);
}

}  // namespace poe
