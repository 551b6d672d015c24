// poe2d_tile_exact.cu -- the step kernel's variants for the reference's FP64 rounding at a spacing whose 24 h has few bits.
// One translation unit per stencil mode, so the variants compile in parallel.
#include "poe2d_tile.cuh"

namespace poe {

int tile_step_exact(const ModelDev &m, const ModelDev *models, const StreamShot *shots, const int4 *items,
                    int nitems, int k, int nk, bool kone, bool coef, int *queue, void *stream)
{
    return tile_launch_mode<SM_EXACT_FEW, PAL_TZ>(m, models, shots, items, nitems, k, nk, kone, coef, queue, (cudaStream_t)stream);
}

}  // namespace poe
