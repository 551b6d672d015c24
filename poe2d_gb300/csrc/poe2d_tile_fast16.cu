// poe2d_tile_fast16.cu -- the step kernel's single-model variants with plain
// FP32 stencils on 60 x 16 tiles (the autotuner's second tile shape: twice the
// tiles per step of the 60 x 32 tile, for grids too small to fill the SMs).
#include "poe2d_tile.cuh"

namespace poe {

int tile_step_fast16(const ModelDev &m, const StreamShot *shots, const int4 *items, int nitems, int k, int nk,
                     bool kone, bool coef, int *queue, void *stream)
{
    return tile_launch_mode<SM_FAST, PAL_TZ_SMALL>(m, nullptr, shots, items, nitems, k, nk, kone, coef, queue,
                                                   (cudaStream_t)stream);
}

}  // namespace poe
