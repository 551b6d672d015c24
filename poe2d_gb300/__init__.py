"""poe2d_gb300 -- GB300-native (sm_103a) 2-D poroelastic C-PML solver.

A drop-in for the velocity-stress time loop of thejatmik/poe2d: the CUDA
kernels live in ``csrc/`` behind the C ABI of ``include/poe2d.h``; this
package builds that library in-tree and drives it through ctypes.
"""
from ._lib import (CTX_FAST_STENCIL, FIELDS, REC_NONE, REC_P, REC_VX, REC_VZ, SPAN_ALWAYS, SPAN_AUTO, SPAN_NEVER,
                   SRC_REF_DGAUSS_P, SRC_RICKER_FZ, PoeError, lib, lib_path)
from .solver import (REFERENCE_FLUID_TABLE, Batch, Solver, biot_material, check_courant, checkpoint_info, coeffs_biot,
                     coeffs_from_medium, grid, material_palette, pml_defaults, pml_profiles, ref_receivers, source,
                     source_table, wait_limit_check)

__all__ = ["Solver", "Batch", "grid", "pml_profiles", "pml_defaults", "coeffs_from_medium", "coeffs_biot",
           "biot_material", "check_courant", "material_palette", "source", "source_table", "ref_receivers",
           "REFERENCE_FLUID_TABLE", "PoeError", "lib", "lib_path", "FIELDS", "SRC_REF_DGAUSS_P", "SRC_RICKER_FZ",
           "REC_VX", "REC_VZ", "REC_P", "REC_NONE", "CTX_FAST_STENCIL", "wait_limit_check", "checkpoint_info",
           "SPAN_NEVER", "SPAN_ALWAYS", "SPAN_AUTO"]
