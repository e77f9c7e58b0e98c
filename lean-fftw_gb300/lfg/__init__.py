"""lfg: GB300-native execute path for lean-fftw's 1-D and batched transforms.

The transforms run in hand-written sm_103a CUDA kernels inside lfg/liblfg.so (C ABI:
include/lfg.h); this package holds the Python mirror of lean-fftw's plan/execute
interface (`plan`), the torch integration and the codelet generator used at build time
(`codegen`).
"""
from ._lib import LfgError, Unsupported, lib  # noqa: F401
from .plan import (R2R_KINDS, Plan, cos_sin_table, plan_1d, plan_c2r, plan_c2r_2d,  # noqa: F401
                   plan_layout, plan_measure, plan_r2c, plan_r2c_2d, plan_r2r, plan_spec, wisdom_count,
                   wisdom_export, wisdom_forget, wisdom_import)
from .ragged import RaggedPlan, plan_ragged, ragged_sizes, shard_ragged  # noqa: F401

__all__ = ["Plan", "plan_1d", "plan_measure", "plan_spec", "cos_sin_table", "LfgError",
           "Unsupported", "lib", "RaggedPlan", "plan_ragged", "ragged_sizes", "shard_ragged", "plan_r2c",
           "plan_c2r", "plan_r2c_2d", "plan_c2r_2d", "plan_r2r", "R2R_KINDS", "wisdom_import",
           "wisdom_export", "wisdom_forget", "wisdom_count", "plan_layout"]
