"""bpm_gb300: GB300-native (sm_103a) beam propagation and vectorial PSFs.

Drop-in for the hot paths of maweigert/bpm:
    from bpm_gb300 import bpm_3d, Bpm3d, psf, psf_u0, psf_lightsheet, focus_field_debye
Every z-step and every focus field runs in hand-written CUDA kernels in the in-tree
library libbpm_gb300.so (C ABI: include/bpm_gb300.h), reached through ctypes.
"""
from .bpm3d import bpm_3d, bpm_3d_batched, Bpm3d, BatchedMarch, MixedBatch, Plan, get_plan  # noqa: F401
from .psf import (focus_field_debye, focus_field_debye_at, focus_field_debye_gauss,  # noqa: F401
                  focus_field_debye_plane, psf, psf_u0, psf_lightsheet)
from .spheres import bpm_3d_spheres, create_dn_buffer  # noqa: F401
from ._native import launch_count  # noqa: F401

__all__ = ["bpm_3d", "bpm_3d_batched", "Bpm3d", "BatchedMarch", "MixedBatch", "psf", "psf_u0", "psf_lightsheet",
           "focus_field_debye", "focus_field_debye_gauss", "focus_field_debye_plane", "focus_field_debye_at",
           "bpm_3d_spheres", "create_dn_buffer", "launch_count"]
