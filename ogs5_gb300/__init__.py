"""GB300-native flow/transport hot path of OpenGeoSys 5.

Element assembly (GROUNDWATER_FLOW, LIQUID_FLOW, MASS_TRANSPORT on linear
quad/hex/tet meshes) into a CSR system and its preconditioned CG/BiCGStab
solve, as hand-written sm_103a CUDA kernels behind the C ABI of
include/ogs_gpu.h.  ``capi`` binds that ABI; ``mesh`` and ``fields`` make
the synthetic decks.
"""
from . import fields, mesh  # noqa: F401

__all__ = ["capi", "mesh", "fields", "build"]
