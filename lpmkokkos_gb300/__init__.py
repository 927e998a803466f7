"""GB300-native (sm_103a) barotropic-vorticity hot path of pbosler/lpmKokkos.

The direct-sum spherical Biot-Savart velocity / stream function and the RK4 stepper that
evaluates it four times per step, as hand-written CUDA behind the C ABI of
include/lpm_bve.h.  ``build()`` compiles the in-tree native library; the Python classes
here (``Context``, ``BVESphere``, ``BVERK4``) mirror the reference's host interface.
"""
from ._build import build  # noqa: F401
from ._lib import (  # noqa: F401
    COLLOCATED, FP32C, FP64, MESH_TARGETS, NO_GRAPH, NO_SYMMETRIC, RCP_APPROX, TREECODE, NO_SORT, NO_VELOCITY, PSI, RENORM, RK4_FIX_QUIRK, SEED_CUBED,
    SEED_ICOS_TRI, SKIP_MASKED_TARGETS, LpmError, lib,
)


def __getattr__(name):
    # bve pulls in torch; import it lazily so build() does not need it.
    import importlib
    if name.startswith("__"):
        raise AttributeError(name)
    bve = importlib.import_module(__name__ + ".bve")
    if name == "bve":
        return bve
    if hasattr(bve, name):
        return getattr(bve, name)
    raise AttributeError(name)
