"""fluidsph — GB300 (sm_103a) SPH step of fluid-toy behind a C ABI.

The compute path is libfluidsph.so (CUDA kernels under ``csrc/``); this
package holds the build recipe, the ctypes binding of ``include/fluidsph.h``,
a Python mirror of the reference's ``SphSimulation3DGrid`` and the seeded
scene generators. There is no CPU implementation of the step in the product:
without the built library every entry point raises.
"""
from .abi import FluidSphError, load  # noqa: F401
from .build import LIB_PATH, build_library  # noqa: F401

__all__ = ["FluidSphError", "load", "LIB_PATH", "build_library"]
