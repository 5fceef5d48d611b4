"""fedg -- GB300-native SCALE-DG nonhydrostatic 3D DG dynamics step (HEVE/HEVI, IMEX-RK).

Host-side package around the CUDA library ``libfedg.so`` (C ABI in ``include/fedg.h``).
"""
from . import cases, element  # noqa: F401

__all__ = ["cases", "element", "lib"]
