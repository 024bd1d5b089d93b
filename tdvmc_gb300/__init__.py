"""GB300-native (sm_103a) implementation of the TDVP step of mathiasgartner/TDVMC.

The compute path is the CUDA library behind the C ABI in include/tdvmc_gpu.h;
this package only binds it (``_native``), mirrors the reference's plugin
interface (``system``) and builds it (``build``).
"""
from .system import BosonsBulk, TDVP  # noqa: F401
