"""GB300-native (sm_103a) implementation of the TDVP step of mathiasgartner/TDVMC.

The compute path is the CUDA library behind the C ABI in include/tdvmc_gpu.h;
this package only binds it (``_native``), mirrors the reference's plugin
interface (``system`` for the periodic bulk system, ``drops`` for batched
trapped drops of uneven particle number) and builds it (``build``).
"""
from .drops import DropsTDVP, TrappedDrops  # noqa: F401
from .system import BosonsBulk, NUBosonsBulkPB, TDVP  # noqa: F401
