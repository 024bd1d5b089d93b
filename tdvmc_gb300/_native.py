"""ctypes binding of the C ABI declared in include/tdvmc_gpu.h.

The library is built in-tree (tdvmc_gb300/build.py).  There is no CPU
fallback: loading fails loudly when the library is missing, and the library
itself reports TDVMC_ERR_CUDA when no GPU is usable.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

OK, ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_STATE, ERR_NOT_PD, ERR_NONFINITE = range(7)
PREC_FP64, PREC_MIXED = 0, 1
POT_NONE, POT_SQUARE, POT_GAUSS, POT_LJ = 0, 1, 2, 3
SYS_BOSONS_BULK, SYS_NU_BOSONS_BULK_PB, SYS_NU_BOSONS_BULK_PB_EXACT = 0, 1, 2

# every entry point of include/tdvmc_gpu.h
EXPORTS = ("tdvmc_status_string", "tdvmc_create", "tdvmc_destroy", "tdvmc_get_stream", "tdvmc_set_time",
           "tdvmc_set_params", "tdvmc_get_params", "tdvmc_set_walkers", "tdvmc_get_walkers", "tdvmc_sample",
           "tdvmc_eval_local", "tdvmc_eval_local_adjoint", "tdvmc_store_samples", "tdvmc_eval_stored",
           "tdvmc_observables",
           "tdvmc_reduce_stats", "tdvmc_tdvp_rhs", "tdvmc_step",
           "tdvmc_get_step_operators", "tdvmc_run_steps", "tdvmc_time_steps", "tdvmc_profile_stage", "tdvmc_autotune", "tdvmc_get_tiles", "tdvmc_launch_count",
           "tdvmc_measure_fp32_peak", "tdvmc_reduce_walkers_noalloc",
           "tdvmc_drops_create", "tdvmc_drops_destroy", "tdvmc_drops_get_stream", "tdvmc_drops_set_params",
           "tdvmc_drops_get_params", "tdvmc_drops_set_walkers", "tdvmc_drops_get_walkers", "tdvmc_drops_sample",
           "tdvmc_drops_eval", "tdvmc_drops_reduce", "tdvmc_drops_tdvp_rhs", "tdvmc_drops_run_steps",
           "tdvmc_drops_time_steps", "tdvmc_drops_profile_stage", "tdvmc_drops_autotune", "tdvmc_drops_get_tiles",
           "tdvmc_drops_launch_count")


class SystemDesc(C.Structure):
    _fields_ = [("dim", C.c_int32), ("n", C.c_int32), ("p", C.c_int32), ("n_user_knots", C.c_int32),
                ("user_knots", C.POINTER(C.c_double)), ("box_length", C.c_double), ("pot_kind", C.c_int32),
                ("n_pot", C.c_int32), ("pot", C.c_double * 5), ("hbar2_2m", C.c_double), ("precision", C.c_int32),
                ("system_type", C.c_int32), ("n_walkers", C.c_int64)]


class DropsDesc(C.Structure):
    _fields_ = [("n_systems", C.c_int32), ("n", C.POINTER(C.c_int32)), ("p", C.c_int32),
                ("rmax", C.POINTER(C.c_double)), ("omega", C.c_double), ("v0", C.c_double), ("sigma", C.c_double),
                ("hbar2_2m", C.c_double), ("precision", C.c_int32), ("walkers_per_system", C.c_int64)]


class Stats(C.Structure):
    _fields_ = [("n_walkers", C.c_int64), ("energy_re", C.c_double), ("energy_im", C.c_double),
                ("other", C.c_double * 9), ("accept_rate", C.c_double), ("status", C.c_int32),
                ("reserved", C.c_int32)]


class StepOpts(C.Structure):
    _fields_ = [("dt", C.c_double), ("imaginary_time", C.c_int32), ("ode_solver", C.c_int32),
                ("lin_solver", C.c_int32), ("precondition", C.c_int32), ("normalize_wf", C.c_int32),
                ("moves_per_stage", C.c_int32), ("mc_step", C.c_double), ("seed", C.c_uint64),
                ("use_adjoint", C.c_int32), ("update_every", C.c_int32), ("update_percent", C.c_double)]


_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load the CUDA library (building it first when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError("tdvmc_gb300 CUDA library not built: %s" % path)
        _build.build()
    L = C.CDLL(path)
    P = C.POINTER
    d = C.c_void_p  # host double arrays are passed as raw pointers
    L.tdvmc_status_string.restype = C.c_char_p
    L.tdvmc_status_string.argtypes = [C.c_int]
    L.tdvmc_create.argtypes = [P(SystemDesc), P(C.c_void_p)]
    L.tdvmc_destroy.argtypes = [C.c_void_p]
    L.tdvmc_get_stream.argtypes = [C.c_void_p, P(C.c_void_p)]
    L.tdvmc_set_time.argtypes = [C.c_void_p, C.c_double]
    L.tdvmc_set_params.argtypes = [C.c_void_p, d, d, C.c_double, C.c_double]
    L.tdvmc_get_params.argtypes = [C.c_void_p, d, d, P(C.c_double), P(C.c_double)]
    L.tdvmc_set_walkers.argtypes = [C.c_void_p, d, C.c_int64]
    L.tdvmc_get_walkers.argtypes = [C.c_void_p, d, C.c_int64]
    L.tdvmc_sample.argtypes = [C.c_void_p, C.c_int32, C.c_double, C.c_uint64, C.c_uint32, P(C.c_int64)]
    L.tdvmc_eval_local.argtypes = [C.c_void_p, d, d, d, d]
    L.tdvmc_eval_local_adjoint.argtypes = [C.c_void_p, d]
    L.tdvmc_store_samples.argtypes = [C.c_void_p]
    L.tdvmc_eval_stored.argtypes = [C.c_void_p, d, d, d, d, d]
    L.tdvmc_observables.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, d, d, P(C.c_int32), d]
    L.tdvmc_reduce_stats.argtypes = [C.c_void_p, P(Stats), d, d, d, d, d]
    L.tdvmc_tdvp_rhs.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, d, d, P(C.c_double), P(C.c_double)]
    L.tdvmc_step.argtypes = [C.c_void_p, P(StepOpts), P(Stats)]
    L.tdvmc_get_step_operators.argtypes = [C.c_void_p, d]
    L.tdvmc_run_steps.argtypes = [C.c_void_p, P(StepOpts), C.c_int32, P(Stats)]
    L.tdvmc_time_steps.argtypes = [C.c_void_p, P(StepOpts), C.c_int32, P(C.c_float)]
    L.tdvmc_profile_stage.argtypes = [C.c_void_p, P(StepOpts), P(C.c_float), P(C.c_char_p), P(C.c_int32)]
    L.tdvmc_autotune.argtypes = [C.c_void_p, C.c_int32, C.c_double]
    L.tdvmc_get_tiles.argtypes = [C.c_void_p, P(C.c_int32), P(C.c_int32), P(C.c_int32), P(C.c_int32)]
    L.tdvmc_launch_count.argtypes = [C.c_void_p]
    L.tdvmc_launch_count.restype = C.c_int64
    L.tdvmc_measure_fp32_peak.argtypes = [P(C.c_double)]
    L.tdvmc_reduce_walkers_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_void_p,
                                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    v = C.c_void_p
    L.tdvmc_drops_create.argtypes = [P(DropsDesc), P(C.c_void_p)]
    L.tdvmc_drops_destroy.argtypes = [v]
    L.tdvmc_drops_get_stream.argtypes = [v, P(C.c_void_p)]
    L.tdvmc_drops_set_params.argtypes = [v, d, d, d, d]
    L.tdvmc_drops_get_params.argtypes = [v, d, d, d, d]
    L.tdvmc_drops_set_walkers.argtypes = [v, d]
    L.tdvmc_drops_get_walkers.argtypes = [v, d]
    L.tdvmc_drops_sample.argtypes = [v, C.c_int32, C.c_double, C.c_uint64, C.c_uint32, P(C.c_int64)]
    L.tdvmc_drops_eval.argtypes = [v, d, d, d, d, d]
    L.tdvmc_drops_reduce.argtypes = [v, d, d, d, d, d, d, d]
    L.tdvmc_drops_tdvp_rhs.argtypes = [v, C.c_int32, C.c_int32, C.c_int32, d, d, d, d, v]
    L.tdvmc_drops_run_steps.argtypes = [v, P(StepOpts), C.c_int32, d, v]
    L.tdvmc_drops_time_steps.argtypes = [v, P(StepOpts), C.c_int32, P(C.c_float)]
    L.tdvmc_drops_profile_stage.argtypes = [v, P(StepOpts), P(C.c_float), P(C.c_char_p), P(C.c_int32)]
    L.tdvmc_drops_autotune.argtypes = [v, C.c_int32, C.c_double]
    L.tdvmc_drops_get_tiles.argtypes = [v, P(C.c_int32), P(C.c_int32)]
    L.tdvmc_drops_launch_count.argtypes = [v]
    L.tdvmc_drops_launch_count.restype = C.c_int64
    _lib = L
    return L


class TdvmcError(RuntimeError):
    def __init__(self, code, where):
        self.code = code
        msg = load().tdvmc_status_string(code).decode()
        super().__init__("%s failed: %s (%d)" % (where, msg, code))


def check(code, where):
    if code != OK:
        raise TdvmcError(code, where)
