"""GB300-native FEDEM dynamics solver core: Python host side.

The compute runs in ``libfedem_solver_core.so`` (CUDA for sm_103a), which
exports the reference's solver-core C ABI (``solverInit``/``solveNext``/...,
see include/fedem_solver_core.h) and the batched ``fgpu_*`` API
(include/fgpu.h).  This package only binds them through ctypes, the same way
fedempy binds the reference library (PythonAPI/src/fedempy/solver.py:154-191).

There is no CPU fallback: if the library is missing, ``load_library`` raises.
"""
import ctypes
import os

from .buildlib import LIB_PATH, build  # noqa: F401

_LIB = None


class FedemException(Exception):
    """Error raised by the solver wrappers (same name as fedempy's)."""


def load_library(path=None):
    """Loads libfedem_solver_core.so and declares the exported signatures."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FedemException(
            f"GPU solver library not built: {p} (run fedem_gb300.build.build())")
    lib = ctypes.CDLL(p)
    c_int, c_dbl, c_bool = ctypes.c_int, ctypes.c_double, ctypes.c_bool
    P = ctypes.POINTER
    c_ll = ctypes.c_longlong
    vp = ctypes.c_void_p
    sig = {
        "solverInit": (c_int, [c_int, P(ctypes.c_char_p), ctypes.c_char_p, P(c_dbl), c_int, P(c_dbl), c_int,
                               P(c_dbl), P(c_int)]),
        "solveNext": (c_bool, [P(c_int)]),
        "startStep": (c_bool, [P(c_int)]),
        "solveIteration": (c_bool, [P(c_int), c_bool]),
        "solverDone": (c_int, [c_bool]),
        "solverClose": (None, []),
        "getTime": (c_dbl, [c_bool, P(c_int)]),
        "getStateVar": (c_int, [c_int, P(c_dbl)]),
        "getEquations": (c_int, [c_int, P(c_int)]),
        "getSystemSize": (c_int, [c_bool]),
        "getSystemMatrix": (c_bool, [P(c_dbl), c_int]),
        "getNewtonMatrix": (c_bool, [P(c_dbl)]),
        "getRhsVector": (c_bool, [P(c_dbl), c_int]),
        "getElementStiffnessMatrix": (c_bool, [P(c_dbl), c_int]),
        "getStateSize": (c_int, []),
        "saveState": (c_bool, [P(c_dbl), c_int]),
        "restartFromState": (c_int, [P(c_dbl), c_int, c_int]),
        "setTime": (c_bool, [c_dbl]),
        "setExtFunc": (c_bool, [c_int, c_dbl]),
        "solveEigenModes": (c_bool, [c_int, P(c_dbl), P(c_dbl), c_bool, c_int, P(c_int)]),
        "evalFunc": (c_dbl, [c_int, ctypes.c_char_p, c_dbl, P(c_int)]),
        "getFuncId": (c_int, [ctypes.c_char_p]),
        "solveWindow": (c_bool, [c_int, c_int, c_int, c_int, P(c_int), P(c_dbl), P(c_dbl), P(c_dbl), c_int,
                                 P(c_dbl), P(c_int)]),
        "setRhsVector": (c_bool, [P(c_dbl)]),
        "addRhsVector": (c_bool, [P(c_dbl)]),
        "fgpu_model_create": (c_int, [ctypes.c_char_p, c_int, P(ctypes.c_char_p), P(vp)]),
        "fgpu_model_destroy": (None, [vp]),
        "fgpu_model_sizes": (c_int, [vp, P(c_ll)]),
        "fgpu_model_meqn": (c_int, [vp, P(c_int)]),
        "fgpu_model_csr_pattern": (c_int, [vp, P(c_int), P(c_int)]),
        "fgpu_model_symbolic": (c_int, [vp, P(c_int), P(c_int)]),
        "fgpu_model_element_matrix": (c_int, [vp, c_int, c_int, P(c_dbl)]),
        "fgpu_batch_create": (c_int, [c_int, P(vp), c_int, c_int, P(vp)]),
        "fgpu_batch_destroy": (None, [vp]),
        "fgpu_batch_run": (c_int, [vp, c_ll, P(c_ll)]),
        "fgpu_batch_model_info": (c_int, [vp, c_int, P(c_int), P(c_int), P(c_dbl), P(c_ll), P(c_ll)]),
        "fgpu_batch_get_triads": (c_int, [vp, c_int, P(c_dbl)]),
        "fgpu_batch_get_all_triads": (c_ll, [vp, P(c_dbl)]),
        "fgpu_batch_get_newton_values": (c_int, [vp, c_int, P(c_dbl)]),
        "fgpu_batch_get_vector": (c_int, [vp, c_int, c_int, P(c_dbl)]),
        "fgpu_batch_get_norms": (c_int, [vp, c_int, P(c_dbl)]),
        "fgpu_batch_norms_noalloc": (c_int, [vp, c_int, P(c_dbl)]),
        "fgpu_batch_step": (c_int, [vp, c_int, P(c_int)]),
        "fgpu_batch_snapshot": (c_int, [vp]),
        "fgpu_batch_restore": (c_int, [vp]),
        "fgpu_batch_phase_timings": (c_ll, [vp, P(c_dbl), P(c_ll), c_int]),
        "fgpu_batch_time_factor": (c_int, [vp, c_int, P(c_dbl)]),
        "fgpu_batch_phase_timings_n": (c_ll, [vp, P(c_dbl), c_int, P(c_ll), c_int]),
        "fgpu_server_create": (c_int, [c_dbl, c_int, c_int, c_int, c_int, c_dbl, P(vp)]),
        "fgpu_server_destroy": (None, [vp]),
        "fgpu_server_submit": (c_int, [vp, vp, P(c_int)]),
        "fgpu_server_pump": (c_int, [vp]),
        "fgpu_server_status": (c_int, [vp, P(c_ll)]),
        "fgpu_server_now": (c_dbl, [vp]),
        "fgpu_server_slot_reuse": (c_int, [vp, c_dbl, P(c_ll)]),
        "fgpu_server_set_max_engines": (c_int, [vp, c_int]),
        "fgpu_server_request": (c_int, [vp, c_int, P(c_int), P(c_dbl), P(c_ll), P(c_ll)]),
        "fgpu_server_result": (c_int, [vp, c_int, P(c_dbl)]),
        "fgpu_set_device": (c_int, [c_int]),
        "fgpu_get_device": (c_int, [P(c_int), ctypes.c_char_p, c_int]),
        "fgpu_batch_device": (c_int, [vp]),
        "fgpu_batch_probe_wait_timeout": (c_int, [vp, c_ll, P(c_int)]),
        "fgpu_batch_probe_root_wait_timeout": (c_int, [vp, c_ll, P(c_int)]),
        "fgpu_measure_fp64_peak": (c_int, [P(c_dbl), P(c_dbl)]),
        "fgpu_measure_tf32_mma_peak": (c_int, [P(c_dbl), P(c_dbl)]),
        "fgpu_batch_set_launch_shape": (c_int, [vp, P(c_int)]),
        "fgpu_batch_launch_shape": (c_int, [vp, P(c_int), P(c_dbl)]),
        "fgpu_batch_results_open": (c_int, [vp, ctypes.c_char_p, c_int]),
        "fgpu_batch_results_close": (c_int, [vp]),
        "fgpu_batch_assemble_newton": (c_int, [vp, c_int, c_dbl, c_dbl, c_dbl]),
        "fgpu_batch_factor": (c_int, [vp, c_int]),
        "fgpu_batch_solve": (c_int, [vp, c_int, P(c_dbl), c_int]),
        "fgpu_last_error": (ctypes.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def _argv(options):
    opts = [str(o) for o in (options or [])]
    arr = (ctypes.c_char_p * max(1, len(opts)))(*[o.encode() for o in opts])
    return len(opts), arr


from .solver import FedemSolver  # noqa: E402,F401
from .batch import Batch, Model, Server  # noqa: E402,F401
