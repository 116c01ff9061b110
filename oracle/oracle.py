"""ctypes binding of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: the oracle is the FP64 CPU restatement of the
reference algorithm that the GPU solver is checked against, and the timed CPU
baseline in bench.py.  The product never imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(ORACLE_DIR, "liboracle.so")
_LIB = None
_P = ctypes.POINTER


def build():
    """Compiles liboracle.so with the Makefile next to this file."""
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    return LIB_PATH


def load():
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        build()
    lib = ctypes.CDLL(LIB_PATH)
    vp, ci, cd = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    sig = {
        "oracle_create": (vp, [ctypes.c_char_p, ci, _P(ctypes.c_char_p), _P(ci)]),
        "oracle_destroy": (None, [vp]),
        "oracle_solve_next": (ci, [vp, _P(ci)]),
        "oracle_get_state_var": (ci, [vp, ci, _P(cd)]),
        "oracle_get_time": (cd, [vp]),
        "oracle_get_ndof": (ci, [vp]),
        "oracle_get_neq": (ci, [vp]),
        "oracle_get_ntriads": (ci, [vp]),
        "oracle_get_nelements": (ci, [vp]),
        "oracle_get_meqn": (ci, [vp, _P(ci)]),
        "oracle_get_triad_ur": (ci, [vp, _P(cd)]),
        "oracle_get_iterations": (ctypes.c_longlong, [vp]),
        "oracle_get_max_displacement": (cd, [vp]),
        "oracle_get_last_norms": (ci, [vp, _P(cd)]),
        "oracle_get_csr_pattern": (ci, [vp, _P(ci), _P(ci)]),
        "oracle_assemble_newton": (ci, [vp, cd, cd, cd, _P(cd)]),
        "oracle_get_element_matrix": (ci, [vp, ci, ci, _P(cd)]),
        "oracle_get_force_vector": (ci, [vp, ci, _P(cd)]),
        "oracle_get_element_size": (ci, [vp, ci]),
        "oracle_get_gen_dofs": (ci, [vp, ci, _P(cd)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


class OracleModel:
    """One model advanced by the CPU oracle (solverInit/solveNext semantics)."""

    def __init__(self, fsi, options=()):
        self.lib = load()
        opts = ["oracle"] + [str(o) for o in options]
        argv = (ctypes.c_char_p * len(opts))(*[o.encode() for o in opts])
        ierr = ctypes.c_int(0)
        h = self.lib.oracle_create(fsi.encode() if isinstance(fsi, str) else fsi, len(opts), argv,
                                   ctypes.byref(ierr))
        if not h:
            raise RuntimeError(f"oracle set-up failed ({ierr.value})")
        self.h = h
        self.ndof = self.lib.oracle_get_ndof(h)
        self.neq = self.lib.oracle_get_neq(h)
        self.ntri = self.lib.oracle_get_ntriads(h)
        self.nel = self.lib.oracle_get_nelements(h)

    def close(self):
        if getattr(self, "h", None):
            self.lib.oracle_destroy(self.h)
            self.h = None

    __del__ = close

    def solve_next(self):
        ierr = ctypes.c_int(0)
        more = self.lib.oracle_solve_next(self.h, ctypes.byref(ierr))
        if ierr.value != 0:
            raise RuntimeError(f"oracle step failed ({ierr.value})")
        return bool(more)

    def run_all(self):
        while self.solve_next():
            pass

    def time(self):
        return self.lib.oracle_get_time(self.h)

    def state_var(self, tid):
        v = (ctypes.c_double * 3)()
        n = self.lib.oracle_get_state_var(self.h, tid, v)
        return list(v[:n])

    def meqn(self):
        v = np.zeros(self.ndof, dtype=np.int32)
        self.lib.oracle_get_meqn(self.h, v.ctypes.data_as(_P(ctypes.c_int)))
        return v

    def triads(self):
        ur = np.zeros(12 * self.ntri)
        self.lib.oracle_get_triad_ur(self.h, ur.ctypes.data_as(_P(ctypes.c_double)))
        return ur.reshape((-1, 4, 3)).transpose(0, 2, 1)

    def iterations(self):
        return self.lib.oracle_get_iterations(self.h)

    def max_displacement(self):
        """Largest triad displacement from the start positions over the steps so far."""
        return self.lib.oracle_get_max_displacement(self.h)

    def csr_upper_pattern(self):
        nnz = self.lib.oracle_get_csr_pattern(self.h, None, None)
        rp = np.zeros(self.neq + 1, dtype=np.int32)
        ci = np.zeros(nnz, dtype=np.int32)
        self.lib.oracle_get_csr_pattern(self.h, rp.ctypes.data_as(_P(ctypes.c_int)),
                                        ci.ctypes.data_as(_P(ctypes.c_int)))
        return rp, ci

    def newton_upper(self, sM, sC, sK):
        rp, ci = self.csr_upper_pattern()
        v = np.zeros(len(ci))
        self.lib.oracle_assemble_newton(self.h, sM, sC, sK, v.ctypes.data_as(_P(ctypes.c_double)))
        return rp, ci, v

    def element_matrix(self, iel, which):
        n = self.lib.oracle_get_element_size(self.h, iel)
        m = np.zeros(n * n)
        self.lib.oracle_get_element_matrix(self.h, iel, which, m.ctypes.data_as(_P(ctypes.c_double)))
        return m.reshape((n, n), order="F")

    def gen_dofs(self, iel):
        """Generalized DOF values of element iel (empty for a beam)."""
        v = np.zeros(max(1, self.lib.oracle_get_gen_dofs(self.h, iel, None)))
        n = self.lib.oracle_get_gen_dofs(self.h, iel, v.ctypes.data_as(_P(ctypes.c_double)))
        return v[:n]

    def force_vector(self, which):
        v = np.zeros(self.neq)
        self.lib.oracle_get_force_vector(self.h, which, v.ctypes.data_as(_P(ctypes.c_double)))
        return v
