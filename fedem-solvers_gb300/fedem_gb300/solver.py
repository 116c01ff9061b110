"""``FedemSolver``: the fedempy driver interface over the GPU solver core.

Mirrors PythonAPI/src/fedempy/solver.py (``FedemSolver``: constructor,
``solver_init`` :322, ``solve_next`` :631, ``solver_done`` :833,
``get_current_time``, ``get_state_var``, ``get_system_size``,
``get_equations``, ``get_newton_matrix``, ``get_rhs_vector``) with the same
argument meaning and error behaviour (``FedemException`` on failure, the
internal error flag blocks further calls after an error).
"""
import ctypes

import numpy as np

from . import FedemException, _argv, load_library


class FedemSolver:
    """Drives one model through libfedem_solver_core.so (process singleton)."""

    def __init__(self, lib_path=None, solver_options=None, fsi=None):
        self._solver = load_library(lib_path)
        self.ierr = ctypes.c_int(-999)
        if solver_options is not None:
            status = self.solver_init(solver_options, fsi)
            if status < 0:
                raise FedemException(f"Initialization failure ({status}). "
                                     + self._solver.fgpu_last_error().decode())

    def __check_error(self, func):
        if self.ierr.value != 0:
            raise FedemException(func + f"() cannot be called due to previous error ({self.ierr.value}).")

    def solver_init(self, options, fsi=None):
        """Reads the model (fsi text or -fsifile option) and initialises it."""
        argc, argv = _argv(["fedem_solver"] + list(options))
        cfsi = fsi.encode() if isinstance(fsi, str) else fsi
        status = self._solver.solverInit(argc, argv, cfsi, None, 0, None, 0, None, None)
        self.ierr.value = 0 if status >= 0 else status
        return status

    def solve_next(self):
        """Advances one time step; returns False at the end or on error."""
        self.__check_error("solve_next")
        return self._solver.solveNext(ctypes.byref(self.ierr))

    def solver_done(self, remove_singletons=True):
        self.ierr.value = self._solver.solverDone(remove_singletons)
        return self.ierr.value

    def get_current_time(self):
        self.__check_error("get_current_time")
        return self._solver.getTime(False, ctypes.byref(self.ierr))

    def get_next_time(self):
        self.__check_error("get_next_time")
        return self._solver.getTime(True, ctypes.byref(self.ierr))

    def get_state_var(self, base_id):
        """Position of the triad with the given base id (list of 3 floats)."""
        var = (ctypes.c_double * 3)()
        n = self._solver.getStateVar(base_id, var)
        return list(var[:n])

    def get_system_size(self, dofs=False):
        return self._solver.getSystemSize(dofs)

    def get_equations(self, base_id):
        meqn = (ctypes.c_int * 6)()
        n = self._solver.getEquations(base_id, meqn)
        return list(meqn[:n])

    def get_newton_matrix(self):
        n = self.get_system_size()
        mat = np.zeros(n * n)
        ok = self._solver.getNewtonMatrix(mat.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        if not ok:
            raise FedemException("get_newton_matrix failed")
        return mat.reshape((n, n), order="F")

    def get_rhs_vector(self):
        n = self.get_system_size()
        vec = np.zeros(n)
        ok = self._solver.getRhsVector(vec.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 0)
        if not ok:
            raise FedemException("get_rhs_vector failed")
        return vec

    def run_all(self):
        """Runs the whole simulation (fedempy's usual solve_next loop)."""
        while self.solve_next():
            pass
        if self.ierr.value != 0:
            raise FedemException(f"Time integration failed ({self.ierr.value})")
