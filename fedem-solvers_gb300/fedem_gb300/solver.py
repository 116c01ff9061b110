"""``FedemSolver``: the fedempy driver interface over the GPU solver core.

Mirrors PythonAPI/src/fedempy/solver.py (``FedemSolver``: constructor,
``solver_init`` :322, ``solve_next`` :631, ``solver_done`` :833,
``get_current_time``, ``get_state_var``, ``get_system_size``,
``get_equations``, ``get_newton_matrix``, ``get_rhs_vector``, ``start_step``
:677, ``solve_iteration`` :707, ``finish_step``, ``set_rhs_vector`` /
``add_rhs_vector`` :1100-1110, ``get_state_size`` :495, ``save_state`` :546,
``restart_from_state`` :398, ``set_ext_func`` :888, ``get_function`` :941,
``get_function_ids`` :973, ``solve_window`` :429, ``solve_modes`` :742) with the same
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

    def solver_init(self, options, fsi=None, state_data=None):
        """Reads the model (fsi text or -fsifile option) and initialises it,
        continuing from state_data (a save_state array) when given."""
        argc, argv = _argv(["fedem_solver"] + list(options))
        cfsi = fsi.encode() if isinstance(fsi, str) else fsi
        sd, nd = None, 0
        if state_data is not None:
            self._state_in = np.ascontiguousarray(state_data, dtype=np.float64)
            sd, nd = self._state_in.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), self._state_in.size
        status = self._solver.solverInit(argc, argv, cfsi, sd, nd, None, 0, None, None)
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

    def get_system_matrix(self, i_mat):
        """Dense system matrix: 0 Newton, 1 stiffness, 2 mass, 3 damping (solverInterface.h:433)."""
        n = self.get_system_size()
        mat = np.zeros(n * n)
        ok = self._solver.getSystemMatrix(mat.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), int(i_mat))
        if not ok:
            raise FedemException("get_system_matrix failed")
        return mat.reshape((n, n), order="F")

    def _rhs(self, i_vec):
        n = self.get_system_size()
        vec = np.zeros(n)
        ok = self._solver.getRhsVector(vec.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), int(i_vec))
        if not ok:
            raise FedemException("get_rhs_vector failed")
        return vec

    def get_rhs_vector(self):
        """Right-hand side of the current linearised system."""
        return self._rhs(0)

    def get_external_force_vector(self):
        """External force vector Q of the current iteration."""
        return self._rhs(5)

    def _vec(self, r_vec):
        v = np.ascontiguousarray(r_vec, dtype=np.float64)
        if v.size != self.get_system_size():
            raise FedemException(f"Invalid vector length {v.size}")
        return v

    def set_rhs_vector(self, r_vec):
        v = self._vec(r_vec)
        return self._solver.setRhsVector(v.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))

    def add_rhs_vector(self, r_vec):
        v = self._vec(r_vec)
        return self._solver.addRhsVector(v.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))

    def start_step(self, time_next=None):
        """Predictor and first linear system of the next step (optionally at time_next)."""
        self.__check_error("start_step")
        ok = True if time_next is None else self._solver.setTime(float(time_next))
        return self._solver.startStep(ctypes.byref(self.ierr)) if ok else False

    def solve_iteration(self):
        """Solves the current system and assembles the next; False once converged."""
        self.__check_error("solve_iteration")
        return self._solver.solveIteration(ctypes.byref(self.ierr), False)

    def finish_step(self):
        """Iterates the started step to convergence; False at the end or on error."""
        self.__check_error("finish_step")
        return self._solver.solveIteration(ctypes.byref(self.ierr), True)

    def set_ext_func(self, func_id, value=None):
        """Value of external function channel func_id (1-based) for the next step."""
        return self._solver.setExtFunc(int(func_id), float(0.0 if value is None else value))

    def get_function(self, uid=0, tag=None, arg=None):
        """Value of the engine with user id uid (or the tagged one), at arg when given."""
        t = tag.encode() if isinstance(tag, str) else tag
        return self._solver.evalFunc(int(uid), t, float(-1.0 if arg is None else arg), ctypes.byref(self.ierr))

    def get_function_ids(self, tags):
        if isinstance(tags, str):
            return self._solver.getFuncId(tags.encode())
        return [self._solver.getFuncId(t.encode()) if isinstance(t, str) else int(t) for t in tags]

    def solve_window(self, n_step, inputs=None, f_out=None, xtimes=None):
        """n_step steps with the external function values of each step (inputs,
        len(inputs) // n_step per step) and step times (xtimes); returns the
        values of the functions f_out after each step and whether the
        simulation goes on."""
        P = ctypes.POINTER
        n_inc, times = 0, None
        if xtimes is not None:
            xt = np.ascontiguousarray(xtimes, dtype=np.float64)
            n_inc, times = xt.size, xt.ctypes.data_as(P(ctypes.c_double))
        n_in, inp = 0, None
        if inputs is not None:
            iv = np.ascontiguousarray(inputs, dtype=np.float64)
            n_in, inp = iv.size // max(int(n_step), 1), iv.ctypes.data_as(P(ctypes.c_double))
        n_out, fo, out = 0, None, None
        if f_out is not None:
            fv = np.ascontiguousarray(f_out, dtype=np.int32)
            n_out, fo = fv.size, fv.ctypes.data_as(P(ctypes.c_int))
            outv = np.zeros(int(n_step) * fv.size)
            out = outv.ctypes.data_as(P(ctypes.c_double))
        more = self._solver.solveWindow(int(n_step), n_inc, n_in, n_out, fo, times, inp, out, 0, None,
                                        ctypes.byref(self.ierr))
        return (list(outv) if f_out is not None else None), more

    def solve_modes(self, n_modes, dof_order=False, use_lapack=0):
        """The n_modes lowest eigenmodes at the current state: (eigenvalues in
        Hz, eigenvectors, success); (None, None, success) when *ierr != 0."""
        self.__check_error("solve_modes")
        dim = self.get_system_size(dofs=True) if dof_order else self.get_system_size()
        e_val = np.zeros(int(n_modes))
        e_vec = np.zeros(dim * int(n_modes))
        P = ctypes.POINTER(ctypes.c_double)
        ok = self._solver.solveEigenModes(int(n_modes), e_val.ctypes.data_as(P), e_vec.ctypes.data_as(P),
                                          bool(dof_order), int(use_lapack), ctypes.byref(self.ierr))
        if self.ierr.value != 0:
            if self.ierr.value > 0:
                self.ierr.value = 0
            return None, None, ok
        return list(e_val), [e_vec[dim * i:dim * (i + 1)] for i in range(int(n_modes))], ok

    def get_state_size(self):
        return self._solver.getStateSize()

    def save_state(self):
        """The solver state as a new float64 array (None if it cannot be saved now)."""
        n = self.get_state_size()
        data = np.zeros(n)
        ok = self._solver.saveState(data.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n)
        return data if ok else None

    def restart_from_state(self, state_data, write_to_rdb=2):
        """Continues from a state saved by save_state; 0 on success."""
        if write_to_rdb not in (0, 1, 2):
            raise TypeError(f"Expected integer value in (0, 1, 2), got {write_to_rdb}.")
        v = np.ascontiguousarray(state_data, dtype=np.float64)
        rc = self._solver.restartFromState(v.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), v.size,
                                           int(write_to_rdb))
        if rc == 0:
            self.ierr.value = 0
        return rc

    def run_all(self):
        """Runs the whole simulation (fedempy's usual solve_next loop)."""
        while self.solve_next():
            pass
        if self.ierr.value != 0:
            raise FedemException(f"Time integration failed ({self.ierr.value})")
