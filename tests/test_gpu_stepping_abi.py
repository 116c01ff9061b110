"""Externally driven stepping and in-core state through the solver C ABI
(solverInterface.h startStep :262, solveIteration :278, setTime :355,
get/set/addRhsVector :472-484, getStateSize :118, saveState :156,
restartFromState :87), the way fedempy's start_step / solve_iteration /
finish_step / save_state / restart_from_state drive them."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1.0e-10
N_EL = 16
OPTS = ["-timeInc=0.001", "-timeEnd=0.04", "-alphaNewmark=0.1", "-tolDispNorm=1.0e-10"]


def _fsi(load=1500.0):
    from fedem_gb300 import models

    return models.beam_chain_fsi(N_EL, 0.25, 0.1, 0.01, clamp=0, load_node=N_EL, load_dof=2, load=load,
                                 **models.STEEL)


def _positions(s):
    return np.array([s.get_state_var(t + 1) for t in range(N_EL + 1)])


def _solver(opts, fsi, mixed=False):
    from fedem_gb300.solver import FedemSolver

    return FedemSolver(solver_options=list(opts) + (["-gpuMixed"] if mixed else []), fsi=fsi)


def _solve_next_history(opts, fsi, mixed=False):
    s = _solver(opts, fsi, mixed)
    hist = []
    while s.solve_next():
        hist.append(_positions(s))
    hist.append(_positions(s))
    assert s.ierr.value == 0
    s.solver_done()
    return np.array(hist)


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_start_step_and_solve_iteration_equal_solve_next(gpu, mixed):
    """start_step + solve_iteration until converged gives the solve_next results bit for bit."""
    fsi = _fsi()
    ref = _solve_next_history(OPTS, fsi, mixed)
    s = _solver(OPTS, fsi, mixed)
    hist, iters = [], []
    while s.start_step():
        n = 1
        while s.solve_iteration():
            n += 1
        assert s.ierr.value == 0
        iters.append(n)
        hist.append(_positions(s))
    assert s.ierr.value == 0
    assert len(hist) == len(ref) == 40
    assert min(iters) >= 2  # at least the predictor and one corrector
    np.testing.assert_array_equal(np.array(hist), ref)
    assert not s.solve_iteration() and s.ierr.value == -999  # no step started
    s.solver_done()


def test_finish_step_and_solve_next_inside_a_step(gpu):
    """finish_step (solveIteration with all = true) and a solve_next issued
    after start_step both complete the started step."""
    fsi = _fsi()
    ref = _solve_next_history(OPTS, fsi)
    s = _solver(OPTS, fsi)
    hist = []
    k = 0
    while s.start_step():
        ok = s.finish_step() if k % 2 == 0 else s.solve_next()
        assert s.ierr.value == 0
        hist.append(_positions(s))
        k += 1
        if not ok:
            break
    assert len(hist) == 40
    np.testing.assert_array_equal(np.array(hist), ref)
    s.solver_done()


def test_start_step_with_time_next_matches_oracle(gpu, oracle_lib):
    """start_step(time_next) sets the step size (setTime): a model with
    timeInc 0.001 driven at 0.0025 matches the oracle run with timeInc 0.0025."""
    from oracle.oracle import OracleModel

    fsi = _fsi()
    opts_o = ["-timeInc=0.0025"] + OPTS[1:]
    o = OracleModel(fsi, opts_o)
    ur0 = o.triads()
    o.run_all()
    s = _solver(OPTS, fsi)
    t = s.get_current_time()
    steps = 0
    while True:
        if not s.start_step(time_next=t + 0.0025):
            break
        s.finish_step()
        assert s.ierr.value == 0
        t = s.get_current_time()
        steps += 1
    assert steps == 16 and abs(t - 0.04) < 1e-12
    assert not s.start_step(time_next=t - 0.001)  # can not go back in time
    assert not s.start_step(time_next=t + 0.5)  # above maxInc (0.1)
    got = _positions(s)
    ref = o.triads()[:, :, 3]
    d_ref = ref - ur0[:, :, 3]
    err = np.abs((got - ur0[:, :, 3]) - d_ref).max() / np.abs(d_ref).max()
    assert err <= FP64_TOL, err
    s.solver_done()


def test_rhs_vector_get_set_add(gpu):
    """getRhsVector sees the assembled right-hand side.  Adding zeros in the
    predictor (kept as zero external forces) and setting the right-hand side
    to itself in a corrector (which keeps no vector) leave the solution bit for
    bit unchanged."""
    fsi = _fsi()
    ref = _solve_next_history(OPTS, fsi)
    s = _solver(OPTS, fsi)
    n = s.get_system_size()
    hist = []
    while s.start_step():
        r = s.get_rhs_vector()
        assert r.shape == (n,) and np.abs(r).max() > 0.0
        assert s.add_rhs_vector(np.zeros(n))
        np.testing.assert_array_equal(s.get_rhs_vector(), r)
        while s.solve_iteration():
            r = s.get_rhs_vector()
            assert s.set_rhs_vector(r)
            np.testing.assert_array_equal(s.get_rhs_vector(), r)
        assert s.ierr.value == 0
        hist.append(_positions(s))
    np.testing.assert_array_equal(np.array(hist), ref)
    assert not s.add_rhs_vector(np.zeros(n))  # no step started
    s.solver_done()


def test_external_rhs_acts_as_a_step_load(gpu):
    """A tip force given with addRhsVector after every start_step (kept as an
    external force through the step's iterations) converges to the response of
    the same force given as a load record; Q (getRhsVector 5) holds it."""
    fsi_load, fsi_free = _fsi(1500.0), _fsi(0.0)
    opts = OPTS[:-1] + ["-tolDispNorm=1.0e-12"]
    ref = _solve_next_history(opts, fsi_load)
    s = _solver(opts, fsi_free)
    eq = s.get_equations(N_EL + 1)[1] - 1
    f = np.zeros(s.get_system_size())
    f[eq] = 1500.0
    hist = []
    while s.start_step():
        assert s.add_rhs_vector(f)
        first = True
        while s.solve_iteration():
            if first:
                q = s.get_external_force_vector()
                assert q[eq] == 1500.0 and np.abs(np.delete(q, eq)).max() == 0.0
                first = False
        assert s.ierr.value == 0
        hist.append(_positions(s))
    hist = np.array(hist)
    x0 = np.array([[0.25 * k, 0.0, 0.0] for k in range(N_EL + 1)])
    d_ref = ref - x0
    err = np.abs((hist - x0) - d_ref).max() / np.abs(d_ref).max()
    assert err <= 1e-7, err
    s.solver_done()


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_save_state_and_restart_reproduce_the_run(gpu, mixed):
    """saveState after 15 steps, restartFromState (and solverInit with the
    state array) continue exactly as the uninterrupted run."""
    fsi = _fsi()
    s = _solver(OPTS, fsi, mixed)
    for _ in range(15):
        assert s.solve_next()
    n = s.get_state_size()
    assert n > 0
    state = s.save_state()
    assert state is not None and state.size == n
    cont = []
    while s.solve_next():
        cont.append(_positions(s))
    cont.append(_positions(s))
    assert s.restart_from_state(state) == 0
    again = []
    while s.solve_next():
        again.append(_positions(s))
    again.append(_positions(s))
    np.testing.assert_array_equal(np.array(again), np.array(cont))
    # a started step refuses saveState; restart clears it
    assert s.restart_from_state(state) == 0
    assert s.start_step()
    assert s.save_state() is None
    assert s.restart_from_state(state) == 0
    s.solver_done()
    s2 = _solver(OPTS, fsi, mixed)
    s2.solver_done()
    from fedem_gb300.solver import FedemSolver

    s3 = FedemSolver()
    assert s3.solver_init(list(OPTS) + (["-gpuMixed"] if mixed else []), fsi, state_data=state) >= 0
    third = []
    while s3.solve_next():
        third.append(_positions(s3))
    third.append(_positions(s3))
    np.testing.assert_array_equal(np.array(third), np.array(cont))
    assert s3.restart_from_state(state[:-1]) < 0  # too short
    s3.solver_done()


def _ext_models():
    from fedem_gb300 import models

    common = dict(clamp=0, load_node=N_EL, load_dof=2, load=1500.0, **models.STEEL)
    fsi_time = models.beam_chain_fsi(N_EL, 0.25, 0.1, 0.01, load_ramp=40.0, **common)
    fsi_ext = models.beam_chain_fsi(N_EL, 0.25, 0.1, 0.01, load_ext=(1, 7, "tipload"), **common)
    return fsi_time, fsi_ext


def test_external_function_load_equals_the_time_engine(gpu):
    """A load driven by an external function (setExtFunc before every step,
    solverInterface.h:342) set to 40 t gives the results of the same load
    driven by a SCALE(40) function of the TIME sensor; evalFunc and getFuncId
    see the engines (solverInterface.h:383, :398)."""
    fsi_time, fsi_ext = _ext_models()
    ref = _solve_next_history(OPTS, fsi_time)
    s = _solver(OPTS, fsi_ext)
    assert s.get_function_ids("tipload") == 7 and s.get_function_ids("nothing") == -1
    assert not s.set_ext_func(2, 1.0)  # the model has one channel
    hist = []
    while True:
        t = s.get_next_time()
        assert s.set_ext_func(1, 40.0 * t)
        ok = s.solve_next()
        assert s.ierr.value == 0
        hist.append(_positions(s))
        assert s.get_function(7) == 40.0 * t
        assert s.get_function(tag="tipload") == 40.0 * t
        if not ok:
            break
    np.testing.assert_allclose(np.array(hist), ref, rtol=0.0, atol=1e-13)
    s.solver_done()
    s = _solver(OPTS, fsi_time)
    s.solve_next()
    uid = 2 * N_EL + 40  # the time engine's id (no extId): its user id
    assert abs(s.get_function(uid) - 40.0 * s.get_current_time()) < 1e-15
    assert s.get_function(uid, arg=0.5) == 20.0
    s.solver_done()


def test_solve_window_equals_step_by_step(gpu):
    """solveWindow (solverInterface.h:110) over 10 steps with the external
    values as inputs and the engine as output equals setExtFunc + solveNext."""
    _, fsi_ext = _ext_models()
    a = _solver(OPTS, fsi_ext)
    times = [a.get_current_time() + 0.001 * (k + 1) for k in range(10)]
    for t in times:
        a.set_ext_func(1, 40.0 * t)
        assert a.start_step(time_next=t)
        a.finish_step()
    ref = _positions(a)
    a.solver_done()
    b = _solver(OPTS, fsi_ext)
    outputs, more = b.solve_window(10, inputs=[40.0 * t for t in times], f_out=[7], xtimes=times)
    assert more and b.ierr.value == 0
    np.testing.assert_array_equal(np.array(outputs), 40.0 * np.array(times))
    np.testing.assert_array_equal(_positions(b), ref)
    outputs, more = b.solve_window(2, inputs=[1.0, 2.0], f_out=[7], xtimes=[0.5])  # too short times array
    assert not more and b.ierr.value == 1 - 2
    b.solver_done()


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_eigenmodes_match_a_dense_generalized_eigensolve(gpu, mixed):
    """solveEigenModes (solverInterface.h:293): the 6 lowest modes of K phi =
    lambda M phi at the initial state against scipy's dense generalized
    eigensolver on the same K and M (getSystemMatrix 1 and 2); frequencies in
    Hz, M-orthonormal vectors, DOF order with zeros at the clamp; the first
    bending frequency near the Euler-Bernoulli value; stepping afterwards is
    unchanged."""
    scipy_linalg = pytest.importorskip("scipy.linalg")
    from fedem_gb300 import models

    fsi = _fsi(0.0)
    s = _solver(OPTS, fsi, mixed)
    n = s.get_system_size()
    K, M = s.get_system_matrix(1), s.get_system_matrix(2)
    lam, phi = scipy_linalg.eigh(K, M, subset_by_index=[0, 5])
    ref = np.sqrt(lam) / (2.0 * np.pi)
    f, vecs, ok = s.solve_modes(6)
    assert ok and s.ierr.value == 0
    f = np.array(f)
    np.testing.assert_allclose(f, ref, rtol=1e-9)
    V = np.array(vecs).T  # n x 6
    np.testing.assert_allclose(V.T @ M @ V, np.eye(6), atol=1e-9)
    # K phi - lambda M phi relative to K phi (the Ritz residual bound is 1e-9 in
    # the M norm of K^-1 M, which K amplifies up to its condition number)
    resid = np.abs(K @ V - (M @ V) * lam).max() / np.abs(K @ V).max()
    assert resid < 1e-6, resid
    # Euler-Bernoulli cantilever, first bending frequency (20 consistent-mass elements: within 1 %)
    area, inertia, _, _ = models.pipe_section(0.1, 0.01)
    L = N_EL * 0.25
    f1 = 1.875104 ** 2 / (2 * np.pi) * np.sqrt(models.STEEL["E"] * inertia / (models.STEEL["rho"] * area * L ** 4))
    assert abs(f[0] - f1) < 0.01 * f1, (f[0], f1)
    fd, vd, ok = s.solve_modes(6, dof_order=True)
    assert ok and len(vd[0]) == s.get_system_size(dofs=True)
    np.testing.assert_allclose(np.array(fd), f, rtol=1e-12)
    assert np.all(np.array(vd)[:, :6] == 0.0)  # the clamped triad
    # the time steps after the eigenvalue analysis are those of a run without it
    for _ in range(10):
        assert s.solve_next()
    after = _positions(s)
    s.solver_done()
    s2 = _solver(OPTS, fsi, mixed)
    for _ in range(10):
        s2.solve_next()
    np.testing.assert_array_equal(after, _positions(s2))
    s2.solver_done()
