"""Failure detection on the GPU path, with every failure made on the host: a
singular model, a NaN load, a Newton loop that cannot converge in its
iteration limit, and a bounded device wait that nothing ends.  Nothing here
faults, traps or hangs the GPU.  In a batch the failing model stops alone
(state 3 with its status bits) and every other model finishes with results
bitwise equal to its standalone run.  Through the solver ABI the error codes
follow the reference: -3 for a singular system (solExtensionModule.f90:
336-354), 1 for the iteration limit (newmarkRoutinesModule.f90:1003-1007)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SS_SINGULAR, SS_MAXIT, SS_NAN, SS_COROT, SS_TIMEOUT = 1, 2, 4, 8, 16
ST_DONE, ST_ERROR = 2, 3
OPTS = ["-timeInc=0.001", "-timeEnd=0.02", "-alphaNewmark=0.1", "-tolDispNorm=1.0e-10"]


def _chain(n_el, clamp=0, load=1500.0, load_dof=2):
    from fedem_gb300 import models

    return models.beam_chain_fsi(n_el, 0.25, 0.1, 0.01, clamp=clamp, load_node=n_el if clamp == 0 else 0,
                                 load_dof=load_dof, load=load, **models.STEEL)


def _unclamped(n_el):
    """A chain with no fixed DOF: its stiffness matrix is singular."""
    return _chain(n_el, clamp=-1)


def _good_cases():
    return [(_chain(12), OPTS), (_chain(40, load=-800.0, load_dof=3), OPTS)]


def _run_alone(case, mixed):
    from fedem_gb300.batch import Batch, Model

    m = Model(*case)
    b = Batch([m], mixed=mixed)
    b.run()
    out = b.triads(0).copy(), b.info(0)
    b.close()
    m.close()
    return out


def _check_batch(bad, mixed, want_bits):
    """[good0, bad, good1] in one batch: the bad model fails alone with
    want_bits in its status, the good ones equal their standalone runs."""
    from fedem_gb300.batch import Batch, Model

    good = _good_cases()
    ms = [Model(*good[0]), Model(*bad), Model(*good[1])]
    b = Batch(ms, mixed=mixed)
    st = b.run()
    assert st["models_failed"] == 1 and st["models_done"] == 2
    info = b.info(1)
    assert info["state"] == ST_ERROR and (info["status"] & want_bits), info
    for k, g in ((0, good[0]), (2, good[1])):
        ur, inf = _run_alone(g, mixed)
        assert b.info(k)["state"] == ST_DONE
        np.testing.assert_array_equal(b.triads(k), ur)
        assert b.info(k)["iterations"] == inf["iterations"]
    b.close()
    for m in ms:
        m.close()


def test_singular_initial_equilibrium_fails_alone(gpu):
    """An unclamped model with -initEquilibrium: its stiffness factorisation
    finds a singular pivot (FP64 fronts); only that model fails."""
    _check_batch((_unclamped(10), OPTS + ["-initEquilibrium", "-tolInitEquil=1.0e-8"]), False, SS_SINGULAR)


def test_singular_model_through_solver_abi_gives_minus_3(gpu):
    from fedem_gb300 import FedemException
    from fedem_gb300.solver import FedemSolver

    with pytest.raises(FedemException, match=r"\(-3\)"):
        FedemSolver(solver_options=OPTS + ["-initEquilibrium", "-tolInitEquil=1.0e-8"], fsi=_unclamped(10))


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_nan_load_fails_alone(gpu, mixed):
    """A NaN point load (written into the model text) makes the residual NaN:
    the model stops with the NaN status bit, the others finish unaffected."""
    fsi = _chain(20).replace("f0 = ", "f0 = nan ! ", 1)
    assert "f0 = nan" in fsi
    _check_batch((fsi, OPTS), mixed, SS_NAN)


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_iteration_limit_fails_alone(gpu, mixed):
    """-maxit=1 with a tolerance no iteration can meet: SS_MAXIT for that model only."""
    _check_batch((_chain(20), ["-timeInc=0.001", "-timeEnd=0.02", "-maxit=1", "-tolDispNorm=1.0e-30"]), mixed,
                 SS_MAXIT)


def test_iteration_limit_through_solver_abi_gives_1(gpu):
    from fedem_gb300.solver import FedemSolver

    s = FedemSolver(solver_options=["-timeInc=0.001", "-timeEnd=0.02", "-maxit=1", "-tolDispNorm=1.0e-30"],
                    fsi=_chain(20))
    assert not s.solve_next()
    assert s.ierr.value == 1
    s.solver_done()


def test_nan_external_force_through_add_rhs_vector(gpu):
    """A NaN external force added to the right-hand side of a started step
    (addRhsVector, kept for the step's iterations) fails the step with an
    error code instead of returning NaN positions."""
    from fedem_gb300.solver import FedemSolver

    s = FedemSolver(solver_options=OPTS, fsi=_chain(20))
    assert s.solve_next() and s.ierr.value == 0
    assert s.start_step()
    rhs = np.zeros(s.get_system_size())
    rhs[-1] = np.nan
    assert s.add_rhs_vector(rhs)
    assert not s.finish_step()
    assert s.ierr.value < 0
    s.solver_done()


def test_bounded_wait_runs_out_and_fails_the_models(gpu):
    """A back-substitution wait on a queue slot that nothing fills gives up
    after its poll limit and sets the batch's wait flag; the batch's running
    models then fail with SS_TIMEOUT, and the context stays usable: a new
    batch afterwards runs to the end."""
    import ctypes

    from fedem_gb300 import load_library
    from fedem_gb300.batch import Batch, Model

    lib = load_library()
    m = Model(*_good_cases()[0])
    b = Batch([m])
    flag = ctypes.c_int(0)
    assert lib.fgpu_batch_probe_wait_timeout(b._h, 4096, ctypes.byref(flag)) == 0, lib.fgpu_last_error()
    assert flag.value == 1
    b.run()
    info = b.info(0)
    assert info["state"] == ST_ERROR and (info["status"] & SS_TIMEOUT)
    b.close()
    b2 = Batch([m])
    st = b2.run()
    assert st["models_done"] == 1 and st["models_failed"] == 0
    b2.close()
    m.close()


def test_root_wait_runs_out_and_fails_the_models(gpu):
    """The fused back substitution's wait for a root's elimination (a release
    that nothing makes) gives up after its poll limit and sets the batch's wait
    flag, like the queue-slot wait; the running models then fail with
    SS_TIMEOUT and the context stays usable."""
    import ctypes

    from fedem_gb300 import load_library
    from fedem_gb300.batch import Batch, Model

    lib = load_library()
    m = Model(*_good_cases()[0])
    b = Batch([m])
    flag = ctypes.c_int(0)
    assert lib.fgpu_batch_probe_root_wait_timeout(b._h, 4096, ctypes.byref(flag)) == 0, lib.fgpu_last_error()
    assert flag.value == 1
    b.run()
    info = b.info(0)
    assert info["state"] == ST_ERROR and (info["status"] & SS_TIMEOUT)
    b.close()
    b2 = Batch([m])
    st = b2.run()
    assert st["models_done"] == 1 and st["models_failed"] == 0
    b2.close()
    m.close()


def test_selected_device_is_honoured(gpu):
    """fgpu_set_device(0): the library's current device and the batch's device
    are ordinal 0, and the PCI bus id of that device is reported."""
    from fedem_gb300.batch import Batch, Model, get_device, set_device

    dev, bus = set_device(0)
    assert dev == 0 and bus.count(":") >= 2
    assert get_device() == (0, bus)
    m = Model(*_good_cases()[0])
    b = Batch([m])
    assert b.device() == 0
    b.close()
    m.close()
