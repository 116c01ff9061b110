"""Master-slave joints on the GPU path against the oracle (FP64 within 1e-10,
mixed precision within 1e-8 of the largest displacement over the run, equal
FP64 iteration counts), the Newton matrix assembled through the constraint
equations, the Gerber-beam statics through the solver ABI, and joint models
batched with others giving the same results as alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1.0e-10
MIXED_TOL = 1.0e-8
DYN = ["-timeInc=0.001", "-timeEnd=0.2", "-tolDispNorm=1.0e-10"]


def _cases():
    from fedem_gb300 import models

    return {
        "revolute_hinge": (models.hinged_beam(joint_type=1, load=2000.0)[0], DYN),
        "rigid_joint": (models.hinged_beam(joint_type=3, load=2000.0)[0], DYN),
        "pendulum": (models.pendulum(length=1.0, theta0=0.1)[0],
                     ["-timeInc=0.001", "-timeEnd=1.0", "-tolDispNorm=1.0e-10"]),
    }


def _oracle_run(fsi, opts):
    from oracle.oracle import OracleModel

    o = OracleModel(fsi, opts)
    o.run_all()
    out = o.triads().copy(), o.iterations(), o.max_displacement()
    o.close()
    return out


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
@pytest.mark.parametrize("name", ["revolute_hinge", "rigid_joint", "pendulum"])
def test_joint_models_match_oracle(gpu, oracle_lib, name, mixed):
    from fedem_gb300.batch import Batch, Model

    fsi, opts = _cases()[name]
    ref, iters, scale = _oracle_run(fsi, opts)
    m = Model(fsi, opts)
    b = Batch([m], mixed=mixed)
    st = b.run()
    assert st["models_done"] == 1 and st["models_failed"] == 0, b.info(0)
    err = np.abs(b.triads(0)[:, :, 3] - ref[:, :, 3]).max() / scale
    assert err <= (MIXED_TOL if mixed else FP64_TOL), err
    if not mixed:
        assert b.info(0)["iterations"] == iters
    b.close()


def test_joint_newton_matrix_matches_oracle(gpu, oracle_lib):
    """The predictor's Newton matrix assembled through the revolute joint's
    constraint equations (T^T N T) equals the oracle's assembly."""
    from fedem_gb300.batch import Batch, Model
    from oracle.oracle import OracleModel

    fsi, opts = _cases()["revolute_hinge"]
    o = OracleModel(fsi, opts)
    beta, gamma, dt, alpha = 0.3025, 0.6, 1.0e-3, -0.1
    sM, sK = 1.0 / (beta * dt * dt), 1.0 + alpha
    rp_u, ci_u, v_u = o.newton_upper(sM, gamma / (beta * dt) * sK, sK)
    m = Model(fsi, opts)
    b = Batch([m])
    b.step(0)
    vals = b.newton_values(0)
    rp, ci = m.csr_pattern()
    dense_gpu = np.zeros((m.neq, m.neq))
    for i in range(m.neq):
        dense_gpu[i, ci[rp[i]:rp[i + 1]]] = vals[rp[i]:rp[i + 1]]
    dense_ref = np.zeros((m.neq, m.neq))
    for i in range(m.neq):
        dense_ref[i, ci_u[rp_u[i]:rp_u[i + 1]]] = v_u[rp_u[i]:rp_u[i + 1]]
    dense_ref = np.triu(dense_ref) + np.triu(dense_ref, 1).T
    scale = np.abs(dense_ref).max()
    assert np.abs(dense_gpu - dense_ref).max() <= 1e-13 * scale
    assert np.array_equal(dense_gpu, dense_gpu.T)
    # the joint DOF's row couples it with the master triad's DOFs
    assert np.count_nonzero(dense_gpu[m.neq - 1]) > 1


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_gerber_beam_statics_through_solver_abi(gpu, mixed):
    """Initial static equilibrium of the revolute-hinged beam through
    solverInit: the hinge deflects P a^3 / 3 EI (the moment is released)."""
    from fedem_gb300 import models
    from fedem_gb300.solver import FedemSolver

    fsi, master, slave = models.hinged_beam(joint_type=1, load=10.0)
    opts = ["-initEquilibrium", "-tolInitEquil=1.0e-12", "-timeInc=0.001", "-timeEnd=0.001"]
    s = FedemSolver(solver_options=opts + (["-gpuMixed"] if mixed else []), fsi=fsi)
    y = s.get_state_var(master)[1]
    ei = 2.1e11 * models.pipe_section(0.1, 0.01)[1]
    theory = 10.0 * 2.0 ** 3 / (3.0 * ei)
    assert abs(y / theory - 1.0) < 1.0e-5, (y, theory)
    assert np.allclose(s.get_state_var(slave), s.get_state_var(master), rtol=0, atol=1e-13)
    s.solver_done()


def test_joint_models_same_alone_and_in_the_mix(gpu):
    from fedem_gb300 import models
    from fedem_gb300.batch import Batch, Model

    cases = list(_cases().values()) + [(f, o) for f, o, _ in models.batch_c4(3, seed=31, n_max=200, steps=200)]
    mix = Batch([Model(f, o) for f, o in cases], mixed=True)
    mix.run()
    for k, (f, o) in enumerate(cases):
        alone = Batch([Model(f, o)], mixed=True)
        alone.run()
        np.testing.assert_array_equal(mix.triads(k), alone.triads(0))
        alone.close()
    mix.close()
