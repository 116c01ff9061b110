"""GPU solver against the oracle (FP64 path within 1e-10, mixed precision
within 1e-8 relative displacement error) and against the reference's goldens,
all through the C ABI."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR

pytestmark = pytest.mark.gpu

FP64_TOL = 1.0e-10   # relative displacement error of the plain FP64 path
MIXED_TOL = 1.0e-8   # relative displacement error of FP32 factor + FP64 refinement
GPU_FEATURES = {"prescribed_motion", "quasi_static"}  # golden-case features the GPU path implements


def _golden_cases():
    with open(os.path.join(GOLDEN_DIR, "golden.json")) as f:
        return json.load(f)["cases"]


def rel_disp_error(ur_gpu, ur_ref, ur0):
    dg = ur_gpu[:, :, 3] - ur0[:, :, 3]
    dr = ur_ref[:, :, 3] - ur0[:, :, 3]
    scale = max(np.abs(dr).max(), 1e-300)
    return np.abs(dg - dr).max() / scale


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
@pytest.mark.parametrize("case", _golden_cases(), ids=lambda c: c["name"])
def test_reference_goldens_through_solver_abi(gpu, case, mixed):
    from fedem_gb300.solver import FedemSolver

    with open(os.path.join(GOLDEN_DIR, case["model"])) as f:
        fsi = f.read()
    missing = set(case["requires"]) - GPU_FEATURES
    if missing:
        pytest.skip("GPU path lacks " + ", ".join(sorted(missing)))
    opts = list(case["options"]) + (["-gpuMixed"] if mixed else [])
    s = FedemSolver(solver_options=opts, fsi=fsi)

    def state():
        return [v for t in case["triads"] for v in s.get_state_var(t)]

    got = [] if case["first_step"] else [state()]
    while len(got) < len(case["expected"]):
        s.solve_next()
        got.append(state())
    assert s.ierr.value == 0
    assert s.solver_done() == 0
    for g, e in zip(got, case["expected"]):
        for a, b in zip(g, e):
            assert abs(a - b) <= case["abs_tol"], (g, e)


def _run_pair(fsi, opts, mixed):
    from fedem_gb300.batch import Batch, Model
    from oracle.oracle import OracleModel

    o = OracleModel(fsi, opts)
    ur0 = o.triads()
    o.run_all()
    m = Model(fsi, opts)
    b = Batch([m], mixed=mixed)
    st = b.run()
    assert st["models_done"] == 1 and st["models_failed"] == 0, (st, b.info(0))
    return b, o, ur0


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_cantilever_1000_steps_matches_oracle(gpu, oracle_lib, mixed):
    from fedem_gb300 import models

    fsi, opts = models.cantilever_c1()
    b, o, ur0 = _run_pair(fsi, opts, mixed)
    err = rel_disp_error(b.triads(0), o.triads(), ur0)
    assert err <= (MIXED_TOL if mixed else FP64_TOL), err
    info = b.info(0)
    assert info["steps"] == 1000 and abs(info["time"] - 1.0) < 1e-9
    if not mixed:
        assert info["iterations"] == o.iterations()


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_batch_of_uneven_models_matches_oracle(gpu, oracle_lib, mixed):
    from fedem_gb300 import models
    from fedem_gb300.batch import Batch, Model
    from oracle.oracle import OracleModel

    cases = models.batch_c4(6, seed=21, n_max=400, steps=60)
    mods = [Model(f, op) for f, op, _ in cases]
    b = Batch(mods, mixed=mixed)
    st = b.run()
    assert st["models_done"] == 6 and st["models_failed"] == 0
    for k, (f, op, _) in enumerate(cases):
        o = OracleModel(f, op)
        ur0 = o.triads()
        o.run_all()
        err = rel_disp_error(b.triads(k), o.triads(), ur0)
        assert err <= (MIXED_TOL if mixed else FP64_TOL), (k, err)
        if not mixed:
            assert b.info(k)["iterations"] == o.iterations()


def test_newton_matrix_matches_oracle(gpu, oracle_lib):
    """FP64 Newton matrix of the first tangent update vs the oracle's assembly."""
    from fedem_gb300 import models
    from fedem_gb300.batch import Batch, Model
    from oracle.oracle import OracleModel

    fsi, opts, _ = models.batch_c4(1, seed=7, n_max=60, steps=1)[0]
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


def test_each_model_same_alone_and_in_the_mix(gpu):
    from fedem_gb300 import models
    from fedem_gb300.batch import Batch, Model

    cases = models.batch_c4(5, seed=33, n_max=200, steps=40)
    mix = Batch([Model(f, op) for f, op, _ in cases])
    mix.run()
    for k in (0, 3):
        f, op, _ = cases[k]
        alone = Batch([Model(f, op)])
        alone.run()
        assert np.array_equal(alone.triads(0), mix.triads(k))


def test_runs_are_bitwise_reproducible(gpu):
    from fedem_gb300 import models
    from fedem_gb300.batch import Batch, Model

    cases = models.batch_c4(3, seed=44, n_max=300, steps=30)
    res = []
    for _ in range(2):
        b = Batch([Model(f, op) for f, op, _ in cases], mixed=True)
        b.run()
        res.append([b.triads(k) for k in range(3)])
    for a, c in zip(res[0], res[1]):
        assert np.array_equal(a, c)


def _prescribed_chain(n_el, tip_d1):
    from fedem_gb300 import models

    return models.beam_chain_fsi(n_el, 0.25, 0.1, 0.01, clamp=0, load_node=n_el // 2, load_dof=3, load=500.0,
                                 motion=(n_el, 2, tip_d1), **models.STEEL)


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_prescribed_motion_dynamics_matches_oracle(gpu, oracle_lib, mixed):
    """Newmark steps with a prescribed tip deflection (ramp 0.05 * t) and a
    mid-span load: constraint values in the predictor, zero in correctors, and
    the prescribed columns moved to the right-hand side."""
    from fedem_gb300.batch import Batch, Model
    from oracle.oracle import OracleModel

    fsi = _prescribed_chain(24, 0.05)
    opts = ["-timeInc=0.002", "-timeEnd=0.3", "-alphaNewmark=0.1", "-tolDispNorm=1.0e-9"]
    o = OracleModel(fsi, opts)
    ur0 = o.triads()
    o.run_all()
    b = Batch([Model(fsi, opts)], mixed=mixed)
    st = b.run()
    assert st["models_done"] == 1 and st["models_failed"] == 0
    err = rel_disp_error(b.triads(0), o.triads(), ur0)
    assert err <= (MIXED_TOL if mixed else FP64_TOL), err
    # the prescribed DOF follows the motion exactly
    assert abs(b.triads(0)[24, 1, 3] - 0.05 * 0.3) < 1e-12
    if not mixed:
        assert b.info(0)["iterations"] == o.iterations()


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_quasi_static_then_dynamic_matches_oracle(gpu, oracle_lib, mixed):
    """Pure linear quasi-static steps (numit = -1) up to t = 0.1, then Newmark
    steps starting from the velocity rinc / dt, against the oracle."""
    from fedem_gb300.batch import Batch, Model
    from oracle.oracle import OracleModel

    fsi = _prescribed_chain(16, 0.2)
    opts = ["-numit=-1", "-timeInc=0.01", "-timeEnd=0.2", "-quasiStatic=0.1", "-tolDispNorm=1.0e-9"]
    o = OracleModel(fsi, opts)
    ur0 = o.triads()
    o.run_all()
    b = Batch([Model(fsi, opts)], mixed=mixed)
    st = b.run()
    assert st["models_done"] == 1 and st["models_failed"] == 0
    err = rel_disp_error(b.triads(0), o.triads(), ur0)
    assert err <= (MIXED_TOL if mixed else FP64_TOL), err
    if not mixed:
        assert b.info(0)["iterations"] == o.iterations()


def _frame_with_axials():
    from fedem_gb300 import models

    return models.beam_chain_fsi(30, 0.25, 0.1, 0.01, clamp=0, load_node=30, load_dof=2, load=800.0,
                                 **models.STEEL, anchors=[(7.5, 1.0, 0.0), (3.0, -1.0, 0.5)],
                                 springs=[(30, ("anchor", 0), 2.0e5, 1.0), (12, 27, 5.0e4, 3.75, 0.002),
                                          (20, ("anchor", 1), 1.0e5, 2.2)],
                                 dampers=[(30, ("anchor", 0), 300.0), (5, 18, 120.0)])


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_axial_springs_and_dampers_dynamics_match_oracle(gpu, oracle_lib, mixed):
    """Beam chain with axial springs (one with stiffness-proportional damping)
    and axial dampers, to ground and across the chain, under a tip step load."""
    from fedem_gb300.batch import Batch, Model
    from oracle.oracle import OracleModel

    fsi = _frame_with_axials()
    opts = ["-timeInc=0.001", "-timeEnd=0.2", "-alphaNewmark=0.1", "-tolDispNorm=1.0e-9"]
    o = OracleModel(fsi, opts)
    ur0 = o.triads()
    o.run_all()
    b = Batch([Model(fsi, opts)], mixed=mixed)
    st = b.run()
    assert st["models_done"] == 1 and st["models_failed"] == 0
    err = rel_disp_error(b.triads(0), o.triads(), ur0)
    assert err <= (MIXED_TOL if mixed else FP64_TOL), err
    if not mixed:
        assert b.info(0)["iterations"] == o.iterations()


def test_axial_newton_matrix_matches_oracle(gpu, oracle_lib):
    """FP64 Newton matrix with spring and damper blocks vs the oracle's assembly."""
    from fedem_gb300.batch import Batch, Model
    from oracle.oracle import OracleModel

    fsi = _frame_with_axials()
    opts = ["-timeInc=0.001", "-timeEnd=0.001"]
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
    assert np.abs(dense_gpu - dense_ref).max() <= 1e-13 * np.abs(dense_ref).max()


def test_axial_spring_linear_static_through_solver_abi(gpu):
    """Cantilever tip tied to ground by an axial spring along the load:
    u = P / (k + 3EI/L^3), through solverInit (linear initial equilibrium)."""
    from fedem_gb300 import models
    from fedem_gb300.solver import FedemSolver

    n, L = 10, 0.25
    _, inertia, _, _ = models.pipe_section(0.1, 0.01)
    kb = 3 * models.STEEL["E"] * inertia / (n * L) ** 3
    fsi = models.beam_chain_fsi(n, L, 0.1, 0.01, clamp=0, load_node=n, load_dof=2, load=1000.0, **models.STEEL,
                                anchors=[(n * L, 1.0, 0.0)], springs=[(n, ("anchor", 0), 2.0 * kb, 1.0)])
    s = FedemSolver(solver_options=["-initEquilibrium", "-tolInitEquil=0.0"], fsi=fsi)
    u = s.get_state_var(n + 1)[1]
    assert abs(u - 1000.0 / (3.0 * kb)) < 1e-10 * u
    assert s.solver_done() == 0


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_engine_driven_load_matches_oracle(gpu, oracle_lib, mixed):
    """Tip load growing as 2 kN * 5 t (F = f0 + f1 * engine, SCALE function of
    the TIME sensor) with axial springs, against the oracle."""
    from fedem_gb300 import models
    from fedem_gb300.batch import Batch, Model
    from oracle.oracle import OracleModel

    fsi = models.beam_chain_fsi(20, 0.25, 0.1, 0.01, clamp=0, load_node=20, load_dof=2, load=2000.0,
                                **models.STEEL, load_ramp=5.0, anchors=[(5.0, 1.0, 0.0)],
                                springs=[(20, ("anchor", 0), 3.0e4, 1.0)])
    opts = ["-timeInc=0.002", "-timeEnd=0.2", "-alphaNewmark=0.1", "-tolDispNorm=1.0e-9"]
    o = OracleModel(fsi, opts)
    ur0 = o.triads()
    o.run_all()
    b = Batch([Model(fsi, opts)], mixed=mixed)
    st = b.run()
    assert st["models_done"] == 1 and st["models_failed"] == 0
    err = rel_disp_error(b.triads(0), o.triads(), ur0)
    assert err <= (MIXED_TOL if mixed else FP64_TOL), err
    if not mixed:
        assert b.info(0)["iterations"] == o.iterations()


def test_system_stiffness_mass_damping_through_solver_abi(gpu, oracle_lib):
    """getSystemMatrix(1, 2, 3) (solverInterface.h:433) against the oracle's
    assembly with unit scales after solverInit: beams with Rayleigh damping,
    axial springs (one with stiffness-proportional damping) and dampers."""
    from fedem_gb300 import models
    from fedem_gb300.solver import FedemSolver
    from oracle.oracle import OracleModel

    fsi = models.beam_chain_fsi(12, 0.25, 0.1, 0.01, clamp=0, load_node=12, load_dof=2, load=100.0,
                                **models.STEEL, anchors=[(3.0, 1.0, 0.0)],
                                springs=[(12, ("anchor", 0), 2.0e5, 1.0, 0.002), (3, 9, 5.0e4, 1.5)],
                                dampers=[(12, ("anchor", 0), 300.0)])
    fsi = fsi.replace("  shadowPosAlg = 1\n", "  shadowPosAlg = 1\n  alpha1 = 0.5\n  alpha2 = 0.001\n")
    opts = ["-timeInc=0.001", "-timeEnd=0.01"]
    o = OracleModel(fsi, opts)
    s = FedemSolver(solver_options=opts, fsi=fsi)
    n = s.get_system_size()
    for i_mat, scales in ((1, (0.0, 0.0, 1.0)), (2, (1.0, 0.0, 0.0)), (3, (0.0, 1.0, 0.0))):
        rp, ci, v = o.newton_upper(*scales)
        ref = np.zeros((n, n))
        for i in range(n):
            ref[i, ci[rp[i]:rp[i + 1]]] = v[rp[i]:rp[i + 1]]
        ref = np.triu(ref) + np.triu(ref, 1).T
        got = s.get_system_matrix(i_mat)
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), i_mat
    assert s.solver_done() == 0
