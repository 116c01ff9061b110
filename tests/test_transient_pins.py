"""Transient dynamics pinned to something outside both restatements.

1. Linear HHT-alpha recurrence.  A 20-beam cantilever under a 10 N tip step
   load stays linear (deflection/length ~1e-4, geometric terms ~1e-8 of the
   response).  Its converged Newton steps must then be the closed-form
   HHT-alpha recurrence of the linear system built from the model's own K, M
   and C, in the reference's form (newmarkRoutinesModule.f90:85-187 predictor
   and Newmark update, :751-805 residual eq. 7.55 with the previous step's
   inertia force):
       M a1 + alpha M a0 + (1 + alpha)(C v1 + K u1) = (1 + alpha) F,
       a1 = (u1 - u0 - h v0) / (beta h^2) - (1 / (2 beta) - 1) a0,
       v1 = v0 + h ((1 - gamma) a0 + gamma a1),
   alpha = -0.1, beta = (1 - alpha)^2 / 4, gamma = 1/2 - alpha, started at
   rest.  The recurrence is solved in numpy; K, M, C come from the oracle's
   assembly (CPU test) and from getSystemMatrix through the solver ABI (GPU
   test).
2. Free-vibration period.  The step-loaded tip oscillates about its static
   deflection with the first bending mode: the period measured from the
   time history matches 1/f1 of the generalized eigenproblem K x = w^2 M x
   (numpy on the oracle's matrices; solveEigenModes on the GPU) within 0.5 %.
"""
import numpy as np
import pytest

N_EL = 20
LOAD = 10.0
ALPHA = -0.1


def _fsi():
    from fedem_gb300 import models

    return models.beam_chain_fsi(N_EL, 0.25, 0.1, 0.01, clamp=0, load_node=N_EL, load_dof=2, load=LOAD,
                                 **models.STEEL)


def _opts(steps):
    return [f"-timeInc=0.001", f"-timeEnd={steps * 0.001!r}", "-alphaNewmark=0.1", "-tolDispNorm=1.0e-13"]


def _hht_linear(K, M, C, F, h, steps, alpha=ALPHA):
    beta = (1.0 - alpha) ** 2 / 4.0
    gamma = 0.5 - alpha
    c0, c1, c2 = 1.0 / (beta * h * h), 1.0 / (beta * h), 1.0 / (2.0 * beta) - 1.0
    S = c0 * M + (1.0 + alpha) * (gamma * h * c0 * C + K)
    n = len(F)
    u, v, a = np.zeros(n), np.zeros(n), np.zeros(n)
    out = []
    for _ in range(steps):
        w = c0 * u + c1 * v + c2 * a  # a1 = c0 u1 - w
        vb = v + h * (1.0 - gamma) * a - h * gamma * w  # v1 = vb + h gamma c0 u1
        rhs = (1.0 + alpha) * F - alpha * (M @ a) + M @ w - (1.0 + alpha) * (C @ vb)
        u1 = np.linalg.solve(S, rhs)
        a1 = c0 * u1 - w
        v = v + h * ((1.0 - gamma) * a + gamma * a1)
        u, a = u1, a1
        out.append(u.copy())
    return np.array(out)


def _upper_to_dense(rp, ci, v, n):
    A = np.zeros((n, n))
    for i in range(n):
        for k in range(rp[i], rp[i + 1]):
            A[i, ci[k]] = v[k]
            A[ci[k], i] = v[k]
    return A


def _period(t, y):
    """Mean period from the upward zero crossings of y (linear interpolation)."""
    up = np.where((y[:-1] < 0.0) & (y[1:] >= 0.0))[0]
    tc = t[up] - y[up] * (t[up + 1] - t[up]) / (y[up + 1] - y[up])
    assert len(tc) >= 4, "too few oscillations"
    return (tc[-1] - tc[0]) / (len(tc) - 1)


def _tip_eq(meqn):
    """Equation (0-based) of the tip triad's y translation."""
    return int(meqn[6 * N_EL + 1]) - 1


# ---- oracle (CPU) ---------------------------------------------------------------
def _oracle_history(steps):
    from oracle.oracle import OracleModel

    o = OracleModel(_fsi(), _opts(steps))
    hist = []
    while o.solve_next():
        hist.append(o.state_var(N_EL + 1)[1])
    hist.append(o.state_var(N_EL + 1)[1])
    o_kmc = OracleModel(_fsi(), _opts(steps))
    n = o_kmc.neq
    K = _upper_to_dense(*o_kmc.newton_upper(0.0, 0.0, 1.0), n)
    M = _upper_to_dense(*o_kmc.newton_upper(1.0, 0.0, 0.0), n)
    C = _upper_to_dense(*o_kmc.newton_upper(0.0, 1.0, 0.0), n)
    meqn = o_kmc.meqn()
    o.close()
    o_kmc.close()
    return np.array(hist), K, M, C, meqn


def test_oracle_follows_the_linear_hht_recurrence(oracle_lib):
    steps = 300
    hist, K, M, C, meqn = _oracle_history(steps)
    assert len(hist) == steps
    tip = _tip_eq(meqn)
    F = np.zeros(len(K))
    F[tip] = LOAD
    lin = _hht_linear(K, M, C, F, 0.001, steps)[:, tip]
    err = np.abs(hist - lin).max() / np.abs(lin).max()
    assert err < 1.0e-6, err


def test_oracle_period_matches_the_first_eigenfrequency(oracle_lib):
    import scipy.linalg

    steps = 2000
    hist, K, M, C, meqn = _oracle_history(steps)
    w2 = scipy.linalg.eigh(K, M, eigvals_only=True, subset_by_index=[0, 0])[0]
    T1 = 2.0 * np.pi / np.sqrt(w2)
    static = np.linalg.solve(K, np.eye(len(K))[_tip_eq(meqn)] * LOAD)[_tip_eq(meqn)]
    t = 0.001 * np.arange(1, steps + 1)
    T = _period(t, hist - static)
    assert abs(T / T1 - 1.0) < 5.0e-3, (T, T1)


# ---- GPU through the solver ABI ---------------------------------------------------
def _gpu_history(steps, mixed):
    from fedem_gb300.solver import FedemSolver

    s = FedemSolver(solver_options=_opts(steps) + (["-gpuMixed"] if mixed else []), fsi=_fsi())
    K, M, C = s.get_system_matrix(1), s.get_system_matrix(2), s.get_system_matrix(3)
    meqn = s.get_equations(N_EL + 1)
    hist = []
    while s.solve_next():
        hist.append(s.get_state_var(N_EL + 1)[1])
    hist.append(s.get_state_var(N_EL + 1)[1])
    assert s.ierr.value == 0
    return s, np.array(hist), K, M, C, meqn


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_gpu_follows_the_linear_hht_recurrence(gpu, mixed):
    steps = 300
    s, hist, K, M, C, meqn = _gpu_history(steps, mixed)
    s.solver_done()
    tip = int(meqn[1]) - 1
    F = np.zeros(len(K))
    F[tip] = LOAD
    lin = _hht_linear(K, M, C, F, 0.001, steps)[:, tip]
    assert len(hist) == steps
    err = np.abs(hist - lin).max() / np.abs(lin).max()
    assert err < 1.0e-6, err


@pytest.mark.gpu
def test_gpu_period_matches_solve_eigen_modes(gpu):
    steps = 2000
    s, hist, K, M, C, meqn = _gpu_history(steps, False)
    # the lowest mode at the end of the run: the deflection is ~1e-4 of the
    # length, so it equals the start configuration's far below the tolerance
    freqs, _, ok = s.solve_modes(1)
    assert ok and freqs is not None
    s.solver_done()
    T1 = 1.0 / float(freqs[0])
    tip = int(meqn[1]) - 1
    static = np.linalg.solve(K, np.eye(len(K))[tip] * LOAD)[tip]
    t = 0.001 * np.arange(1, steps + 1)
    T = _period(t, hist - static)
    assert abs(T / T1 - 1.0) < 5.0e-3, (T, T1)
