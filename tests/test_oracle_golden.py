"""The oracle against the reference's own golden values (test_solver.C:93-262)."""
import json
import os

import pytest

from conftest import GOLDEN_DIR


def _cases():
    with open(os.path.join(GOLDEN_DIR, "golden.json")) as f:
        return json.load(f)["cases"]


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c["name"])
def test_oracle_reproduces_reference_goldens(oracle_lib, case):
    from oracle.oracle import OracleModel

    with open(os.path.join(GOLDEN_DIR, case["model"])) as f:
        fsi = f.read()
    o = OracleModel(fsi, case["options"])

    def state():
        return [v for t in case["triads"] for v in o.state_var(t)]

    got = [] if case["first_step"] else [state()]
    while len(got) < len(case["expected"]):
        o.solve_next()
        got.append(state())
    for g, e in zip(got, case["expected"]):
        assert len(g) == len(e)
        for a, b in zip(g, e):
            assert abs(a - b) <= case["abs_tol"], (g, e)


def test_oracle_quasi_static_prescribed_is_linear_in_time(oracle_lib):
    """Pure linear quasi-static steps restart from the initial configuration:
    the response to the prescribed deflection d1 * t scales with t exactly
    up to round-off, and the run switches to Newmark dynamics after the
    quasi-static end time."""
    from oracle.oracle import OracleModel

    with open(os.path.join(GOLDEN_DIR, "cantilever_prescribed.fsi")) as f:
        fsi = f.read()
    opts = ["-numit=-1", "-timeInc=0.2", "-timeEnd=1.4", "-quasiStatic=1.0"]
    o = OracleModel(fsi, opts)
    xs = []
    for _ in range(5):
        o.solve_next()
        xs.append(o.state_var(4)[0])
    for k, x in enumerate(xs):
        assert abs(x - (k + 1) * xs[0]) < 1e-12 * (k + 1)
    o.solve_next()  # t = 1.2: dynamic step, tip still follows the motion
    assert abs(o.state_var(6)[0] - 1.2) < 1e-12


def test_oracle_linear_cantilever_matches_beam_theory(oracle_lib):
    """Linear static tip deflection = PL^3/3EI + PL/(G A / kappa) (Timoshenko)."""
    from oracle.oracle import OracleModel

    with open(os.path.join(GOLDEN_DIR, "cantilever_pipe.fsi")) as f:
        fsi = f.read()
    o = OracleModel(fsi, ["-initEquilibrium", "-tolInitEquil=0.0"])
    P, L, E, G, A, I, kappa = 1.0e5, 10.0, 2.1e11, 8.139534884e10, 1.5394e-2, 4.621989652e-4, 2.0
    expected = P * L ** 3 / (3 * E * I) + P * L * kappa / (G * A)
    assert abs(o.state_var(6)[0] - expected) < 2e-5 * expected


def test_oracle_dynamic_run_is_deterministic(oracle_lib):
    import numpy as np

    from fedem_gb300 import models
    from oracle.oracle import OracleModel

    fsi, opts = models.cantilever_c1()
    opts = [o if not o.startswith("-timeEnd") else "-timeEnd=0.05" for o in opts]
    runs = []
    for _ in range(2):
        o = OracleModel(fsi, opts)
        o.run_all()
        runs.append(o.triads())
    assert np.array_equal(runs[0], runs[1])
    # the tip moves in +Y under the +Y step load
    assert runs[0][20, 1, 3] > 0.0


def _spring_cantilever(k_factor=2.0, damper=None, alpha2=0.0):
    from fedem_gb300 import models

    n, L = 10, 0.25
    E = models.STEEL["E"]
    _, inertia, _, _ = models.pipe_section(0.1, 0.01)
    kb = 3 * E * inertia / (n * L) ** 3
    k = k_factor * kb
    fsi = models.beam_chain_fsi(n, L, 0.1, 0.01, clamp=0, load_node=n, load_dof=2, load=1000.0, **models.STEEL,
                                anchors=[(n * L, 1.0, 0.0)], springs=[(n, ("anchor", 0), k, 1.0, alpha2)],
                                dampers=[(n, ("anchor", 0), damper)] if damper else None)
    return fsi, k, kb


def test_oracle_axial_spring_linear_static_matches_theory(oracle_lib):
    """Tip of an Euler-Bernoulli cantilever tied to ground by an axial spring
    along the load: u = P / (k + 3EI/L^3)."""
    from oracle.oracle import OracleModel

    fsi, k, kb = _spring_cantilever()
    o = OracleModel(fsi, ["-initEquilibrium", "-tolInitEquil=0.0"])
    u = o.state_var(11)[1]
    assert abs(u - 1000.0 / (k + kb)) < 1e-10 * u


def test_oracle_axial_damper_and_spring_newton_blocks(oracle_lib):
    """Damper coefficient c and spring stiffness k enter the Newton matrix as
    n n^T blocks on the translational DOFs (addInDamperMat, calcSpringStiffness):
    with n = +y, the tip's y-y entry of N(sM=0, sC, sK) grows by sK*k + sC*c."""
    import numpy as np

    from oracle.oracle import OracleModel

    c = 250.0
    fsi0, k, _ = _spring_cantilever(k_factor=0.0)
    fsi1, k1, _ = _spring_cantilever(damper=c)

    def yy(fsi, sC, sK):
        o = OracleModel(fsi, [])
        meqn = o.meqn()
        rp, ci, v = o.newton_upper(0.0, sC, sK)
        eq = meqn[6 * 10 + 1] - 1  # tip y DOF
        row = v[rp[eq]:rp[eq + 1]]
        return row[list(ci[rp[eq]:rp[eq + 1]]).index(eq)]

    for sC, sK in ((0.0, 1.0), (1.0, 0.0), (0.7, 1.3)):
        d = yy(fsi1, sC, sK) - yy(fsi0, sC, sK)
        assert abs(d - (sK * k1 + sC * c)) < 1e-9 * (sK * k1 + sC * c)
