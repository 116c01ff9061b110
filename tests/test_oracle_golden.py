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
